"""Shared by the diagnostic-build tests (not collected): builds a variant of the library
and runs tests/_check_run.py against it in a child process."""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def asan_runtime():
    """Path of the compiler's AddressSanitizer runtime, or None."""
    gcc = shutil.which("gcc")
    if not gcc:
        return None
    p = subprocess.run([gcc, "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def run_child(mode: str, lib: str, sanitize: bool, timeout: int = 1200):
    env = dict(os.environ, SHG_LIB=lib)
    if sanitize:
        env["LD_PRELOAD"] = asan_runtime()
        # the CUDA driver maps the low shadow gap; leaks of the interpreter are not ours
        env["ASAN_OPTIONS"] = "protect_shadow_gap=0:detect_leaks=0:halt_on_error=1"
        env["UBSAN_OPTIONS"] = "halt_on_error=1:print_stacktrace=1"
    r = subprocess.run([sys.executable, os.path.join(HERE, "_check_run.py"), mode], env=env, capture_output=True,
                       text=True, timeout=timeout)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    report = json.loads(lines[-1]) if lines else None
    return r.returncode, report, r.stderr
