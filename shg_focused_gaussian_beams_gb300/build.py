"""Builds the CUDA library ``_build/libshg_gb300.so`` (and the ``shg`` CLI) for sm_103a.

Every translation unit in ``csrc/`` is compiled in parallel with nvcc; host code is built
with -ffp-contract=off so the crystal set-up keeps the reference's float operation order
on x86 and Arm alike.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libshg_gb300.so")
CLI = os.path.join(OUT, "shg")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          f"-I{os.path.join(HERE, '..', 'include')}"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        [os.path.join(HERE, "..", "include", "shg.h"), __file__]


def _obj(src):
    return os.path.join(OUT, os.path.basename(src) + ".o")


def _compile(src, verbose=False):
    cmd = [NVCC] + ARCH + COMMON + ["-c", src, "-o", _obj(src)]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + ["-x", "cu", "-c", src, "-o", _obj(src)] + ARCH
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return _obj(src), r.stderr


def up_to_date() -> bool:
    if not (os.path.isfile(LIB) and os.path.isfile(CLI)):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, jobs: int = 8, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    srcs = [s for s in _sources() if not s.endswith("shg_cli.cpp")]
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs + [os.path.join(CSRC, "shg_cli.cpp")]))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    objs = [_obj(s) for s in srcs]
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], check=True)
    os.replace(tmp, LIB)
    tmp = CLI + f".tmp{os.getpid()}"
    subprocess.run([NVCC] + ARCH + ["-o", tmp, _obj(os.path.join(CSRC, "shg_cli.cpp"))] + objs, check=True)
    os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
