"""The C / C++ snippets of INTEGRATION.md compile against include/shg.h (syntax and types
only: each block becomes the body of a function, with the caller's variables declared in
front of it), so the integration notes cannot drift from the header."""
import os
import re
import shutil
import subprocess

import pytest

from _util import ROOT

# the caller-side names the snippets use, as a reference caller (SHG.cpp) would have them
PRELUDE = r"""
#include <complex>
#include <iostream>
#include <string>
#include <vector>
#include "shg.h"
static const int NX = 128, NY = 128, NZ = 200, K = 4, count = 4;
static const float LX = 463.26f, LY = 463.26f, LZ = 30000.0f;
template <typename T> void saveMatrixComplex(T *, std::string) {}  // Files.h:36
"""

VARS = r"""
    float Power = 10, waist = 29, focalpoint = 15000, Temp = 50, T_inf = 25, Tpeltier1 = 50, Tpeltier2 = 50;
    bool save_only_last = true, save_temperature = false;
    shg_config cfg; shg_config_init(&cfg);
    shg_handle *h = nullptr;
    float temp = 50, power = 10, focal = 15000, *sh_out_all = nullptr, P[count] = {}, T[count] = {};
    void *d_pump_in = nullptr, *d_grad_pump = nullptr, *d_grad_sh = nullptr, *stream = nullptr, *d_pumps = nullptr,
         *d_grads = nullptr;
    double p_sh[count], p_in[count];
"""


def _blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```(?:c|cpp)\n(.*?)```", text, flags=re.S)


def test_integration_notes_have_c_snippets():
    assert len(_blocks()) >= 3


@pytest.mark.parametrize("k", range(3))
def test_integration_snippet_compiles(k, tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    body = "\n".join(l for l in _blocks()[k].splitlines() if not l.startswith("#include"))
    # a caller-side declaration the snippet makes itself wins over the prelude's
    declared = set(re.findall(r"\b(?:shg_handle|shg_batch|shg_thgrad|shg_config)\s*\*?\s*(\w+)\s*[;=\[]", body))
    vars_ = "\n".join(l for l in VARS.splitlines()
                      if not any(re.search(r"\b%s\b" % d, l) for d in declared))
    src = tmp_path / "snippet.cpp"
    src.write_text(PRELUDE + "int snippet() {\n" + vars_ + "\n" + body + "\nreturn 0;\n}\n")
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wno-unused", "-I", os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + "\n" + src.read_text()


def test_ctypes_stub_matches_the_binding(monkeypatch):
    """The ctypes stub of the integration notes declares shg_config field for field like the
    packaged binding, and its shg_config_init call fills the reference defaults (run up to
    that call: the rest needs a GPU)."""
    from shg_focused_gaussian_beams_gb300 import _lib
    if not os.path.isfile(_lib.LIB_PATH):
        pytest.skip("library not built")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    stub = re.search(r"```python\n(.*?)```", text, flags=re.S).group(1)
    stub = stub.split("h = C.c_void_p()")[0]
    monkeypatch.chdir(ROOT)  # the stub loads the library by its path in the checkout
    ns = {}
    exec(compile(stub, "INTEGRATION.md", "exec"), ns)
    assert ns["shg_config"]._fields_ == _lib.Config._fields_
    cfg = ns["cfg"]
    assert (cfg.nx, cfg.ny, cfg.nz, cfg.lz, cfg.crystal) == (64, 64, 200, 30000.0, 0)
