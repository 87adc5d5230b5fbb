"""ORACLE recipe — test infrastructure only.

Builds the reference (alfredos84/SHG_Focused_Gaussian_Beams, header-only C++) from its
own sources where they lie, one shared library (and one CLI) per grid/crystal
configuration, into ``oracle/_ref/`` (git-ignored). The translation unit is
``oracle/ref_driver.cpp``; FFTW resolves to ``oracle/fftw_shim``.

The reference sources exist only in the development container; on a machine without
them this recipe does nothing, and the tests fall back to the committed golden fixtures
and the oracle restatement.

Usage: python oracle/build_ref.py [tag ...]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_SRC = os.environ.get("SHG_REFERENCE_SRC", "/root/reference/src")

sys.path.insert(0, HERE)
from configs import REF_BUILDS  # noqa: E402


def _defines(cfg: dict) -> list[str]:
    d = {
        "REF_NX": cfg["nx"], "REF_NY": cfg["ny"], "REF_NZ": cfg["nz"],
        "REF_LX": f"{cfg['lx']!r}f", "REF_LY": f"{cfg['ly']!r}f", "REF_LZ": f"{cfg['lz']!r}f",
        "REF_DEFF": f"{cfg['deff']!r}f", "REF_LAMBDA": f"{cfg['lambda_qpm']!r}f",
        "REF_ALPHA_P": f"{cfg['alpha_p']!r}f", "REF_ALPHA_S": f"{cfg['alpha_s']!r}f",
        "REF_BETA_S": f"{cfg['beta_s']!r}f", "REF_RHO_P": f"{cfg['rho_p']!r}f",
        "REF_RHO_S": f"{cfg['rho_s']!r}f", "REF_KTH": f"{cfg['kth']!r}f",
        "REF_HTC": f"{cfg['htc']!r}f",
    }
    out = [f"-D{k}={v}" for k, v in d.items()]
    if cfg.get("thermal"):
        out.append("-DTHERMAL")
    return out


def _compile(tag: str, cfg: dict) -> str:
    common = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", f"-I{REF_SRC}",
              f"-I{os.path.join(HERE, 'fftw_shim')}"] + _defines(cfg)
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "fftw_shim", "fftw_shim.cpp")]
    so = os.path.join(OUT, f"libshg_ref_{tag}.so")
    exe = os.path.join(OUT, f"shg_ref_{tag}")
    subprocess.run(common + ["-fPIC", "-shared", "-o", so] + srcs, check=True)
    subprocess.run(common + ["-DORACLE_REF_MAIN", "-o", exe] + srcs, check=True)
    return so


def available() -> bool:
    return os.path.isfile(os.path.join(REF_SRC, "headers", "Solver.h"))


def build(tags=None, jobs: int = 8) -> list[str]:
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    todo = {t: c for t, c in REF_BUILDS.items() if tags is None or t in tags}
    built = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(_compile, t, c): t for t, c in todo.items()}
        for f in cf.as_completed(futs):
            built.append(f.result())
    return built


if __name__ == "__main__":
    if not available():
        print("reference sources not present; nothing built")
        sys.exit(0)
    for p in build(sys.argv[1:] or None):
        print(p)
