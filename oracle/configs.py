"""ORACLE — test infrastructure only.

Grid/crystal configurations compiled by ``build_ref.py`` (the reference fixes them at
compile time: SHG.cpp:11-13, Crystal.h:31-53). Each tag becomes
``oracle/_ref/libshg_ref_<tag>.so`` and ``oracle/_ref/shg_ref_<tag>``.
"""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from shg_focused_gaussian_beams_gb300.workloads import (  # noqa: E402
    CRYSTAL_QPM50, CRYSTAL_REFERENCE, crystal_dict, config_plain_128, plain_instance)


def _cfg(crystal, nx, ny, nz, lx=None, ly=None, thermal=False):
    d = crystal_dict(crystal)
    d.update(nx=nx, ny=ny, nz=nz, thermal=thermal)
    if lx is not None:
        d["lx"] = lx
    if ly is not None:
        d["ly"] = ly
    return d


_c0 = config_plain_128()
_c0_small = plain_instance(64, 100, 10.0, 2.84, 50.0)
_th_small = plain_instance(32, 24, 30.0, 2.84, 50.0, window_waists=16.0)

REF_BUILDS = {
    # the reference exactly as shipped (64x64x200, 2000x1000 um window, its crystal)
    "stock": _cfg(CRYSTAL_REFERENCE, 64, 64, 200),
    "stock_thermal": _cfg(CRYSTAL_REFERENCE, 64, 64, 200, thermal=True),
    # plain 128x128x200 workload and a 64x64x100 reduction of it
    "c0": _cfg(CRYSTAL_QPM50, 128, 128, 200, _c0.lx, _c0.ly),
    "c0_small": _cfg(CRYSTAL_QPM50, 64, 64, 100, _c0_small.lx, _c0_small.ly),
    # small THERMAL grids for component and end-to-end checks
    "th_small": _cfg(CRYSTAL_QPM50, 32, 32, 24, _th_small.lx, _th_small.ly, thermal=True),
    "th_rect": _cfg(CRYSTAL_QPM50, 24, 16, 12, 900.0, 500.0, thermal=True),
    "th_mid": _cfg(CRYSTAL_QPM50, 64, 64, 100, _c0_small.lx, _c0_small.ly, thermal=True),
    # walk-off on (rho != 0) and a non-power-of-two grid
    "walkoff": _cfg(CRYSTAL_QPM50, 64, 64, 60, _c0_small.lx, _c0_small.ly) | {"rho_p": 0.01, "rho_s": 0.012},
    "odd48": _cfg(CRYSTAL_QPM50, 48, 48, 40, _c0_small.lx, _c0_small.ly),
}
