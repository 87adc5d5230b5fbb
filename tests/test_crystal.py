"""Crystal selection (no GPU): the refractive index n(L, T) of the C ABI (shg_index) for the
reference's MgO:sPPLT (Crystal.h:55-71) and for periodically poled lithium niobate, the
crystal family the reference's README names (README.md:48-49) and whose index its code does
not hold.

The PPLN index is the temperature-dependent Sellmeier fit of congruent LiNbO3 by Jundt
(Opt. Lett. 22, 1553-1555 (1997), extraordinary ray). Nothing in the reference pins it, so
the checks are: the library's host evaluation equals the oracle's and the Python workload
helper's restatements bit for bit, an independent float64 evaluation of the published
formula to float rounding, and the fit's well-known values: n_e = 2.156 at 1064 nm and
2.234 at 532 nm near room temperature, a first-order quasi-phase-matching period of about
6.8 um for 1064 -> 532 nm SHG, and a thermo-optic coefficient of a few 1e-5 per kelvin.
"""
import ctypes as C
import math

import numpy as np
import pytest


def _index(crystal, L, T):
    from shg_focused_gaussian_beams_gb300 import _lib
    n = C.c_float()
    _lib.check(_lib.lib().shg_index(crystal, L, T, C.byref(n)), "shg_index")
    return np.float32(n.value)


def _jundt64(L, T):
    a = (5.35583, 0.100473, 0.20692, 100.0, 11.34927, 1.5334e-2)
    b = (4.629e-7, 3.862e-8, -0.89e-8, 2.657e-5)
    f = (T - 24.5) * (T + 570.82)
    n2 = (a[0] + b[0] * f + (a[1] + b[1] * f) / (L * L - (a[2] + b[2] * f) ** 2) + (a[3] + b[3] * f) /
          (L * L - a[4] ** 2) - a[5] * L * L)
    return math.sqrt(n2)


@pytest.mark.parametrize("crystal", [0, 1])
def test_index_equals_the_restatements(crystal):
    import oracle as O
    from shg_focused_gaussian_beams_gb300.workloads import index_n
    for T in np.linspace(15, 95, 33, dtype=np.float32):
        for L in (np.float32(1.064), np.float32(0.532), np.float32(0.8), np.float32(1.55)):
            got = _index(crystal, L, T)
            assert got == index_n(L, T, crystal) == np.float32(O.lib().oracle_index_f32(crystal, L, T))
            if crystal == 1:
                assert abs(float(got) - _jundt64(float(L), float(T))) <= 1.2e-7 * float(got)


def test_ppln_known_values():
    from shg_focused_gaussian_beams_gb300.workloads import CRYSTAL_PPLN_QPM50, qpm_period
    assert abs(float(_index(1, 1.064, 24.5)) - 2.156) < 1e-3
    assert abs(float(_index(1, 0.532, 24.5)) - 2.234) < 1e-3
    assert 6.7 < qpm_period(50.0, crystal=1) < 6.9      # first-order QPM period, um
    assert CRYSTAL_PPLN_QPM50.crystal == 1 and CRYSTAL_PPLN_QPM50.lambda_qpm == qpm_period(50.0, crystal=1)
    dndt = float(_index(1, 1.064, 60.0)) - float(_index(1, 1.064, 50.0))
    assert 2e-5 < dndt / 10.0 < 8e-5                    # thermo-optic coefficient, 1/K


def test_unknown_crystal_is_rejected():
    from shg_focused_gaussian_beams_gb300 import _lib
    n = C.c_float()
    assert _lib.lib().shg_index(7, 1.064, 50.0, C.byref(n)) == 1
    assert b"crystal" in _lib.lib().shg_last_error()
    c = _lib.default_config()
    assert c.crystal == 0
