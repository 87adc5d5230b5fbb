"""The seeded synthetic workloads are the ones the benchmark describes: grid, power, focusing,
window and temperature distributions, and the recorded total work of the 512-solve sweep
(no GPU needed)."""
import math

import numpy as np

from shg_focused_gaussian_beams_gb300 import workloads as W


def _xi(inst, temp=W.PM_TEMP_C):
    """Focusing parameter L / (2 z_R) of an instance's waist (n_p at the waist's temperature)."""
    n_p = float(W.sellmeier_n(W.LP_UM, temp))
    zr = math.pi * n_p * inst.waist ** 2 / W.LP_UM
    return W.LZ_UM / (2 * zr)


def test_phase_matched_crystal_and_plain_config():
    # Lambda_PM(50 C) = lp / (2 (n_s - n_p)) with the reference's n(L, T)
    assert abs(W.CRYSTAL_QPM50.lambda_qpm - 7.983862) < 2e-6
    c = W.config_plain_128()
    assert (c.nx, c.ny, c.nz, c.power, c.temp) == (128, 128, 200, 10.0, 50.0)
    assert abs(c.waist - 28.954) < 1e-3 and abs(_xi(c) - 2.84) < 1e-5
    assert c.lx == c.ly and abs(c.lx - 16 * c.waist) < 1e-3 and c.focal == 0.5 * W.LZ_UM


def test_thermal_config():
    c = W.config_thermal_256()
    assert (c.nx, c.ny, c.nz, c.power, c.lx, c.ly, c.bc, c.thermal) == (256, 256, 400, 30.0, 2000.0, 1000.0, 1, True)
    assert 45.0 <= c.temp <= 55.0 and c.t1 == c.t2 == c.temp
    assert W.config_thermal_256() == c  # seeded


def test_sweep_distributions_and_recorded_work():
    s = W.config_sweep()
    assert len(s) == 512 and W.config_sweep() == s
    assert {i.nx for i in s} == {64, 128, 256} and {i.nz for i in s} == {100, 200, 400}
    assert all(i.nx == i.ny and i.lx == i.ly for i in s)
    p = np.array([i.power for i in s])
    assert p.min() >= 1.0 and p.max() <= 50.0
    # log-uniform: the median sits near the geometric mean sqrt(50) W
    assert 5.0 < np.median(p) < 9.5
    assert all(48.0 <= i.temp <= 52.0 for i in s)
    xi = np.array([_xi(i) for i in s])
    assert xi.min() >= 0.5 - 1e-4 and xi.max() <= 5.0 + 1e-4
    # the work the bench line reports for this sweep (pt_steps_per_step)
    assert sum(i.pt_steps for i in s) == 3463577600


def test_thermal_adjoint_config():
    s = W.config_thermal_adjoint()
    assert len(s) == 64 and all((i.nx, i.nz, i.bc) == (256, 400, 1) for i in s)
    assert all(5.0 <= i.power <= 40.0 and 49.0 <= i.temp <= 51.0 for i in s)
