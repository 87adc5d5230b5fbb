"""Argument checks of the Python interface that run before any device call (no GPU needed):
every wrapper that hands a raw device pointer to the C ABI refuses a tensor the call would
read or write past its end, and the host-array components refuse mismatched shapes."""
import types

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from shg_focused_gaussian_beams_gb300 import solver as S  # noqa: E402


def test_device_field_refuses_host_wrongly_typed_and_short_tensors():
    c64 = torch.complex64
    with pytest.raises(ValueError, match="pump_in: .*got a torch.complex64 cpu tensor of shape \\(4, 4\\)"):
        S._device_field(torch.zeros(4, 4, dtype=c64), 16, "pump_in")
    with pytest.raises(ValueError, match="torch.complex128"):
        S._device_field(torch.zeros(4, 4, dtype=torch.complex128), 16, "x")
    with pytest.raises(ValueError, match="not contiguous"):
        S._device_field(torch.zeros(8, 8, dtype=c64)[:, ::2], 32, "x")
    with pytest.raises(ValueError, match="got ndarray"):
        S._device_field(np.zeros(16, np.complex64), 16, "x")


def test_dft2d_refuses_a_non_square_array_before_any_device_call():
    with pytest.raises(ValueError, match="square"):
        S.dft2d_device(torch.zeros(4, 8, dtype=torch.complex64), -1)
    with pytest.raises(ValueError, match="CUDA tensor"):
        S.dft2d_device(torch.zeros(8, 8, dtype=torch.complex64), -1)


def test_batched_thermal_pumps_must_cover_every_solve():
    fake = types.SimpleNamespace(count=3, ny=8, nx=8, device=0)
    with pytest.raises(ValueError, match="pump: .*192 elements"):
        S.ThermalGradBatch._check_pump(fake, torch.zeros(2, 8, 8, dtype=torch.complex64))
    with pytest.raises(ValueError, match="grad: "):
        S.ThermalGradBatch._check_pump(fake, torch.zeros(3, 8, 8, dtype=torch.complex64), "grad")


def test_heat_source_must_match_the_temperature_grid():
    T = np.zeros((4, 8, 8), np.float32)
    with pytest.raises(ValueError, match="heat source of shape"):
        S.heat_sweeps(None, T, np.zeros((4, 8, 9), np.float32), 25.0, 1, 0)


def test_host_buffers_of_a_sweep_and_a_solve_are_checked():
    """Sweep.run's caller-owned buffers and Solver.set_input_fields's arrays must hold
    exactly what the C call copies (checked before the call; the objects here are stand-ins
    with the attributes the methods read, so no device is needed)."""
    sweep = types.SimpleNamespace(n=3, field_offsets=lambda: np.array([0, 4, 8, 12]))
    with pytest.raises(ValueError, match="eta_out"):
        S.Sweep.run(sweep, eta_out=np.zeros(3, np.float32))
    with pytest.raises(ValueError, match="eta_out"):
        S.Sweep.run(sweep, eta_out=np.zeros(2))
    with pytest.raises(ValueError, match="sh_out_all"):
        S.Sweep.run(sweep, eta_out=np.zeros(3), sh_out_all=np.zeros(11, np.complex64))
    with pytest.raises(ValueError, match="with_fields"):
        S.Sweep.run(sweep, with_fields=True, sh_out_all=12345)
    solve = types.SimpleNamespace(nx=8, ny=8)
    with pytest.raises(ValueError, match="pump: 48 points"):
        S.Solver.set_input_fields(solve, np.zeros((6, 8), np.complex64))
    with pytest.raises(ValueError, match="sh: 72 points"):
        S.Solver.set_input_fields(solve, np.zeros((8, 8), np.complex64), np.zeros((9, 8), np.complex64))
