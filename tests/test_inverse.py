"""Host-side pieces of the Hermite-Gauss input design (CPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from shg_focused_gaussian_beams_gb300 import inverse as I  # noqa: E402
from shg_focused_gaussian_beams_gb300.autograd import C_UM_PS, EPS0  # noqa: E402
from shg_focused_gaussian_beams_gb300.workloads import sellmeier_n  # noqa: E402


def test_hermite_recurrence():
    x = torch.linspace(-2, 2, 9, dtype=torch.float64)
    assert torch.allclose(I.hermite(2, x), 4 * x ** 2 - 2)
    assert torch.allclose(I.hermite(3, x), 8 * x ** 3 - 12 * x)


def test_modes_unit_power_and_orthogonal():
    n, lx, w, f, T = 96, 463.26, 28.954, 15000.0, 50.0
    m, idx = I.hermite_gauss_modes(n, n, lx, lx, w, f, T, mmax=3, device="cpu")
    assert m.shape == (16, n, n) and idx[0] == (0, 0) and idx[-1] == (3, 3)
    dx = lx / (n - 1)
    k = 0.5 * EPS0 * C_UM_PS * float(sellmeier_n(1.064, T)) * dx * dx
    gram = k * torch.einsum("ayx,byx->ab", m.conj(), m)
    # orthonormal up to the grid's sampling of the beam (about 6 cells per waist)
    assert torch.allclose(gram, torch.eye(16, dtype=gram.dtype), atol=1e-4)


def test_fundamental_mode_is_the_reference_gaussian_shape():
    from shg_focused_gaussian_beams_gb300.autograd import gaussian_pump
    n, lx, w, f, T = 64, 463.26, 28.954, 15000.0, 50.0
    m, _ = I.hermite_gauss_modes(n, n, lx, lx, w, f, T, mmax=0, device="cpu")
    g = gaussian_pump(n, n, lx, lx, 1.0, w, f, T, device="cpu")
    # the same field up to the discrete vs continuous power normalisation
    r = m[0] / g
    assert float((r - r.mean()).abs().max()) < 1e-12 and abs(float(r.mean().real) - 1) < 1e-4


def test_admixtures_and_power_normalisation():
    c = I.seeded_admixtures(5, 16, seed=3, cmax=0.2)
    assert torch.all(c[:, 0] == 1) and float(c[:, 1:].abs().max()) <= 0.2
    assert torch.equal(c, I.seeded_admixtures(5, 16, seed=3, cmax=0.2))
    n, lx = 64, 463.26
    m, _ = I.hermite_gauss_modes(n, n, lx, lx, 28.954, 15000.0, 50.0, mmax=3, device="cpu")
    modes = m[None].expand(5, -1, -1, -1)
    P = torch.tensor([1.0, 5.0, 10.0, 20.0, 40.0], dtype=torch.float64)
    a = I.pumps_from_coefficients(c, modes, P)
    dx = lx / (n - 1)
    k = 0.5 * EPS0 * C_UM_PS * float(sellmeier_n(1.064, 50.0)) * dx * dx
    got = k * (a.abs() ** 2).sum(dim=(1, 2))
    assert torch.allclose(got, P, rtol=1e-9)
