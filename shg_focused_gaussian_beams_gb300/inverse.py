"""Input-beam design on a THERMAL crystal: gradient steps on Hermite-Gauss admixtures.

The workload behind ``ThermalGradBatch``: each solve's temperature field is solved once
(Solver::run with -DTHERMAL, Solver.h:287-340) and then held fixed; its input pump is a
superposition of Hermite-Gauss modes HG_mn (m, n <= 3) of the reference's focused beam
(Efields.h:74-104: waist w0 at the focus, focus at distance f inside the crystal),
rescaled to a fixed total power. Each outer step runs the batched forward and adjoint
z-march of all solves at once and moves the mode coefficients along the gradient of the
conversion efficiency.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .autograd import C_UM_PS, EPS0, thermal_batch_power
from .workloads import sellmeier_n


def hermite(m: int, x: torch.Tensor) -> torch.Tensor:
    """Physicists' Hermite polynomial H_m(x) by the three-term recurrence."""
    h0 = torch.ones_like(x)
    if m == 0:
        return h0
    h1 = 2 * x
    for k in range(1, m):
        h0, h1 = h1, 2 * x * h1 - 2 * k * h0
    return h1


def hermite_gauss_modes(nx, ny, lx, ly, waist, focal, temp, mmax=3, lp=1.064, device="cuda"):
    """HG_mn (m, n <= mmax) at the crystal input for the Gaussian beam of Efields.h:74-104
    (complex beam factor M = 1 - i f/z_R, centre (0.5 NX, 0.5 NY)), each scaled to unit
    power P = 1/2 eps0 c n_p sum |A|^2 dx dy. Returns ((mmax+1)^2, NY, NX) complex128 in the
    order (m, n) = (0,0), (0,1), ..., and the list of (m, n)."""
    rd = torch.float64
    n_p = float(sellmeier_n(lp, float(temp)))
    dx, dy = lx / (nx - 1), ly / (ny - 1)
    x = (torch.arange(nx, dtype=rd, device=device) - 0.5 * nx) * dx
    y = (torch.arange(ny, dtype=rd, device=device) - 0.5 * ny) * dy
    zr = math.pi * n_p * waist * waist / lp
    M = complex(1.0, -focal / zr)
    wz = waist * abs(M)
    r2 = y[:, None] ** 2 + x[None, :] ** 2
    g00 = torch.exp(-r2.to(torch.complex128) / (waist * waist * M)) / M
    gouy = M.conjugate() / abs(M)
    modes, idx = [], []
    for m in range(mmax + 1):
        for n in range(mmax + 1):
            u = hermite(m, math.sqrt(2) * x / wz)[None, :] * hermite(n, math.sqrt(2) * y / wz)[:, None]
            a = u.to(torch.complex128) * g00 * gouy ** (m + n)
            pw = 0.5 * EPS0 * C_UM_PS * n_p * dx * dy * float((a.abs() ** 2).sum())
            modes.append(a / math.sqrt(pw))
            idx.append((m, n))
    return torch.stack(modes), idx


def seeded_admixtures(count, nmodes, seed, cmax=0.2):
    """Coefficients with c_00 = 1 and the other modes drawn with |c| <= cmax (uniform
    modulus and phase), seeded."""
    g = np.random.default_rng(seed)
    c = np.zeros((count, nmodes), np.complex128)
    c[:, 0] = 1.0
    mod = g.uniform(0, cmax, (count, nmodes - 1))
    ph = g.uniform(0, 2 * math.pi, (count, nmodes - 1))
    c[:, 1:] = mod * np.exp(1j * ph)
    return torch.from_numpy(c)


def pumps_from_coefficients(coef, modes, power):
    """A_b = sqrt(P_b / P(a_b)) a_b with a_b = sum_k c_bk u_bk; P(a_b) is measured on the
    grid against the unit-power mode u_b0."""
    a = torch.einsum("bk,bkyx->byx", coef, modes)
    pw = (a.abs() ** 2).sum(dim=(1, 2)) / (modes[:, 0].abs() ** 2).sum(dim=(1, 2))
    return a * torch.sqrt(power / pw)[:, None, None]


def optimize_inputs(batch, coef0, modes, power, steps=20, lr=0.05, checkpoints=20, callback=None):
    """`steps` outer gradient steps (Adam on the real and imaginary parts of the mode
    coefficients) maximising every solve's efficiency eta_b = P_SH,b / P_b at fixed input
    power P_b. modes: (count, K, NY, NX) per-solve modes of unit power; power: (count,)
    tensor [W]. Returns (coefficients, efficiency history of shape (steps + 1, count))."""
    dev = modes.device
    c = coef0.to(dev).clone().requires_grad_(True)
    opt = torch.optim.Adam([c], lr=lr)
    hist = []
    for k in range(steps + 1):
        a = pumps_from_coefficients(c, modes, power)
        psh = thermal_batch_power(batch, a.to(torch.complex64).contiguous(), checkpoints)
        eta = psh / power
        hist.append(eta.detach().cpu().numpy())
        if callback:
            callback(k, eta.detach())
        if k == steps:
            break
        opt.zero_grad()
        (-eta.sum()).backward()
        opt.step()
    return c.detach(), np.array(hist)
