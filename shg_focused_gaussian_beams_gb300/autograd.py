"""torch.autograd.Function over the adjoint z-march.

``shg_power(solver, pump, temp, lambda_qpm)`` returns the output SH power of the plain
CWES (a float64 0-dim tensor) and back-propagates to the input pump field, the oven
temperature (input fields held fixed) and the poling period through the hand-written
adjoint (``shg_grad_device``), with the checkpoint count of the solver wrapper. Build the
pump with torch operations (e.g. ``gaussian_pump``) to carry gradients on to its own
parameters (focus position, waist, power).

``run_power(solver, power, waist, focal, temp, lambda_qpm)`` is Solver::run's plain path
(Gaussian pump of setPump, optionally times a fixed complex factor) and back-propagates to
the focal point, waist, pump power, oven temperature (through the pump's index as well) and
poling period with the gradients the C ABI returns (``shg_grad_run``): the pump-parameter
derivatives are formed on the device, with no torch restatement of the pump.

``thermal_batch_power(batch, pumps)`` does the same for a batch of THERMAL solves whose
temperature fields are held fixed (``shg_thgrad_gradient``), differentiable in the pumps.
"""
from __future__ import annotations

import math

import torch

from .workloads import sellmeier_n

EPS0 = float(torch.tensor(8.8541878128e-12 * 1e12 / 1e6, dtype=torch.float32))
C_UM_PS = float(torch.tensor(299792458 * 1e6 / 1e12, dtype=torch.float32))


class _SHGPower(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pump, temp, lam, solver, checkpoints):
        if float(lam) != solver.cfg.lambda_qpm:
            solver.set_poling_period(float(lam))
        p32 = pump.detach().to(torch.complex64).contiguous()
        r = solver.grad(float(temp), p32, checkpoints=checkpoints)
        ctx.save_for_backward(r["grad_pump"])
        ctx.pump_dtype = pump.dtype
        ctx.dT = r["dT"]
        ctx.dL = r["dLambda"]
        return torch.tensor(r["loss"], dtype=torch.float64, device=pump.device)

    @staticmethod
    def backward(ctx, g):
        (gp,) = ctx.saved_tensors
        gpump = (g.to(torch.float32) * gp).to(ctx.pump_dtype)
        gT = (g * ctx.dT).reshape(()).to(torch.float64)
        gLam = (g * ctx.dL).reshape(()).to(torch.float64)
        return gpump, gT, gLam, None, None


def shg_power(solver, pump, temp, lambda_qpm, checkpoints=20):
    """Output SH power (W) of the plain CWES, differentiable in pump, temp, lambda_qpm."""
    temp = torch.as_tensor(temp, dtype=torch.float64, device=pump.device)
    lam = torch.as_tensor(lambda_qpm, dtype=torch.float64, device=pump.device)
    return _SHGPower.apply(pump, temp, lam, solver, checkpoints)


class _RunPower(torch.autograd.Function):
    @staticmethod
    def forward(ctx, power, waist, focal, temp, lam, solver, factor, checkpoints):
        if float(lam) != solver.cfg.lambda_qpm:
            solver.set_poling_period(float(lam))
        r = solver.grad_run(float(power), float(waist), float(focal), float(temp), pump_factor=factor,
                            checkpoints=checkpoints, device=power.device)
        ctx.grads = (r["dpower"], r["dwaist"], r["dfocal"], r["dT_total"], r["dLambda"])
        return torch.tensor(r["loss"], dtype=torch.float64, device=power.device)

    @staticmethod
    def backward(ctx, g):
        gs = [(g * d).reshape(()).to(torch.float64) for d in ctx.grads]
        return gs[0], gs[1], gs[2], gs[3], gs[4], None, None, None


def run_power(solver, power, waist, focal, temp, lambda_qpm, pump_factor=None, checkpoints=20, device="cuda"):
    """SH output power (W) of Solver::run's plain path, differentiable in the pump power,
    waist, focal point, oven temperature and poling period (pump_factor is held fixed)."""
    args = [torch.as_tensor(v, dtype=torch.float64, device=device)
            for v in (power, waist, focal, temp, lambda_qpm)]
    return _RunPower.apply(*args, solver, pump_factor, checkpoints)


class _ThermalBatchPower(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pump, batch, checkpoints):
        p32 = pump.detach().to(torch.complex64).contiguous()
        r = batch.gradient(p32, checkpoints=checkpoints)
        ctx.save_for_backward(r["grad"])
        ctx.pump_dtype = pump.dtype
        return torch.as_tensor(r["p_sh"], dtype=torch.float64, device=pump.device)

    @staticmethod
    def backward(ctx, g):
        (gp,) = ctx.saved_tensors
        gpump = (g.to(torch.float32)[:, None, None] * gp).to(ctx.pump_dtype)
        return gpump, None, None


def thermal_batch_power(batch, pump, checkpoints=20):
    """SH output powers (W, float64 tensor of shape (count,)) of a ThermalGradBatch for the
    input pumps (count, NY, NX), differentiable in the pumps (temperature fields fixed).
    The gradient pass runs with the forward call."""
    return _ThermalBatchPower.apply(pump, batch, checkpoints)


def gaussian_pump(nx, ny, lx, ly, power, waist, focal, temp, lp=1.064, dtype=torch.complex128, device="cuda"):
    """Focused Gaussian pump of Efields.h:74-104 as differentiable torch operations (in the
    given precision): A = Ap0/M exp(-r^2/(w^2 M)), M = 1 - i f/z_R, centre at (0.5 NX, 0.5 NY)."""
    rd = torch.float64 if dtype == torch.complex128 else torch.float32
    n_p = float(sellmeier_n(lp, float(temp)))
    power = torch.as_tensor(power, dtype=rd, device=device)
    waist = torch.as_tensor(waist, dtype=rd, device=device)
    focal = torch.as_tensor(focal, dtype=rd, device=device)
    dx, dy = lx / (nx - 1), ly / (ny - 1)
    x = (torch.arange(nx, dtype=rd, device=device) - 0.5 * nx) * dx
    y = (torch.arange(ny, dtype=rd, device=device) - 0.5 * ny) * dy
    r2 = y[:, None] ** 2 + x[None, :] ** 2
    w2 = waist * waist
    zr = math.pi * n_p * w2 / lp
    ap0 = torch.sqrt(4 * power / (EPS0 * C_UM_PS * math.pi * n_p * w2))
    M = torch.complex(torch.ones_like(zr), -focal / zr)
    return (ap0 / M) * torch.exp(-r2 / (w2 * M))
