"""Adjoint z-march against FP64 central finite differences (GB300 only).

The finite differences use the oracle's FP64 run of the same method. The device march
uses the reference's float delta-k; the FP64 model is pinned to that value at the base
point and varies with T and the poling period as the double-precision model does
(delta-k(T) = dk32(T0) + dk64(T) - dk64(T0)), so both differentiate the same function.
Bar: agreement to 1e-3 (relative).
"""
import math
import os

import numpy as np
import pytest

import oracle as O
from _util import smooth_noise

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402
from shg_focused_gaussian_beams_gb300.autograd import gaussian_pump, shg_power  # noqa: E402
from shg_focused_gaussian_beams_gb300.solver import Solver  # noqa: E402

FD_RTOL = 1e-3
N, NZ, T0, P0 = 64, 40, 50.0, 20.0


@pytest.fixture(scope="module")
def case():
    inst = W.plain_instance(N, NZ, P0, 2.84, T0)
    cfg = O.make_cfg(W.CRYSTAL_QPM50, N, N, NZ, inst.lx, inst.ly)
    o = O.Oracle(cfg)
    rng = np.random.default_rng(31)
    pert = 1 + 0.05 * smooth_noise(rng, N)
    pump64 = o.set_pump64(inst.power, inst.focal, inst.waist, T0) * pert
    dk32 = float(o.dk_constant(T0))
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=N, ny=N, nz=NZ, lx=inst.lx, ly=inst.ly)
    pump_t = torch.from_numpy(pump64.astype(np.complex64)).cuda()
    r = s.grad(T0, pump_t, checkpoints=7)
    torch.cuda.synchronize()
    return dict(inst=inst, cfg=cfg, o=o, pump64=pump64, dk32=dk32, s=s, r=r, pert=pert, rng=rng)


def loss64(c, pump64, T=T0, lam=None):
    cfg = c["cfg"]
    o = c["o"]
    dk = c["dk32"] + (o.dk_constant64(T) - o.dk_constant64(T0))
    if lam is not None:
        dk += 2 * math.pi * (1.0 / lam - 1.0 / cfg.lambda_qpm)
    _, so, _, _ = o.cwes_plain64(pump64, np.zeros_like(pump64), T, dk)
    eps0 = float(np.float32(8.8541878128e-12 * 1e12 / 1e6))
    cl = float(np.float32(299792458 * 1e6 / 1e12))
    dx = float(np.float32(cfg.lx / (N - 1)))
    dy = float(np.float32(cfg.ly / (N - 1)))
    return 0.5 * eps0 * cl * o.n64(0.532, T) * dx * dy * float(np.sum(np.abs(so) ** 2))


def torch_loss64(c, pump):
    """The plain method (Solver.h:65-117, 156-276 with its quirks) in torch complex128, from the
    same FP64 constants as the oracle's double model (delta-k pinned to the float value):
    the reference gradient, by torch autograd, of the SH output power."""
    cfg, o = c["cfg"], c["o"]
    n, nz = cfg.nx, cfg.nz
    dev = pump.device
    pi = 3.14159265358979323846
    cl, eps0 = 299792458 * 1e6 / 1e12, 8.8541878128e-12 * 1e12 / 1e6
    lp = float(cfg.lp)
    ls = 0.5 * lp
    n_p, n_s = o.n64(lp, T0), o.n64(ls, T0)
    dq = (2.0 / pi) * float(cfg.deff)
    kp, ks = pi * dq / (n_p * lp), 0.5 * pi * dq / (n_s * ls)
    hp, hs = 0.5 * float(cfg.alpha_p), 0.5 * float(cfg.alpha_s)
    tpa = 0.5 * float(cfg.beta_s) * 0.5 * cl * eps0 * n_s
    dz = float(cfg.lz) / (nz - 1)
    hp_shift, hs_shift = (torch.from_numpy(h).to(dev) for h in o.propagators64(T0))
    dk = c["dk32"]

    def dadz(P, S, ph):
        e = torch.exp(torch.tensor(-1j * ph, dtype=torch.complex128, device=dev))
        dP = 1j * kp * S * P.conj() * e - hp * P
        dS = 1j * ks * P * P * e.conj() - (hs + tpa * (S.abs() ** 2)) * S
        return dP, dS

    def rk4(P, S, z):
        ph = z * dk
        k1 = dadz(P, S, ph)
        k2 = dadz(P + 0.5 * k1[0], S + 0.5 * k1[1], ph)
        k3 = dadz(P + 0.5 * k2[0], S + 0.5 * k2[1], ph)
        k4 = dadz(P + k3[0], S + k3[1], ph)
        return (P + dz / 6 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0]),
                S + dz / 6 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1]))

    def diffraction(A, H):
        return torch.fft.fft2(H * torch.fft.ifft2(A))

    P, S = pump, torch.zeros_like(pump)
    z = 0.0
    for _ in range(nz - 1):
        P, S = rk4(P, S, z)
        P, S = diffraction(P, hp_shift), diffraction(S, hs_shift)
        P, S = rk4(P, S, z)
        z += dz
    # the loss scale of loss64 (float-rounded eps0 and c, n_s at 0.532 um)
    eps0f = float(np.float32(8.8541878128e-12 * 1e12 / 1e6))
    clf = float(np.float32(299792458 * 1e6 / 1e12))
    dx = float(np.float32(cfg.lx / (n - 1)))
    dy = float(np.float32(cfg.ly / (n - 1)))
    return 0.5 * eps0f * clf * o.n64(0.532, T0) * dx * dy * (S.abs() ** 2).sum()


def test_gradient_field_vs_torch_fp64_reference(case):
    """The whole pump-gradient field against torch autograd through a complex128
    restatement of the method; the restatement's loss is pinned to the oracle's FP64 run."""
    p = torch.from_numpy(case["pump64"]).cuda().requires_grad_(True)
    L = torch_loss64(case, p)
    assert abs(L.item() - loss64(case, case["pump64"])) / L.item() < 1e-9
    L.backward()
    ref = p.grad.cpu().numpy()
    got = case["r"]["grad_pump"].cpu().numpy().astype(np.complex128)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < FD_RTOL, rel


@pytest.mark.parametrize("n", [16, 32, 128])
def test_gradient_field_every_grid_size(n):
    """The fused adjoint row and column passes at the grid sizes the 64^2 and 256^2 cases do
    not reach: the whole pump-gradient field (12 slices, 3 checkpoints) against torch
    autograd through the complex128 restatement."""
    nz = 12
    inst = W.plain_instance(n, nz, P0, 2.84, T0)
    cfg = O.make_cfg(W.CRYSTAL_QPM50, n, n, nz, inst.lx, inst.ly)
    o = O.Oracle(cfg)
    rng = np.random.default_rng(n)
    pump64 = o.set_pump64(inst.power, inst.focal, inst.waist, T0) * (1 + 0.05 * smooth_noise(rng, n, cells=2))
    c = dict(cfg=cfg, o=o, dk32=float(o.dk_constant(T0)))
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=n, ny=n, nz=nz, lx=inst.lx, ly=inst.ly)
    r = s.grad(T0, torch.from_numpy(pump64.astype(np.complex64)).cuda(), checkpoints=3)
    p = torch.from_numpy(pump64).cuda().requires_grad_(True)
    L = torch_loss64(c, p)
    L.backward()
    ref = p.grad.cpu().numpy()
    got = r["grad_pump"].cpu().numpy().astype(np.complex128)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < FD_RTOL
    assert abs(r["loss"] - L.item()) / L.item() < 1e-4


def test_loss_matches_fp64(case):
    L = loss64(case, case["pump64"])
    assert abs(case["r"]["loss"] - L) / L < 1e-4


def test_field_gradient_vs_fd(case):
    g = case["r"]["grad_pump"].cpu().numpy().astype(np.complex128)
    p = case["pump64"]
    rng = np.random.default_rng(7)
    adj, fd = [], []
    for _ in range(8):
        d = smooth_noise(rng, N) * p  # directions shaped like the beam
        eps = 1e-4 * np.linalg.norm(p) / np.linalg.norm(d)
        fd.append((loss64(case, p + eps * d) - loss64(case, p - eps * d)) / (2 * eps))
        adj.append(float(np.sum(np.real(np.conj(g) * d))))
    adj, fd = np.array(adj), np.array(fd)
    assert np.linalg.norm(adj - fd) / np.linalg.norm(fd) < FD_RTOL, (adj, fd)


def test_temperature_gradient_vs_fd(case):
    h = 1e-4 * T0
    fd = (loss64(case, case["pump64"], T=T0 + h) - loss64(case, case["pump64"], T=T0 - h)) / (2 * h)
    assert abs(case["r"]["dT"] - fd) / abs(fd) < FD_RTOL, (case["r"]["dT"], fd)


def test_poling_period_gradient_vs_fd(case):
    """delta-k moves by 2 pi h / Lambda^2 per step h: over the 30 mm crystal a relative step
    of 1e-4 turns the phase by 2.4 rad, far outside the linear range, so the step is 1e-7."""
    lam = case["cfg"].lambda_qpm
    h = 1e-7 * lam
    fd = (loss64(case, case["pump64"], lam=lam + h) - loss64(case, case["pump64"], lam=lam - h)) / (2 * h)
    assert abs(case["r"]["dLambda"] - fd) / abs(fd) < FD_RTOL, (case["r"]["dLambda"], fd)


@pytest.mark.parametrize("checkpoints", [1, 3, NZ - 1])
def test_checkpoint_count_does_not_change_the_gradient(case, checkpoints):
    """One segment (full replay), a few segments, and every step stored (no replay)."""
    r2 = case["s"].grad(T0, torch.from_numpy(case["pump64"].astype(np.complex64)).cuda(), checkpoints=checkpoints)
    g1 = case["r"]["grad_pump"].cpu().numpy()
    g2 = r2["grad_pump"].cpu().numpy()
    assert np.linalg.norm(g1 - g2) / np.linalg.norm(g1) < 1e-5
    assert abs(r2["dT"] - case["r"]["dT"]) / abs(case["r"]["dT"]) < 1e-5
    assert abs(r2["loss"] - case["r"]["loss"]) / case["r"]["loss"] < 1e-6


def test_graph_replay_with_new_input(case):
    """The captured gradient pass is reused across calls: a different pump in between must
    not leak into the next result."""
    s = case["s"]
    p = torch.from_numpy(case["pump64"].astype(np.complex64)).cuda()
    ra = s.grad(T0, p, checkpoints=7)
    rb = s.grad(T0, 0.5 * p, checkpoints=7)
    rc = s.grad(T0, p, checkpoints=7)
    assert rb["loss"] < 0.5 * ra["loss"]
    np.testing.assert_allclose(rc["grad_pump"].cpu().numpy(), ra["grad_pump"].cpu().numpy(), rtol=0, atol=0)
    # parameter sums are FP64 atomics (order-dependent in the last bits)
    assert abs(rc["loss"] - ra["loss"]) <= 1e-12 * ra["loss"] and abs(rc["dT"] - ra["dT"]) <= 1e-12 * abs(ra["dT"])


def test_autograd_focus_and_temperature(case):
    """torch.autograd through the adjoint: focus gradient via a torch-built pump."""
    inst = case["inst"]
    pert = torch.from_numpy(case["pert"]).cuda()
    focal = torch.tensor(inst.focal, dtype=torch.float64, device="cuda", requires_grad=True)
    temp = torch.tensor(T0, dtype=torch.float64, device="cuda", requires_grad=True)
    pump = gaussian_pump(N, N, inst.lx, inst.ly, inst.power, inst.waist, focal, T0) * pert
    L = shg_power(case["s"], pump, temp, case["cfg"].lambda_qpm, checkpoints=7)
    L.backward()
    o = case["o"]
    h = 1e-4 * inst.focal
    Lp = loss64(case, o.set_pump64(inst.power, inst.focal + h, inst.waist, T0) * case["pert"])
    Lm = loss64(case, o.set_pump64(inst.power, inst.focal - h, inst.waist, T0) * case["pert"])
    fd = (Lp - Lm) / (2 * h)
    assert abs(focal.grad.item() - fd) / abs(fd) < FD_RTOL, (focal.grad.item(), fd)
    assert abs(temp.grad.item() - case["r"]["dT"]) / abs(case["r"]["dT"]) < 1e-6


def _loss_params64(c, power, waist, focal, T, pert):
    """FP64 loss of Solver::run's plain path for the pump of (power, waist, focal) at index
    temperature T times the fixed perturbation; delta-k follows T as in loss64."""
    o = c["o"]
    return loss64(c, o.set_pump64(power, focal, waist, T) * pert, T=T)


def test_grad_run_pump_parameters_vs_fd(case):
    """shg_grad_run (Gaussian pump of setPump built on the device, times the seeded
    perturbation): focal point, waist, power and the total temperature derivative (the pump's
    index follows T too) against FP64 central differences; the pump-gradient field and the
    fixed-field derivatives equal those of shg_grad_device on the same input."""
    inst = case["inst"]
    pert = case["pert"]
    s = case["s"]
    fac = torch.from_numpy(pert.astype(np.complex64)).cuda()
    r = s.grad_run(inst.power, inst.waist, inst.focal, T0, pump_factor=fac, checkpoints=7)
    f0, w0, p0 = float(np.float32(inst.focal)), float(np.float32(inst.waist)), float(np.float32(inst.power))
    checks = [("dfocal", 1e-4 * f0, lambda h: _loss_params64(case, p0, w0, f0 + h, T0, pert)),
              ("dwaist", 1e-4 * w0, lambda h: _loss_params64(case, p0, w0 + h, f0, T0, pert)),
              ("dpower", 1e-4 * p0, lambda h: _loss_params64(case, p0 + h, w0, f0, T0, pert)),
              ("dT_total", 1e-4 * T0, lambda h: _loss_params64(case, p0, w0, f0, T0 + h, pert))]
    for key, h, fn in checks:
        fd = (fn(h) - fn(-h)) / (2 * h)
        assert abs(r[key] - fd) / abs(fd) < FD_RTOL, (key, r[key], fd)
    # the same input through shg_grad_device: pump built on the device equals the float pump
    pump32 = (case["o"].set_pump(inst.power, inst.focal, inst.waist, T0) * pert).astype(np.complex64)
    r2 = s.grad(T0, torch.from_numpy(pump32).cuda(), checkpoints=7)
    g1, g2 = r["grad_pump"].cpu().numpy(), r2["grad_pump"].cpu().numpy()
    assert np.linalg.norm(g1 - g2) / np.linalg.norm(g2) < 1e-5
    assert abs(r["dT"] - r2["dT"]) / abs(r2["dT"]) < 1e-5
    assert abs(r["loss"] - r2["loss"]) / r2["loss"] < 1e-6


def test_run_power_autograd_uses_the_c_abi_gradients(case):
    """autograd.run_power back-propagates the C ABI's pump-parameter gradients."""
    from shg_focused_gaussian_beams_gb300.autograd import run_power
    inst = case["inst"]
    fac = torch.from_numpy(case["pert"].astype(np.complex64)).cuda()
    args = [torch.tensor(v, dtype=torch.float64, device="cuda", requires_grad=True)
            for v in (inst.power, inst.waist, inst.focal, T0, case["cfg"].lambda_qpm)]
    L = run_power(case["s"], *args, pump_factor=fac, checkpoints=7)
    L.backward()
    r = case["s"].grad_run(inst.power, inst.waist, inst.focal, T0, pump_factor=fac, checkpoints=7)
    for t, key in zip(args, ("dpower", "dwaist", "dfocal", "dT_total", "dLambda")):
        assert abs(t.grad.item() - r[key]) <= 1e-9 * abs(r[key]), key
    assert abs(L.item() - r["loss"]) <= 1e-12 * r["loss"]


def _fd_job(args):
    """One FP64 loss evaluation of the full-size case in a separate process."""
    import oracle as Ox
    cfg_t, pump, T, dk = args
    o = Ox.Oracle(Ox.Cfg(*cfg_t))
    _, so, _, _ = o.cwes_plain64(pump, np.zeros_like(pump), T, dk)
    return float(np.sum(np.abs(so) ** 2)) * o.n64(0.532, T)


def test_config_adjoint_256x400_full_size():
    """The adjoint workload at full size: 256x256x400, P = 20 W, xi = 2.84, Gaussian pump
    times a seeded 5 % perturbation smooth over 8 cells, 20 checkpoints; FP64 central
    differences (run in parallel processes) on 32 seeded field directions, T, Lambda and the
    focus position (through shg_grad_run), as the adjoint workload specifies."""
    import multiprocessing as mpx
    n, nz = 256, 400
    inst = W.plain_instance(n, nz, 20.0, 2.84, T0)
    cfg = O.make_cfg(W.CRYSTAL_QPM50, n, n, nz, inst.lx, inst.ly)
    o = O.Oracle(cfg)
    rng = np.random.default_rng(12)
    pert = 1 + 0.05 * smooth_noise(rng, n)
    pump = o.set_pump64(inst.power, inst.focal, inst.waist, T0) * pert
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=n, ny=n, nz=nz, lx=inst.lx, ly=inst.ly)
    r = s.grad(T0, torch.from_numpy(pump.astype(np.complex64)).cuda(), checkpoints=20)
    rr = s.grad_run(inst.power, inst.waist, inst.focal, T0, checkpoints=20,
                    pump_factor=torch.from_numpy(pert.astype(np.complex64)).cuda())
    g = r["grad_pump"].cpu().numpy().astype(np.complex128)
    dk32 = float(o.dk_constant(T0))
    lam = cfg.lambda_qpm
    cfg_t = tuple(getattr(cfg, f) for f, _ in O.Cfg._fields_)
    eps0 = float(np.float32(8.8541878128e-12 * 1e12 / 1e6))
    cl = float(np.float32(299792458 * 1e6 / 1e12))
    kl = 0.5 * eps0 * cl * float(np.float32(inst.lx / (n - 1))) * float(np.float32(inst.ly / (n - 1)))
    dirs = [smooth_noise(rng, n) * pump for _ in range(32)]
    jobs, meta = [], []
    for d in dirs:
        eps = 1e-4 * np.linalg.norm(pump) / np.linalg.norm(d)
        jobs += [(cfg_t, pump + eps * d, T0, dk32), (cfg_t, pump - eps * d, T0, dk32)]
        meta.append(("field", 2 * eps, d))
    hT = 1e-4 * T0
    for sgn in (1, -1):
        jobs.append((cfg_t, pump, T0 + sgn * hT, dk32 + o.dk_constant64(T0 + sgn * hT) - o.dk_constant64(T0)))
    meta.append(("T", 2 * hT, None))
    hL = 1e-7 * lam
    for sgn in (1, -1):
        jobs.append((cfg_t, pump, T0, dk32 + 2 * math.pi * (1.0 / (lam + sgn * hL) - 1.0 / lam)))
    meta.append(("L", 2 * hL, None))
    # focus position: the Gaussian of setPump moved by +-h, the same perturbation
    hf = 1e-4 * inst.focal
    for sgn in (1, -1):
        jobs.append((cfg_t, o.set_pump64(inst.power, inst.focal + sgn * hf, inst.waist, T0) * pert, T0, dk32))
    meta.append(("f", 2 * hf, None))
    with mpx.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        vals = [kl * v for v in pool.map(_fd_job, jobs)]
    adj, fd = [], []
    for k, (kind, h, d) in enumerate(meta):
        fdk = (vals[2 * k] - vals[2 * k + 1]) / h
        if kind == "field":
            adj.append(float(np.sum(np.real(np.conj(g) * d))))
            fd.append(fdk)
        elif kind == "T":
            assert abs(r["dT"] - fdk) / abs(fdk) < FD_RTOL, (r["dT"], fdk)
        elif kind == "f":
            assert abs(rr["dfocal"] - fdk) / abs(fdk) < FD_RTOL, (rr["dfocal"], fdk)
        else:
            assert abs(r["dLambda"] - fdk) / abs(fdk) < FD_RTOL, (r["dLambda"], fdk)
    adj, fd = np.array(adj), np.array(fd)
    assert np.linalg.norm(adj - fd) / np.linalg.norm(fd) < FD_RTOL, (adj, fd)
    # the whole gradient field against the complex128 autograd reference
    p = torch.from_numpy(pump).cuda().requires_grad_(True)
    torch_loss64({"cfg": cfg, "o": o, "dk32": dk32}, p).backward()
    ref = p.grad.cpu().numpy()
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < FD_RTOL
