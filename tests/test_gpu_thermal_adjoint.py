"""Batched gradient of the THERMAL z-march with fixed temperature fields (GB300 only).

Forward: the batch's fixed-temperature CWES against the oracle's restatement of the
THERMAL CWES (Solver.h:245-276) with T held fixed — fields within 1e-4 relative L2 — and,
from a golden fixture's final temperature field, against the reference run's own output
(its last outer iteration ran on that field). Gradient: FP64 central differences of the
oracle's double-precision run (delta-k pinned to the float table of PhaseMatching.h:41-54)
on seeded directions, 1e-3 relative; the checkpoint count, the batch composition and graph
replay do not change it; the autograd wrapper and the Hermite-Gauss design loop use it.
"""
import math

import numpy as np
import pytest

import oracle as O
from _util import FIELD_RTOL, bits_equal, cfg_from_golden, crystal_from_golden, golden, rel_l2, smooth_noise

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402
from shg_focused_gaussian_beams_gb300 import inverse as I  # noqa: E402
from shg_focused_gaussian_beams_gb300.autograd import thermal_batch_power  # noqa: E402
from shg_focused_gaussian_beams_gb300.solver import Solver, ThermalGradBatch  # noqa: E402

FD_RTOL = 1e-3
N, NZ = 64, 60
FOCAL = float(np.float32(0.5 * 30000.0))
EPS0 = float(np.float32(8.8541878128e-12 * 1e12 / 1e6))
CL = float(np.float32(299792458 * 1e6 / 1e12))


def synthetic_T(kind):
    """Seeded smooth temperature fields with a hot spot and a z gradient (deg C)."""
    z = np.arange(NZ, dtype=np.float64)[:, None, None] / (NZ - 1)
    y = (np.arange(N) - N / 2)[None, :, None] / N
    x = (np.arange(N) - N / 2)[None, None, :] / N
    if kind == 1:
        T = 49.7 + 0.6 * np.exp(-(x ** 2 + y ** 2) / 0.02) * (0.5 + z) + 0.2 * y
    else:
        T = 50.2 - 0.4 * z + 0.3 * np.exp(-((x - 0.1) ** 2 + y ** 2) / 0.05)
    return np.broadcast_to(T, (NZ, N, N)).astype(np.float32).copy()


@pytest.fixture(scope="module")
def case():
    inst = W.plain_instance(N, NZ, 30.0, 2.84, 50.0)
    cfg = O.make_cfg(W.CRYSTAL_QPM50, N, N, NZ, inst.lx, inst.ly)
    o = O.Oracle(cfg)
    tb = ThermalGradBatch(3, crystal=W.CRYSTAL_QPM50, nx=N, ny=N, nz=NZ, lx=inst.lx, ly=inst.ly)
    counts = tb.solve_temperature(0, 30.0, inst.waist, FOCAL, 50.0)
    tb.set_temperature(1, synthetic_T(1), 20.0, inst.waist, FOCAL)
    tb.set_temperature(2, synthetic_T(2), 10.0, 1.3 * inst.waist, FOCAL)
    Ts = [tb.temperature(i) for i in range(3)]
    tcs = [float(T[0, N // 2, N // 2]) for T in Ts]
    gp = tb.gaussian_pumps()
    rng = np.random.default_rng(21)
    pumps64 = np.stack([gp[b].cpu().numpy().astype(np.complex128) * (1 + 0.05 * smooth_noise(rng, N))
                        for b in range(3)])
    pumps = torch.from_numpy(pumps64.astype(np.complex64)).cuda()
    r = tb.gradient(pumps, checkpoints=7)
    torch.cuda.synchronize()
    return dict(inst=inst, cfg=cfg, o=o, tb=tb, counts=counts, Ts=Ts, tcs=tcs, gp=gp, pumps64=pumps64,
                pumps=pumps, r=r, rng=rng)


def loss64(case, b, pump):
    o, T, tc = case["o"], case["Ts"][b], case["tcs"][b]
    _, so = o.cwes_thermal64(T, pump, np.zeros_like(pump), tc, dk3=o.dk_thermal(T))
    ns = float(o.n(np.float32(0.532), tc))
    dx = float(np.float32(case["inst"].lx / (N - 1)))
    dy = float(np.float32(case["inst"].ly / (N - 1)))
    return 0.5 * EPS0 * CL * ns * dx * dy * float(np.sum(np.abs(so) ** 2))


def test_temperature_solve_ran(case):
    # the reference rule on this case (restatement): sweeps [1, 5001, 5001, 1], T up to 50.76 C
    assert case["counts"] == [1, 5001, 5001, 1, -1]
    assert 50.7 < case["Ts"][0].max() < 50.8


def test_gaussian_reference_pump(case):
    """Efields.h:74-104 at the solve's centre temperature: the float operations are the
    reference's; only the device's expf/sincosf differ (by an ulp or two)."""
    o, inst = case["o"], case["inst"]
    for b, (p, w) in enumerate([(30.0, inst.waist), (20.0, inst.waist), (10.0, 1.3 * inst.waist)]):
        ref = o.set_pump(p, FOCAL, float(np.float32(w)), case["tcs"][b])
        assert rel_l2(case["gp"][b].cpu().numpy(), ref) < 1e-6


def test_forward_matches_oracle(case):
    tb, o = case["tb"], case["o"]
    f = tb.forward(case["pumps"], with_fields=True)
    for b in range(3):
        p32 = case["pumps64"][b].astype(np.complex64)
        po, so = o.cwes_thermal(case["Ts"][b], p32, np.zeros_like(p32), case["tcs"][b])
        assert rel_l2(f["sh_out"][b].cpu().numpy(), so) < FIELD_RTOL
        assert rel_l2(f["pump_out"][b].cpu().numpy(), po) < FIELD_RTOL
        ns, np_ = o.n(np.float32(0.532), case["tcs"][b]), o.n(1.064, case["tcs"][b])
        assert abs(f["p_sh"][b] - o.power(so, ns)) / o.power(so, ns) < FIELD_RTOL
        assert abs(f["p_in"][b] - o.power(p32, np_)) / o.power(p32, np_) < 1e-6
    # the gradient pass reports the same losses
    np.testing.assert_allclose(case["r"]["p_sh"], f["p_sh"], rtol=1e-6)


def test_forward_matches_device_thermal_run(case):
    """Solve 0's temperature came from Solver::run (THERMAL); its forward pass from the
    Gaussian pump repeats that run's last CWES."""
    inst = case["inst"]
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=N, ny=N, nz=NZ, lx=inst.lx, ly=inst.ly, thermal=True)
    s.run(30.0, inst.waist, FOCAL, 50.0)
    po, so = s.fields()
    f = case["tb"].forward(case["gp"], with_fields=True)
    assert rel_l2(f["sh_out"][0].cpu().numpy(), so) < 1e-5
    assert rel_l2(f["pump_out"][0].cpu().numpy(), po) < 1e-5
    assert np.array_equal(s.temperature(), case["Ts"][0])


@pytest.mark.parametrize("name", ["thermal_topopen.npz", "thermal_oven.npz"])
def test_forward_reproduces_reference_run_from_its_temperature(name):
    g = golden(name)
    nz, ny, nx = g["T"].shape
    tb = ThermalGradBatch(1, crystal=crystal_from_golden(g), nx=nx, ny=ny, nz=nz, lx=float(g["cfg_lx"]),
                          ly=float(g["cfg_ly"]), bc=int(g["bc"]))
    tb.set_temperature(0, g["T"], float(g["power"]), float(g["waist"]), FOCAL)
    f = tb.forward(tb.gaussian_pumps(), with_fields=True)
    assert rel_l2(f["sh_out"][0].cpu().numpy(), g["sh_out"]) < FIELD_RTOL
    assert rel_l2(f["pump_out"][0].cpu().numpy(), g["pump_out"]) < FIELD_RTOL
    o = O.Oracle(cfg_from_golden(g))
    tc = float(g["T"][0, ny // 2, nx // 2])
    psh = o.power(g["sh_out"], o.n(np.float32(0.532), tc))
    assert abs(f["p_sh"][0] - psh) / psh < FIELD_RTOL


def test_gradient_vs_fp64_fd(case):
    """Two seeded beam-shaped directions per solve; FP64 central differences."""
    g = case["r"]["grad"].cpu().numpy().astype(np.complex128)
    rng = np.random.default_rng(5)
    for b in range(3):
        p = case["pumps64"][b]
        adj, fd = [], []
        for _ in range(2):
            d = smooth_noise(rng, N) * p
            eps = 1e-4 * np.linalg.norm(p) / np.linalg.norm(d)
            fd.append((loss64(case, b, p + eps * d) - loss64(case, b, p - eps * d)) / (2 * eps))
            adj.append(float(np.sum(np.real(np.conj(g[b]) * d))))
        adj, fd = np.array(adj), np.array(fd)
        assert np.linalg.norm(adj - fd) / np.linalg.norm(fd) < FD_RTOL, (b, adj, fd)


def test_loss_matches_fp64(case):
    for b in range(3):
        ref = loss64(case, b, case["pumps64"][b])
        assert abs(case["r"]["p_sh"][b] - ref) / ref < 1e-4


@pytest.mark.parametrize("checkpoints", [1, 4, NZ - 1])
def test_checkpoint_count_does_not_change_the_gradient(case, checkpoints):
    r2 = case["tb"].gradient(case["pumps"], checkpoints=checkpoints)
    g1 = case["r"]["grad"].cpu().numpy()
    g2 = r2["grad"].cpu().numpy()
    assert np.linalg.norm(g1 - g2) / np.linalg.norm(g1) < 1e-5
    np.testing.assert_allclose(r2["p_sh"], case["r"]["p_sh"], rtol=1e-6)


def test_batch_composition(case):
    """Solve 2 alone gives the same gradient as inside the batch of three."""
    inst = case["inst"]
    tb1 = ThermalGradBatch(1, crystal=W.CRYSTAL_QPM50, nx=N, ny=N, nz=NZ, lx=inst.lx, ly=inst.ly)
    tb1.set_temperature(0, case["Ts"][2], 10.0, 1.3 * inst.waist, FOCAL)
    r1 = tb1.gradient(case["pumps"][2:3].contiguous(), checkpoints=7)
    assert bits_equal(r1["grad"][0].cpu().numpy(), case["r"]["grad"][2].cpu().numpy())
    assert abs(r1["p_sh"][0] - case["r"]["p_sh"][2]) <= 1e-12 * case["r"]["p_sh"][2]


def test_graph_replay_with_new_input(case):
    tb, p = case["tb"], case["pumps"]
    ra = tb.gradient(p, checkpoints=7)
    rb = tb.gradient(0.5 * p, checkpoints=7)
    rc = tb.gradient(p, checkpoints=7)
    assert np.all(rb["p_sh"] < 0.5 * ra["p_sh"])
    assert bits_equal(rc["grad"].cpu().numpy(), ra["grad"].cpu().numpy())


def test_autograd_wrapper(case):
    p = case["pumps"].clone().requires_grad_(True)
    L = thermal_batch_power(case["tb"], p, checkpoints=7)
    w = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64, device=p.device)
    (L * w).sum().backward()
    g = case["r"]["grad"]
    want = (w.to(torch.float32)[:, None, None] * g).cpu().numpy()
    assert np.linalg.norm(p.grad.cpu().numpy() - want) / np.linalg.norm(want) < 1e-6


def test_design_loop_raises_efficiency(case):
    """Three outer steps on Hermite-Gauss admixtures at fixed power (the gradient
    workload's loop) raise the mean efficiency."""
    inst, tb = case["inst"], case["tb"]
    waists = [inst.waist, inst.waist, 1.3 * inst.waist]
    modes = torch.stack([I.hermite_gauss_modes(N, N, inst.lx, inst.ly, float(np.float32(w)), FOCAL, tc,
                                               mmax=2)[0] for w, tc in zip(waists, case["tcs"])])
    coef0 = I.seeded_admixtures(3, modes.shape[1], seed=9, cmax=0.2)
    power = torch.tensor([30.0, 20.0, 10.0], dtype=torch.float64, device=modes.device)
    _, hist = I.optimize_inputs(tb, coef0, modes, power, steps=3, lr=0.05, checkpoints=7)
    assert hist.shape == (4, 3)
    assert hist[-1].mean() > hist[0].mean()
