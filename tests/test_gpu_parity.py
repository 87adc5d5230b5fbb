"""CUDA path against the oracle and the reference's golden outputs (GB300 only).

Tolerance (stated bar): output fields within relative L2 1e-4 and conversion efficiency
within 1e-4 relative, against the reference's FP32 build (golden fixtures and the
bit-exact restatement) and against the FP64 run of the same method.
"""
import numpy as np
import pytest

import oracle as O
from _util import ETA_RTOL, FIELD_RTOL, cfg_from_golden, crystal_from_golden, eta, golden, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300.solver import Solver, Sweep, dft2d_device  # noqa: E402
from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256])
@pytest.mark.parametrize("sign", [-1, 1])
def test_dft2d_vs_numpy(n, sign):
    rng = np.random.default_rng(n + sign)
    a = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    ref = np.fft.fft2(a.astype(np.complex128)) if sign < 0 else np.fft.ifft2(a.astype(np.complex128)) * n * n
    x = torch.from_numpy(a).cuda()
    y = dft2d_device(x, sign)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref) < 2e-6
    # in place
    dft2d_device(x, sign, out=x)
    torch.cuda.synchronize()
    assert rel_l2(x.cpu().numpy(), ref) < 2e-6


def _solver_for(g):
    return Solver(crystal=crystal_from_golden(g), nx=int(g["cfg_nx"]), ny=int(g["cfg_ny"]), nz=int(g["cfg_nz"]),
                  lx=float(g["cfg_lx"]), ly=float(g["cfg_ly"]))


@pytest.mark.parametrize("name", ["stock_plain.npz", "c0_small.npz", "c0_128x200.npz", "walkoff.npz"])
def test_run_matches_reference_golden(name):
    """Solver::run on the device (Gaussian pump and propagators built on the device)."""
    g = golden(name)
    s = _solver_for(g)
    s.run(float(g["power"]), float(g["waist"]), float(g["focal"]), float(g["temp"]))
    po, so = s.fields()
    assert rel_l2(so, g["sh_out"]) < FIELD_RTOL
    assert rel_l2(po, g["pump_out"]) < FIELD_RTOL
    e_ref = eta(g["pump_in"], g["sh_out"], g["n_p"], g["n_s"])
    assert abs(s.efficiency() - e_ref) / e_ref < ETA_RTOL


@pytest.mark.parametrize("name", ["c0_small.npz", "stock_plain.npz"])
def test_cwes_from_given_fields_matches_oracle(name):
    """Arbitrary input fields (host API) against the bit-exact restatement."""
    g = golden(name)
    o = O.Oracle(cfg_from_golden(g))
    temp = float(g["temp"])
    rng = np.random.default_rng(5)
    pump = g["pump_in"] * (1 + 0.05 * (rng.standard_normal(g["pump_in"].shape) +
                                       1j * rng.standard_normal(g["pump_in"].shape)))
    pump = pump.astype(np.complex64)
    sh = (0.01 * pump * np.exp(1j * rng.uniform(0, 6.28, pump.shape))).astype(np.complex64)
    po_r, so_r, _, _ = o.cwes_plain(pump, sh, temp)
    s = _solver_for(g)
    s.set_input_fields(pump, sh)
    s.cwes(temp)
    po, so = s.fields()
    assert rel_l2(so, so_r) < FIELD_RTOL
    assert rel_l2(po, po_r) < FIELD_RTOL


@pytest.mark.parametrize("march", ["auto", "streaming"])
@pytest.mark.parametrize("n", [16, 32, 64, 128, 256])
def test_lone_solve_every_grid_size_vs_oracle(n, march, monkeypatch):
    """A lone streaming solve runs the one-thread-per-point row pass and the narrow-tile
    column pass; every compiled grid size, with the schedule the autotuner picks and with
    the streaming passes forced, against the oracle's FP32 restatement (perturbed fields,
    SH seeded, 12 slices)."""
    monkeypatch.setenv("SHG_MARCH", march)
    inst = W.plain_instance(n, 12, 20.0, 2.84, 50.0)
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, n, n, 12, inst.lx, inst.ly))
    rng = np.random.default_rng(n)
    pump = o.set_pump(inst.power, inst.focal, inst.waist, inst.temp)
    pump = (pump * (1 + 0.05 * (rng.standard_normal(pump.shape) + 1j * rng.standard_normal(pump.shape))))
    pump = pump.astype(np.complex64)
    sh = (0.01 * pump * np.exp(1j * rng.uniform(0, 6.28, pump.shape))).astype(np.complex64)
    po_r, so_r, _, _ = o.cwes_plain(pump, sh, inst.temp)
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=n, ny=n, nz=12, lx=inst.lx, ly=inst.ly)
    s.set_input_fields(pump, sh)
    s.cwes(inst.temp)
    po, so = s.fields()
    assert rel_l2(so, so_r) < FIELD_RTOL
    assert rel_l2(po, po_r) < FIELD_RTOL


def test_device_pointer_cwes_matches_host_api():
    g = golden("c0_small.npz")
    s = _solver_for(g)
    temp = float(g["temp"])
    s.set_input_fields(g["pump_in"])
    s.cwes(temp)
    po_h, so_h = s.fields()
    p = torch.from_numpy(g["pump_in"]).cuda()
    po_d, so_d = s.cwes_device(temp, p)
    torch.cuda.synchronize()
    assert np.array_equal(so_d.cpu().numpy(), so_h)
    assert np.array_equal(po_d.cpu().numpy(), po_h)


def test_fp64_parity_config_plain_128():
    """Plain 128x128x200 workload: efficiency within 1e-4 of the FP64 run (FP32 delta-k)."""
    g = golden("c0_128x200.npz")
    o = O.Oracle(cfg_from_golden(g))
    temp = float(g["temp"])
    pump64 = o.set_pump64(float(g["power"]), float(g["focal"]), float(g["waist"]), temp)
    _, so64, _, _ = o.cwes_plain64(pump64, np.zeros_like(pump64), temp, float(g["dk"]))
    e64 = eta(pump64, so64, o.n64(1.064, temp), o.n64(0.532, temp))
    s = _solver_for(g)
    s.run(float(g["power"]), float(g["waist"]), float(g["focal"]), temp)
    _, so = s.fields()
    assert abs(s.efficiency() - e64) / e64 < ETA_RTOL
    assert rel_l2(so, so64) < FIELD_RTOL


def test_sweep_matches_oracle_and_single_solves():
    insts = W.config_sweep(count=512, seed=2024)
    # a spread of sizes and step counts, kept small enough for the CPU oracle
    pick = [i for i in insts if i.nx <= 128 and i.nz <= 200][:10] + [i for i in insts if i.nx == 256][:2]
    pick = [W.Instance(**{**i.as_dict(), "nz": min(i.nz, 100)}) for i in pick]
    sw = Sweep(pick, crystal=W.CRYSTAL_QPM50)
    eta_gpu, fields = sw.run(with_fields=True)
    cfg = O.make_cfg(W.CRYSTAL_QPM50, 64, 64, 100)
    eta_cpu = O.sweep_plain(cfg, pick, threads=8)
    np.testing.assert_allclose(eta_gpu, eta_cpu, rtol=ETA_RTOL, atol=0)
    # the batched result equals the single-solve path
    k = 0
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=pick[k].nx, ny=pick[k].ny, nz=pick[k].nz, lx=pick[k].lx, ly=pick[k].ly)
    s.run(pick[k].power, pick[k].waist, pick[k].focal, pick[k].temp)
    _, so = s.fields()
    assert rel_l2(fields[k], so) < 1e-6
    # repeated runs (graph replay) agree; the double-precision power sums are accumulated
    # with atomics, so only their last bits may differ
    np.testing.assert_allclose(sw.run(), eta_gpu, rtol=1e-12, atol=0)
    assert sw.launch_count() > 0


def test_errors_are_reported():
    from shg_focused_gaussian_beams_gb300._lib import ShgError
    with pytest.raises(ShgError, match="UNSUPPORTED"):
        Solver(nx=48, ny=48, nz=10)
    with pytest.raises(ShgError, match="UNSUPPORTED"):
        Solver(nx=64, ny=32, nz=10)
    s = Solver(nx=32, ny=32, nz=10)
    with pytest.raises(ShgError, match="STATE"):
        s.fields()
    with pytest.raises(ShgError, match="STATE"):
        s.cwes(50.0)


RESIDENT_VARIANTS = {64: [(1, 1), (1, 2), (2, 2), (2, 4), (4, 4), (8, 8)],
                     128: [(2, 1), (4, 1), (4, 2), (8, 4), (16, 8)], 256: [(8, 1), (16, 1), (16, 2)]}


def test_every_schedule_gives_identical_fields():
    """Every resident variant (cluster size, CTAs per SM) with the default line-FFT split
    runs the same arithmetic as the streaming row/column kernels: identical output fields
    for every size class; the other split agrees to rounding; the autotuner's choice runs."""
    from shg_focused_gaussian_beams_gb300._lib import ShgError
    insts = W.config_sweep(count=512, seed=77)
    pick = [i for i in insts if i.nx == 64][:5] + [i for i in insts if i.nx == 128][:4] + \
        [i for i in insts if i.nx == 256][:3]
    pick = [W.Instance(**{**i.as_dict(), "nz": min(i.nz, 60)}) for i in pick]
    ref = Sweep(pick, crystal=W.CRYSTAL_QPM50)
    for n in RESIDENT_VARIANTS:
        ref.set_schedule(n, resident=False)
    eta_r, fr = ref.run(with_fields=True)
    ran = {n: 0 for n in RESIDENT_VARIANTS}
    for k in range(6):
        sw = Sweep(pick, crystal=W.CRYSTAL_QPM50)
        for n, vs in RESIDENT_VARIANTS.items():
            cs, mb = vs[min(k, len(vs) - 1)]
            try:
                sw.set_schedule(n, True, cs, mb)
                ran[n] += 1
            except ShgError as e:  # a variant that does not fit this device
                assert "UNSUPPORTED" in str(e)
                sw.set_schedule(n, resident=False)
        eta, f = sw.run(with_fields=True)
        for x, y in zip(f, fr):
            assert np.array_equal(x, y)
        np.testing.assert_allclose(eta, eta_r, rtol=1e-12, atol=0)
    assert all(v > 0 for v in ran.values()), ran
    # the other line-FFT split of the 64-point grid (16 x 4 instead of 8 x 8): same method,
    # different rounding
    alt = Sweep(pick, crystal=W.CRYSTAL_QPM50)
    alt.set_schedule(64, True, 1, 1, threads_per_line=4)
    alt.set_schedule(128, resident=False)
    alt.set_schedule(256, resident=False)
    _, fa = alt.run(with_fields=True)
    for x, y, inst in zip(fa, fr, pick):
        if inst.nx == 64:
            assert 0 < rel_l2(x, y) < FIELD_RTOL
        else:
            assert np.array_equal(x, y)
    at = Sweep(pick, crystal=W.CRYSTAL_QPM50)
    at.autotune()
    text = at.schedule()
    assert "untuned" not in text and all(f"n={n}" in text for n in RESIDENT_VARIANTS), text
    eta_t, ft = at.run(with_fields=True)
    for x, y in zip(ft, fr):
        assert rel_l2(x, y) < FIELD_RTOL


def test_schedule_list_from_environment(monkeypatch):
    """SHG_MARCH lists a schedule per grid; unlisted grids go to the autotuner."""
    monkeypatch.setenv("SHG_MARCH", "64:streaming,128:4/2")
    insts = W.config_sweep(count=512, seed=5)
    pick = [i for i in insts if i.nx == 64][:2] + [i for i in insts if i.nx == 128][:2] + \
        [i for i in insts if i.nx == 256][:1]
    pick = [W.Instance(**{**i.as_dict(), "nz": min(i.nz, 30)}) for i in pick]
    sw = Sweep(pick, crystal=W.CRYSTAL_QPM50)
    text = sw.schedule()
    assert "n=64 solves=2: streaming" in text and "n=128 solves=2: resident cs=4 minb=2" in text
    assert "n=256 solves=1: untuned" in text
    sw.run()
    assert "untuned" not in sw.schedule()


@pytest.mark.parametrize("n,nz", [(32, 40), (64, 60), (128, 100), (256, 48)])
def test_persistent_grid_matches_streaming(n, nz):
    """A batch of one solve on the persistent cooperative grid (the whole march in one
    launch, grid-wide barriers between the row and column passes) gives the streaming
    kernels' fields bit for bit, on repeated runs of the captured graph."""
    inst = W.plain_instance(n, nz, 10.0, 2.84, 50.0)
    ref = Sweep([inst], crystal=W.CRYSTAL_QPM50)
    ref.set_schedule(n, resident=False)
    eta_r, fr = ref.run(with_fields=True)
    sw = Sweep([inst], crystal=W.CRYSTAL_QPM50)
    sw.set_schedule(n, resident="coop")
    assert "coop" in sw.schedule() and sw.launch_count() == 3
    for _ in range(3):
        eta, f = sw.run(with_fields=True)
        for x, y in zip(f, fr):
            assert np.array_equal(x, y)
        # the power sums are double atomics: order-dependent in the last bits
        np.testing.assert_allclose(eta, eta_r, rtol=1e-12, atol=0)
    ref.close()
    sw.close()


def test_persistent_grid_is_offered_to_a_lone_solve_only(monkeypatch):
    from shg_focused_gaussian_beams_gb300._lib import ShgError
    insts = [W.plain_instance(64, 20, p, 2.84, 50.0) for p in (5.0, 10.0)]
    sw = Sweep(insts, crystal=W.CRYSTAL_QPM50)
    with pytest.raises(ShgError, match="UNSUPPORTED"):
        sw.set_schedule(64, resident="coop")
    sw.close()
    monkeypatch.setenv("SHG_MARCH", "64:coop")
    lone = Sweep(insts[:1], crystal=W.CRYSTAL_QPM50)
    assert "coop" in lone.schedule()
    two = Sweep(insts, crystal=W.CRYSTAL_QPM50)
    assert "untuned" in two.schedule()
    lone.close()
    two.close()
    # the autotuner times it among the candidates of a lone solve
    monkeypatch.delenv("SHG_MARCH")
    at = Sweep([W.plain_instance(128, 30, 10.0, 2.84, 50.0)], crystal=W.CRYSTAL_QPM50)
    at.autotune()
    assert "coop" in at.schedule()
    at.close()


@pytest.mark.parametrize("n,nzs", [(64, [60]), (128, [100]), (256, [48]), (128, [40, 25, 40]), (64, [30, 20])])
def test_cluster_march_matches_streaming(n, nzs):
    """The cluster march (one cluster per solve, both fields in the cluster's shared memory,
    one thread per point in the pointwise phase) gives the streaming kernels' fields bit for
    bit, for a lone solve and for a batch of solves of different lengths, on repeated runs of
    the captured graph."""
    insts = [W.plain_instance(n, nz, 10.0 + 5.0 * i, 2.84, 50.0 + 0.5 * i) for i, nz in enumerate(nzs)]
    ref = Sweep(insts, crystal=W.CRYSTAL_QPM50)
    ref.set_schedule(n, resident=False)
    eta_r, fr = ref.run(with_fields=True)
    sw = Sweep(insts, crystal=W.CRYSTAL_QPM50)
    sw.set_schedule(n, resident="cluster")
    assert "cluster march" in sw.schedule() and sw.launch_count() == 3
    for _ in range(2):
        eta, f = sw.run(with_fields=True)
        for x, y in zip(f, fr):
            assert np.array_equal(x, y)
        np.testing.assert_allclose(eta, eta_r, rtol=1e-12, atol=0)
    ref.close()
    sw.close()


@pytest.mark.parametrize("nz", [2, 3])
@pytest.mark.parametrize("n,schedules", [(64, ["streaming", "1/1", "8/8", "coop", "cluster"]),
                                         (128, ["streaming", "2/1", "16/8", "coop", "cluster"]),
                                         (256, ["streaming", "16/2", "coop", "cluster"])])
def test_shortest_solves_on_every_schedule_vs_oracle(n, schedules, nz):
    """The shortest marches the method allows (NZ = 2: one SSFM step; NZ = 3) on the streaming
    passes, resident clusters, the persistent grid and the cluster march, against the oracle:
    the first and last stage of a march coincide or touch, and no schedule may drop or repeat
    one."""
    inst = W.plain_instance(n, nz, 25.0, 2.84, 50.0)
    po_r, so_r = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, n, n, nz, inst.lx, inst.ly)).run_plain(
        inst.power, inst.waist, inst.focal, inst.temp)
    for sched in schedules:
        sw = Sweep([inst], crystal=W.CRYSTAL_QPM50)
        if sched in ("streaming", "coop", "cluster"):
            sw.set_schedule(n, resident=False if sched == "streaming" else sched)
        else:
            cs, mb = (int(v) for v in sched.split("/"))
            sw.set_schedule(n, cluster_size=cs, ctas_per_sm=mb)
        _, f = sw.run(with_fields=True)
        sw.close()
        assert rel_l2(f[0], so_r) < FIELD_RTOL, sched
