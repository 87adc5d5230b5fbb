"""The benchmarked workloads at their own sizes against the oracle (GB300 only).

* THERMAL 256x256x400, oven-surrounded faces at a seeded U(45, 55) C, P = 30 W: the whole
  Solver::run (five outer iterations with the reference's Jacobi stop rule) on the device
  and in the restatement (heat sweeps on several host threads, which changes no result),
  plus the pieces on the device's own final temperature field: heat sweeps and delta-k(T)
  bit for bit, and the fixed-temperature THERMAL CWES in FP32 and in FP64 (float delta-k).
* The 512-solve sweep: the first solve of each of the nine (N, Nz) classes at its full
  length, batched on the device, against the FP32 restatement and the FP64 run.

Bar: output fields within relative L2 1e-4 and conversion efficiency within 1e-4 relative
of the FP32 restatement (the reference's arithmetic); bit-identity where the reference's
float arithmetic is reproduced exactly. Against the FP64 run the reference's own FP32
arithmetic already differs by up to ~2.5e-4 on some solves (FFT rounding over 400 slices,
and efficiencies far from phase matching), so there the bar is 1e-4 or 1.5 times the
reference's own FP32-to-FP64 distance on the same solve, whichever is larger.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import oracle as O
from _util import ETA_RTOL, FIELD_RTOL, bits_equal, eta, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import solver as S  # noqa: E402
from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402

THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def thermal256():
    inst = W.config_thermal_256()
    s = S.Solver(crystal=W.CRYSTAL_QPM50, nx=inst.nx, ny=inst.ny, nz=inst.nz, lx=inst.lx, ly=inst.ly, thermal=True,
                 bc=inst.bc)
    s.run(inst.power, inst.waist, inst.focal, inst.temp, inst.t_inf, inst.t1, inst.t2)
    po, so = s.fields()
    dev = dict(counts=s.jacobi_counts(), T=s.temperature(), pump=po, sh=so, eta=s.efficiency())
    s.close()
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, inst.nx, inst.ny, inst.nz, inst.lx, inst.ly))
    return inst, o, dev


def test_thermal256_full_run_vs_oracle(thermal256):
    """The complete THERMAL run on both sides: Jacobi counts equal, temperatures within
    1e-4 K (they differ only through the heat source, which the fields feed), fields and
    efficiency within the bar."""
    inst, o, dev = thermal256
    O.set_threads(THREADS)
    try:
        ref = o.thermal_run(inst.power, inst.waist, inst.focal, inst.temp, inst.t_inf, inst.t1, inst.t2, bc=inst.bc)
    finally:
        O.set_threads(1)
    assert dev["counts"] == ref["counts"], (dev["counts"], ref["counts"])
    assert np.max(np.abs(dev["T"] - ref["T"])) < 1e-4
    assert rel_l2(dev["sh"], ref["sh"]) < FIELD_RTOL
    assert rel_l2(dev["pump"], ref["pump"]) < FIELD_RTOL
    nx, ny = inst.nx, inst.ny
    tc = float(ref["T"][0, ny // 2, nx // 2])
    pin = o.set_pump(inst.power, inst.focal, inst.waist, tc)
    e_ref = eta(pin, ref["sh"], o.n(1.064, tc), o.n(np.float32(0.532), tc))
    assert abs(dev["eta"] - e_ref) / e_ref < ETA_RTOL


def test_thermal256_components_on_device_temperature(thermal256):
    """On the device run's final temperature field: delta-k(T) and both indices bit-exact,
    and 40 heat sweeps (seeded heat source, oven-surrounded) bit-exact with the restatement."""
    inst, o, dev = thermal256
    T = dev["T"]
    D, NP, NS = S.dk_thermal(W.CRYSTAL_QPM50, T, lx=inst.lx, ly=inst.ly)
    assert bits_equal(D, o.dk_thermal(T))
    tt = T.ravel()[:: 4099]
    assert bits_equal(NP.ravel()[:: 4099], np.array([o.n(1.064, t) for t in tt], np.float32))
    assert bits_equal(NS.ravel()[:: 4099], np.array([o.n(np.float32(0.532), t) for t in tt], np.float32))
    rng = np.random.default_rng(40)
    Q = (rng.random(T.shape) * 5e-9).astype(np.float32)
    O.set_threads(THREADS)
    try:
        ref = o.heat_sweeps(T, Q, inst.t_inf, 40, inst.bc)
    finally:
        O.set_threads(1)
    got = S.heat_sweeps(W.CRYSTAL_QPM50, T, Q, inst.t_inf, 40, inst.bc, lx=inst.lx, ly=inst.ly)
    assert bits_equal(got, ref)


def test_thermal256_fixed_temperature_cwes(thermal256):
    """The last outer iteration's CWES runs on the final temperature field: the restatement's
    fixed-T THERMAL CWES from that field reproduces the device's output within the bar, in
    FP32 and in FP64 (delta-k pinned to the float table)."""
    inst, o, dev = thermal256
    T = dev["T"]
    nx, ny = inst.nx, inst.ny
    tc = float(T[0, ny // 2, nx // 2])
    pump = o.set_pump(inst.power, inst.focal, inst.waist, tc)
    pump64 = o.set_pump64(inst.power, inst.focal, inst.waist, tc)
    dk = o.dk_thermal(T)
    with cf.ThreadPoolExecutor(2) as ex:
        f32 = ex.submit(o.cwes_thermal, T, pump, np.zeros_like(pump), tc)
        f64 = ex.submit(o.cwes_thermal64, T, pump64, np.zeros_like(pump64), tc, dk)
        po, so = f32.result()
        po64, so64 = f64.result()
    assert rel_l2(dev["sh"], so) < FIELD_RTOL
    assert rel_l2(dev["pump"], po) < FIELD_RTOL
    e32 = eta(pump, so, o.n(1.064, tc), o.n(np.float32(0.532), tc))
    e64 = eta(pump64, so64, o.n64(1.064, tc), o.n64(0.532, tc))
    assert abs(dev["eta"] - e32) / e32 < ETA_RTOL
    assert rel_l2(dev["sh"], so64) < fp64_bar(rel_l2(so, so64))
    assert rel_l2(dev["pump"], po64) < fp64_bar(rel_l2(po, po64))
    assert abs(dev["eta"] - e64) / e64 < fp64_bar(abs(e32 - e64) / e64)


def _class_representatives():
    insts = W.config_sweep(count=512, seed=2024)
    pick = {}
    for i in insts:
        pick.setdefault((i.nx, i.nz), i)
    assert len(pick) == 9
    return [pick[k] for k in sorted(pick)]


def fp64_bar(d32):
    """Bar against the FP64 run: 1e-4, or 1.5 x the reference arithmetic's own distance."""
    return max(FIELD_RTOL, 1.5 * d32)


def _oracle_solve(inst):
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, inst.nx, inst.ny, inst.nz, inst.lx, inst.ly))
    pump = o.set_pump(inst.power, inst.focal, inst.waist, inst.temp)
    po, so, _, _ = o.cwes_plain(pump, np.zeros_like(pump), inst.temp)
    pump64 = o.set_pump64(inst.power, inst.focal, inst.waist, inst.temp)
    po64, so64, _, _ = o.cwes_plain64(pump64, np.zeros_like(pump64), inst.temp, float(o.dk_constant(inst.temp)))
    e32 = eta(pump, so, o.n(1.064, inst.temp), o.n(np.float32(0.532), inst.temp))
    e64 = eta(pump64, so64, o.n64(1.064, inst.temp), o.n64(0.532, inst.temp))
    return dict(po=po, so=so, po64=po64, so64=so64, e32=e32, e64=e64, d_so=rel_l2(so, so64),
                d_e=abs(e32 - e64) / e64)


def test_sweep512_every_class_full_length():
    """One solve of each (N, Nz) class of the 512-solve sweep, N in {64, 128, 256} and Nz in
    {100, 200, 400} at full length (256x256x400 included), batched on the device with the
    schedule the autotuner picks, against the FP32 restatement and the FP64 run."""
    pick = _class_representatives()
    with cf.ThreadPoolExecutor(min(len(pick), THREADS)) as ex:
        refs = list(ex.map(_oracle_solve, pick))
    sw = S.Sweep(pick, crystal=W.CRYSTAL_QPM50)
    eta_gpu, _ = sw.run(with_fields=True)
    pumps, shs = sw.fields()
    for k, (inst, r) in enumerate(zip(pick, refs)):
        tag = (inst.nx, inst.nz)
        assert rel_l2(shs[k], r["so"]) < FIELD_RTOL, tag
        assert rel_l2(pumps[k], r["po"]) < FIELD_RTOL, tag
        assert abs(eta_gpu[k] - r["e32"]) / r["e32"] < ETA_RTOL, tag
        assert rel_l2(shs[k], r["so64"]) < fp64_bar(r["d_so"]), (tag, rel_l2(shs[k], r["so64"]), r["d_so"])
        assert abs(eta_gpu[k] - r["e64"]) / r["e64"] < fp64_bar(r["d_e"]), (tag, eta_gpu[k], r["e64"], r["d_e"])
    sw.close()
