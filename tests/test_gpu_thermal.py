"""THERMAL path on the device against the reference (GB300 only).

The heat stencil, the initial temperature and delta-k(T) must be bit-identical to the
reference's build (golden fixtures). A full THERMAL run must take the reference's
Jacobi sweep counts and agree within the parity bar (fields 1e-4 relative L2, efficiency
1e-4); its temperature differs only through the heat source, which depends on the fields.
"""
import numpy as np
import pytest

import oracle as O
from _util import ETA_RTOL, FIELD_RTOL, bits_equal, cfg_from_golden, crystal_from_golden, eta, golden, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import solver as S  # noqa: E402
from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402

FOCAL = float(np.float32(0.5 * 30000.0))


def _geom(g):
    return dict(lx=float(g["cfg_lx"]), ly=float(g["cfg_ly"]))


def test_tma_wait_timeout_is_reported_and_recoverable(monkeypatch):
    """Failure detection without a GPU fault: with the producer issuing no copies
    (SHG_HEAT_TMA_STARVE=1) every consumer wait of the TMA-staged sweep runs out after its
    bounded number of polls, the kernel sets its error flag and returns, and the host call
    reports the error. The next sweeps in the same process are bit-exact again."""
    from shg_focused_gaussian_beams_gb300._lib import ShgError
    monkeypatch.setenv("SHG_HEAT", "tma")
    monkeypatch.setenv("SHG_HEAT_TB", "1")
    n, nz = 40, 33
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, n, n, nz, 600.0, 600.0))
    rng = np.random.default_rng(3)
    T = o.init_temperature(48.0, 50.0, 46.5, 1)
    T = (T + rng.normal(0, 0.05, T.shape)).astype(np.float32)
    Q = (rng.random(T.shape) * 5e-9).astype(np.float32)
    monkeypatch.setenv("SHG_HEAT_TMA_STARVE", "1")
    with pytest.raises(ShgError, match="TMA pipeline wait gave up"):
        S.heat_sweeps(W.CRYSTAL_QPM50, T, Q, 25.0, 1, 1, lx=600.0, ly=600.0)
    monkeypatch.delenv("SHG_HEAT_TMA_STARVE")
    ref = o.heat_sweeps(T, Q, 25.0, 3, 1)
    got = S.heat_sweeps(W.CRYSTAL_QPM50, T, Q, 25.0, 3, 1, lx=600.0, ly=600.0)
    assert bits_equal(got, ref)


@pytest.mark.parametrize("name", ["thermal_topopen.npz", "thermal_oven.npz"])
def test_heat_components_bitexact(name):
    g = golden(name)
    cr = crystal_from_golden(g)
    nz, ny, nx = g["T0"].shape
    bc = int(g["bc"])
    T0 = S.init_temperature(cr, nx, ny, nz, float(g["temp"]), float(g["t1"]), float(g["t2"]), bc, **_geom(g))
    assert bits_equal(T0, g["T0"])
    T37 = S.heat_sweeps(cr, g["T0"], g["Q"], 25.0, 37, bc, **_geom(g))
    assert bits_equal(T37, g["T37"])
    D, NP, NS = S.dk_thermal(cr, g["T"], **_geom(g))
    assert bits_equal(D, g["dk_T"])


def test_heat_sweeps_bitexact_vs_oracle_random():
    cfg = O.make_cfg(W.CRYSTAL_QPM50, 64, 64, 40, 900.0, 450.0)
    o = O.Oracle(cfg)
    rng = np.random.default_rng(4)
    for bc in (0, 1):
        T = o.init_temperature(47.0, 49.0, 45.5, bc)
        T = (T + rng.normal(0, 0.01, T.shape)).astype(np.float32)
        Q = (rng.random(T.shape) * 5e-9).astype(np.float32)
        ref = o.heat_sweeps(T, Q, 25.0, 61, bc)
        got = S.heat_sweeps(W.CRYSTAL_QPM50, T, Q, 25.0, 61, bc, lx=900.0, ly=450.0)
        assert bits_equal(got, ref)
    D, NP, NS = S.dk_thermal(W.CRYSTAL_QPM50, T, lx=900.0, ly=450.0)
    assert bits_equal(D, o.dk_thermal(T))


@pytest.mark.parametrize("kind,levels,shape", [("ws8", "1", (40, 40, 33)), ("ws4", "1", (40, 40, 33)),
                                               ("ws4b", "1", (40, 40, 33)), ("tma", "1", (40, 40, 33)),
                                               ("tma", "1", (44, 44, 35)), ("tma1", "1", (44, 44, 35)),
                                               ("tma2", "1", (44, 44, 35)), ("tma8", "1", (44, 44, 35)),
                                               ("tma8", "1", (72, 72, 9)), ("tma4", "1", (136, 136, 11)),
                                               ("25", "1", (40, 40, 33)),
                                               ("simple", "1", (40, 40, 33)), ("ws4", "2", (40, 40, 33)),
                                               ("ws4", "3", (40, 40, 33)), ("ws4", "4", (40, 40, 33))])
def test_heat_kernels_bitexact(kind, levels, shape, monkeypatch):
    """Every heat-sweep kernel (warp strips of 8 or 4 rows, the TMA-staged tile, the 2.5D
    tile, the plain kernel) and K sweeps per launch (temporal blocking) equal the reference's
    sweeps bit for bit: grids that the tile sizes do not divide (nx x ny x nz given),
    sweep counts around multiples of K, both BC modes."""
    monkeypatch.setenv("SHG_HEAT", kind)
    monkeypatch.setenv("SHG_HEAT_TB", levels)
    nx, ny, nz = shape
    cfg = O.make_cfg(W.CRYSTAL_QPM50, nx, ny, nz, 600.0, 600.0)
    o = O.Oracle(cfg)
    rng = np.random.default_rng(11)
    for bc in (0, 1):
        T = o.init_temperature(48.0, 50.0, 46.5, bc)
        T = (T + rng.normal(0, 0.05, T.shape)).astype(np.float32)
        Q = (rng.random(T.shape) * 5e-9).astype(np.float32)
        for ns in (1, 3, 4, 5, 9):
            ref = o.heat_sweeps(T, Q, 25.0, ns, bc)
            got = S.heat_sweeps(W.CRYSTAL_QPM50, T, Q, 25.0, ns, bc, lx=600.0, ly=600.0)
            assert bits_equal(got, ref), (bc, ns)


@pytest.mark.parametrize("name", ["thermal_topopen.npz", "thermal_oven.npz"])
def test_thermal_run_matches_reference(name):
    g = golden(name)
    nz, ny, nx = g["T"].shape
    s = S.Solver(crystal=crystal_from_golden(g), nx=nx, ny=ny, nz=nz, thermal=True, bc=int(g["bc"]), **_geom(g))
    s.run(float(g["power"]), float(g["waist"]), FOCAL, float(g["temp"]), 25.0, float(g["t1"]), float(g["t2"]))
    assert s.jacobi_counts() == list(g["counts"])
    po, so = s.fields()
    assert rel_l2(so, g["sh_out"]) < FIELD_RTOL
    assert rel_l2(po, g["pump_out"]) < FIELD_RTOL
    T = s.temperature()
    assert np.max(np.abs(T - g["T"])) < 1e-4
    o = O.Oracle(cfg_from_golden(g))
    tc = float(g["T"][0, ny // 2, nx // 2])
    pin = o.set_pump(float(g["power"]), FOCAL, float(g["waist"]), tc)
    e_ref = eta(pin, g["sh_out"], o.n(1.064, tc), o.n(np.float32(0.532), tc))
    assert abs(s.efficiency() - e_ref) / e_ref < ETA_RTOL


def test_thermal_run_64_oven_vs_oracle():
    """64x64x60 oven-surrounded run against the restatement (five outer iterations)."""
    inst = W.plain_instance(64, 60, 25.0, 2.84, 51.0)
    cfg = O.make_cfg(W.CRYSTAL_QPM50, 64, 64, 60, inst.lx, inst.ly)
    ref = O.Oracle(cfg).thermal_run(25.0, inst.waist, FOCAL, 51.0, 25.0, 51.0, 51.0, bc=1)
    s = S.Solver(crystal=W.CRYSTAL_QPM50, nx=64, ny=64, nz=60, lx=inst.lx, ly=inst.ly, thermal=True, bc=1)
    s.run(25.0, inst.waist, FOCAL, 51.0, 25.0, 51.0, 51.0)
    assert s.jacobi_counts() == ref["counts"]
    po, so = s.fields()
    assert rel_l2(so, ref["sh"]) < FIELD_RTOL
    assert np.max(np.abs(s.temperature() - ref["T"])) < 1e-4


def test_relative_residual_stop_rule():
    """The THERMAL workload's relative-residual rule: each Jacobi solve stops once one
    sweep changes T by less than 1e-6 relative; the counts differ from the reference rule's
    and the fields agree to the convergence level of the two rules (Jacobi converges slowly,
    so a 1e-6 relative step leaves a residual error of a fraction of a kelvin)."""
    inst = W.plain_instance(64, 60, 25.0, 2.84, 51.0)
    a = S.Solver(crystal=W.CRYSTAL_QPM50, nx=64, ny=64, nz=60, lx=inst.lx, ly=inst.ly, thermal=True, bc=1)
    a.run(25.0, inst.waist, FOCAL, 51.0, 25.0, 51.0, 51.0)
    b = S.Solver(crystal=W.CRYSTAL_QPM50, nx=64, ny=64, nz=60, lx=inst.lx, ly=inst.ly, thermal=True, bc=1)
    b.set_jacobi_rule(1e-6, check_every=50)
    b.run(25.0, inst.waist, FOCAL, 51.0, 25.0, 51.0, 51.0)
    assert 0 <= b.jacobi_residual() < 1e-6
    cb = b.jacobi_counts()
    assert cb[0] >= 50 and all(c % 50 == 0 for c in cb if c > 0)
    assert cb != a.jacobi_counts()
    assert np.max(np.abs(b.temperature() - a.temperature())) < 0.25
    assert abs(b.efficiency() - a.efficiency()) / a.efficiency() < 0.1


@pytest.mark.parametrize("n,nz,bc", [(64, 40, 1), (256, 24, 0), (32, 16, 1)])
def test_persistent_thermal_march_matches_streaming(n, nz, bc, monkeypatch):
    """The THERMAL march as one persistent cooperative launch (row and column passes between
    bounded grid barriers) gives the two-launches-per-step march's fields, temperature and
    Jacobi counts bit for bit, over a whole Solver::run (five outer iterations)."""
    inst = W.plain_instance(n, nz, 25.0, 2.84, 51.0)
    out = {}
    for mode in ("streaming", "coop"):
        monkeypatch.setenv("SHG_THERMAL_MARCH", mode)
        s = S.Solver(crystal=W.CRYSTAL_QPM50, nx=n, ny=n, nz=nz, lx=inst.lx, ly=inst.ly, thermal=True, bc=bc)
        s.run(25.0, inst.waist, FOCAL, 51.0, 25.0, 51.0, 51.0)
        out[mode] = (s.fields(), s.temperature(), s.jacobi_counts(), s.efficiency())
        s.close()
    (fs, Ts, cs, es), (fc, Tc, cc, ec) = out["streaming"], out["coop"]
    assert cs == cc
    assert bits_equal(Ts, Tc)
    for a, b in zip(fs, fc):
        assert bits_equal(a, b)
    assert abs(es - ec) <= 1e-12 * abs(es)
