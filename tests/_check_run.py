"""Child process of tests/test_gpu_check.py (not collected): small solves through a
diagnostic build of the library, selected with SHG_LIB.

mode "check": the SHG_CHECK build. Its reporting path is shown first (a self-test kernel
records a failure without touching memory), then every kernel family runs at 16-64 point
grids: the plain march on each schedule (streaming, resident variants, persistent grid,
cluster march), THERMAL runs (TMA heat sweep), heat-sweep and delta-k components, the
adjoint, the batched THERMAL adjoint and the allocation-free entry point. Results are held
to the oracle at the usual bar, and no check may fail.

mode "sanitize": the host code built with AddressSanitizer and UBSan (the parent preloads
the runtime). Host-buffer paths only: plain and THERMAL runs with their file outputs, the
batch with its schedules, the heat components, argument errors.

mode "host": the sanitizer build's paths that need no GPU (crystal indices, argument
errors), for the CPU test suite.

mode "fullsize": the SHG_CHECK build on the benchmarked workloads at their own sizes.

Prints one JSON line; exit status 0 when every comparison held.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [ROOT, HERE, os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from _util import FIELD_RTOL, bits_equal, rel_l2  # noqa: E402
from shg_focused_gaussian_beams_gb300 import _lib  # noqa: E402
from shg_focused_gaussian_beams_gb300 import solver as S  # noqa: E402
from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402

MODE = sys.argv[1]
CR = W.CRYSTAL_QPM50
FOCAL = float(np.float32(0.5 * 30000.0))
report = {"mode": MODE, "lib": _lib.LIB_PATH, "cases": {}}
ok = True


def record(name, good, **info):
    global ok
    ok &= bool(good)
    report["cases"][name] = {"ok": bool(good), **info}


def status():
    e, s, v = C.c_int(), C.c_int(), C.c_longlong()
    _lib.check(_lib.lib().shg_check_status(C.byref(e), C.byref(s), C.byref(v)), "shg_check_status")
    return e.value, s.value, v.value


def plain_cases():
    for n, nz in ((16, 12), (32, 20), (64, 24)):
        inst = W.plain_instance(n, nz, 10.0, 2.84, 50.0)
        s = S.Solver(crystal=CR, nx=n, ny=n, nz=nz, lx=inst.lx, ly=inst.ly)
        out = tempfile.mkdtemp(prefix="shg_chk_")
        s.set_output_dir(out)
        s.run(inst.power, inst.waist, inst.focal, inst.temp)
        po, so = s.fields()
        s.close()
        ref_p, ref_s = O.Oracle(O.make_cfg(CR, n, n, nz, inst.lx, inst.ly)).run_plain(inst.power, inst.waist,
                                                                                      inst.focal, inst.temp)
        e = max(rel_l2(so, ref_s), rel_l2(po, ref_p))
        record(f"plain{n}x{nz}", e < FIELD_RTOL, rel_l2=e, files=len(os.listdir(out)))


def schedule_cases():
    for n, nz in ((16, 10), (32, 12), (64, 16)):
        insts = [W.plain_instance(n, nz, p, 2.84, 50.0) for p in (5.0, 12.0)]
        ref = S.Sweep(insts, crystal=CR)
        ref.set_schedule(n, resident=False)
        eta_r, f_r = ref.run(with_fields=True)
        ref.close()
        scheds = [dict(resident=True, cluster_size=1, ctas_per_sm=1)]
        if n == 64:
            scheds += [dict(resident=True, cluster_size=cs, ctas_per_sm=mb) for cs, mb in ((1, 2), (2, 2), (2, 4),
                                                                                          (4, 4), (8, 8))]
        for kw in scheds:
            sw = S.Sweep(insts, crystal=CR)
            sw.set_schedule(n, **kw)
            eta, f = sw.run(with_fields=True)
            sw.close()
            record(f"sweep{n}:{kw['cluster_size']}/{kw['ctas_per_sm']}", all(bits_equal(a, b) for a, b in zip(f, f_r)))
        for mode in ("coop", "cluster"):
            lone = S.Sweep(insts[:1], crystal=CR)
            try:
                lone.set_schedule(n, resident=mode)
            except _lib.ShgError:
                lone.close()
                continue
            eta, f = lone.run(with_fields=True)
            lone.close()
            record(f"sweep{n}:{mode}", bits_equal(f[0], f_r[0]))


def thermal_cases():
    n, nz = 32, 16
    inst = W.plain_instance(n, nz, 25.0, 2.84, 51.0)
    for bc in (0, 1):
        s = S.Solver(crystal=CR, nx=n, ny=n, nz=nz, lx=inst.lx, ly=inst.ly, thermal=True, bc=bc)
        s.run(25.0, inst.waist, FOCAL, 51.0, 25.0, 51.0, 51.0)
        po, so = s.fields()
        counts = s.jacobi_counts()
        s.close()
        ref = O.Oracle(O.make_cfg(CR, n, n, nz, inst.lx, inst.ly)).thermal_run(25.0, inst.waist, FOCAL, 51.0, 25.0,
                                                                              51.0, 51.0, bc=bc)
        e = rel_l2(so, ref["sh"])
        record(f"thermal{n}x{nz}:bc{bc}", e < FIELD_RTOL and list(counts) == list(ref["counts"]), rel_l2=e)
    # heat sweeps and delta-k(T), bit for bit
    o = O.Oracle(O.make_cfg(CR, 40, 40, 20, 600.0, 600.0))
    rng = np.random.default_rng(5)
    T = o.init_temperature(48.0, 50.0, 46.5, 1)
    T = (T + rng.normal(0, 0.05, T.shape)).astype(np.float32)
    Q = (rng.random(T.shape) * 5e-9).astype(np.float32)
    got = S.heat_sweeps(CR, T, Q, 25.0, 7, 1, lx=600.0, ly=600.0)
    record("heat40x40x20", bits_equal(got, o.heat_sweeps(T, Q, 25.0, 7, 1)))
    D, NP, NS = S.dk_thermal(CR, T, lx=600.0, ly=600.0)
    record("dk40x40x20", bool(np.all(np.isfinite(D))))


def device_cases():
    """Paths that take device buffers (torch), check build only."""
    import torch
    n, nz = 32, 20
    inst = W.plain_instance(n, nz, 10.0, 2.84, 50.0)
    s = S.Solver(crystal=CR, nx=n, ny=n, nz=nz, lx=inst.lx, ly=inst.ly)
    r = s.grad_run(inst.power, inst.waist, inst.focal, inst.temp, checkpoints=4)
    record("grad_run32", all(np.isfinite(r[k]) for k in ("loss", "dT_total", "dfocal")))
    s.close()
    from shg_focused_gaussian_beams_gb300.solver import ThermalGradBatch
    tb = ThermalGradBatch(2, crystal=CR, nx=n, ny=n, nz=nz, lx=inst.lx, ly=inst.ly)
    tb.solve_temperature(0, 20.0, inst.waist, FOCAL, 50.0)
    tb.solve_temperature(1, 10.0, inst.waist, FOCAL, 50.0)
    pumps = tb.gaussian_pumps()
    g = tb.gradient(pumps, checkpoints=3)
    record("thgrad32", bool(torch.isfinite(torch.view_as_real(g["grad"])).all().item()))
    tb.close()
    cfg = S._cfg_from(CR, nx=n, ny=n, nz=nz)
    p = torch.zeros((n, n), dtype=torch.complex64, device="cuda") + 1.0
    po = torch.empty_like(p)
    so = torch.empty_like(p)
    eta = C.c_double()
    _lib.check(_lib.lib().shg_cwes_noalloc(C.byref(cfg), 50.0, p.data_ptr(), None, po.data_ptr(), so.data_ptr(),
                                           C.byref(eta), None), "shg_cwes_noalloc")
    record("noalloc32", np.isfinite(eta.value))


def error_cases():
    bad = _lib.default_config(nx=48, ny=48, nz=10)
    h = C.c_void_p()
    rc = _lib.lib().shg_create(C.byref(bad), C.byref(h))
    record("bad_grid", rc == 2)
    rc = _lib.lib().shg_create(None, C.byref(h))
    record("null_config", rc == 1)


def fullsize_cases():
    """The benchmarked workloads at their own sizes: the 512-solve sweep (its autotuner runs
    every candidate schedule of every class once), lone solves on the persistent grid at
    128x128x200 and 256x256x400, and a THERMAL 256x256x400 run (persistent THERMAL march,
    TMA heat sweeps, 1e-6 relative-residual rule)."""
    from shg_focused_gaussian_beams_gb300.parallel import rank_sweep
    sw = S.Sweep(rank_sweep(512, 2024, 0, 1, "weak"), crystal=CR)
    eta = sw.run()
    sw.close()
    record("sweep512", bool(np.all(np.isfinite(eta))))
    for n, nz in ((128, 200), (256, 400)):
        lone = S.Sweep([W.plain_instance(n, nz, 10.0, 2.84, 50.0)], crystal=CR)
        lone.set_schedule(n, resident="coop")
        record(f"coop{n}x{nz}", bool(np.isfinite(lone.run()[0])))
        lone.close()
    inst = W.config_thermal_256()
    s = S.Solver(crystal=CR, nx=inst.nx, ny=inst.ny, nz=inst.nz, lx=inst.lx, ly=inst.ly, thermal=True, bc=inst.bc)
    s.set_jacobi_rule(1e-6, 100, 1000)
    s.run(inst.power, inst.waist, inst.focal, inst.temp, inst.t_inf, inst.t1, inst.t2)
    record("thermal256x400", np.isfinite(s.efficiency()), counts=s.jacobi_counts())
    s.close()


def host_cases():
    """Host-only paths (no GPU needed): crystal indices bit-equal to the oracle's, argument
    errors, and the check-status call of a build without checks."""
    L = _lib.lib()
    v = C.c_float()
    same = True
    for T in np.linspace(10, 90, 17, dtype=np.float32):
        for lam in (1.064, float(np.float32(0.532))):
            _lib.check(L.shg_index(0, lam, float(T), C.byref(v)), "shg_index")
            same &= v.value == O.lib().oracle_n_f32(lam, float(T))
            _lib.check(L.shg_index(1, lam, float(T), C.byref(v)), "shg_index")
            same &= bool(np.isfinite(v.value))
    record("index", same)
    record("index_bad_crystal", L.shg_index(7, 1.064, 50.0, C.byref(v)) != 0)
    record("null_args", L.shg_config_init(None) == 1 and L.shg_batch_create(None, None, 0, None) == 1)
    h = C.c_void_p()
    grids = [dict(nx=48, ny=48), dict(nx=64, ny=32), dict(nx=512, ny=512), dict(nz=1)]
    record("unsupported_grids", all(L.shg_create(C.byref(_lib.default_config(**g)), C.byref(h)) in (1, 2)
                                    and len(L.shg_last_error()) > 0 for g in grids))
    cfg = _lib.default_config()
    record("empty_batches", L.shg_batch_create(C.byref(cfg), None, 0, C.byref(h)) == 1
           and L.shg_thgrad_create(C.byref(cfg), 0, C.byref(h)) == 2)
    record("bad_dft_and_handles", L.shg_dft2d_device(48, -1, None, None, None) == 1
           and L.shg_run(None, 1, 1, 1, 1, 1, 1, 1, 1, 0) == 1 and L.shg_destroy(None) == 0
           and L.shg_batch_destroy(None) == 0 and L.shg_heat_sweeps(None, None, None, 25.0, 1, 0) == 1)
    e, s_, val = C.c_int(), C.c_int(), C.c_longlong()
    record("check_status", L.shg_check_status(C.byref(e), C.byref(s_), C.byref(val)) == 0 and e.value == 0)


if MODE == "host":
    host_cases()
    print(json.dumps(report))
    sys.exit(0 if ok else 1)
if MODE == "fullsize":
    fullsize_cases()
    en, site, val = status()
    record("no_failed_check", en == 1 and site == 0, site=site, value=val)
    print(json.dumps(report))
    sys.exit(0 if ok else 1)
if MODE == "check":
    en, site, val = status()
    record("enabled", en == 1)
    _lib.check(_lib.lib().shg_check_selftest(424242), "shg_check_selftest")
    en, site, val = status()
    record("selftest_reported", site == 1 and val == 424242, site=site, value=val)
    record("cleared", status()[1] == 0)
plain_cases()
schedule_cases()
thermal_cases()
error_cases()
if MODE == "check":
    device_cases()
    en, site, val = status()
    record("no_failed_check", site == 0, site=site, value=val)
print(json.dumps(report))
sys.exit(0 if ok else 1)
