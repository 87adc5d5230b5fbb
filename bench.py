#!/usr/bin/env python
"""Headline benchmark: grid-pt*z-steps/s of the batched SSFM sweep (and solves/s).

Workload (default ``sweep``): 512 independent plain solves, seeded: pump power
log-U(1, 50) W, focusing xi U(0.5, 5), oven 50 C +- 2 K, grid N^2 with N in {64, 128, 256},
Nz in {100, 200, 400}, MgO:sPPLT crystal of the plain 128x128x200 workload, window 16 w0.
One step = one pass of every solve (set-up + z-march + efficiency). Units: a solve of an
N x N grid with Nz slices counts N*N*Nz grid-pt*z-steps (the reference's loop count,
Solver.h:249), for both arms.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sweep|plain128]

--impl ours (default): ``value`` = device-resident throughput (instance table already on
the GPU, CUDA events on the launching stream, K graph launches), ``e2e`` = the same
through the public C ABI with host buffers (instance parameters uploaded and efficiencies
plus all SH output fields read back every step), ``roofline`` from per-launch CUDA
events of an instrumented run, ``cpu_baseline`` = the oracle restatement of the
reference on a bounded sample on all host cores.
--impl reference: the reference's CPU algorithm (the oracle restatement; the reference's
own build needs sources absent on this machine) on all host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402

METRIC = "grid-pt·z-steps/s (batched SSFM sweep, 512 solves; solves/s alongside)"
UNIT = "grid-pt·z-steps/s"
FALLBACK_HBM_GBS = 6800.0


def pt_steps(insts):
    return sum(i.nx * i.ny * i.nz for i in insts)


def workload(name, rank=0, world=1):
    if name == "sweep":
        from shg_focused_gaussian_beams_gb300.parallel import rank_sweep
        insts = rank_sweep(512, 2024, rank, world, "weak")
        desc = {"workload": "sweep512: 512 plain solves, N in {64,128,256}, Nz in {100,200,400}, P log-U(1,50) W, "
                            "xi U(0.5,5), T 50+-2 C, window 16 w0",
                "solves": len(insts)}
    elif name == "rows256":
        # ncu-sized case: 64 solves of 256x256x100 (fields + propagators 200 MB > L2)
        insts = [W.plain_instance(256, 100, 10.0, 2.84, 50.0) for _ in range(64)]
        desc = {"workload": "64 plain solves 256x256x100 (profiling case)", "solves": len(insts)}
    elif name == "resident256":
        # ncu-sized case for the resident march: 38 solves of 256x256x100 (two per cluster slot)
        insts = [W.plain_instance(256, 100, 10.0, 2.84, 50.0) for _ in range(38)]
        desc = {"workload": "38 plain solves 256x256x100, resident cs16/2 schedule (profiling case)",
                "solves": len(insts)}
    elif name == "plain128":
        insts = [W.config_plain_128()]
        desc = {"workload": "plain 128x128x200, P=10 W, xi=2.84, 50 C, window 16 w0", "solves": 1,
                "l2": "single-solve latency case: the 0.5 MB of fields stay in L2 between steps, as in any "
                      "lone solve"}
    else:
        raise SystemExit(f"unknown workload {name}")
    desc["pt_steps_per_step"] = pt_steps(insts)
    return insts, desc


def heat_sweep_time(inst, nsweeps):
    """Mean time of one heat sweep (CUDA events on the launching stream) on device buffers."""
    import ctypes as C
    import torch
    from shg_focused_gaussian_beams_gb300 import _lib
    from shg_focused_gaussian_beams_gb300.solver import _cfg_from, init_temperature
    cfg = _cfg_from(W.CRYSTAL_QPM50, nx=inst.nx, ny=inst.ny, nz=inst.nz, lx=inst.lx, ly=inst.ly)
    T0 = init_temperature(W.CRYSTAL_QPM50, inst.nx, inst.ny, inst.nz, inst.temp, inst.temp, inst.temp, inst.bc,
                          lx=inst.lx, ly=inst.ly)
    Ta = torch.from_numpy(T0).cuda()
    Tb = Ta.clone()
    QK = torch.full_like(Ta, 1e-4)
    st = torch.cuda.current_stream()
    L = _lib.lib()
    _lib.check(L.shg_heat_sweeps_device(C.byref(cfg), Ta.data_ptr(), Tb.data_ptr(), QK.data_ptr(), 25.0, 4, inst.bc,
                                        st.cuda_stream), "shg_heat_sweeps_device")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    _lib.check(L.shg_heat_sweeps_device(C.byref(cfg), Ta.data_ptr(), Tb.data_ptr(), QK.data_ptr(), 25.0, nsweeps,
                                        inst.bc, st.cuda_stream), "shg_heat_sweeps_device")
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) * 1e-3 / nsweeps


def run_adjoint(args):
    """Adjoint 256x256x400 (P = 20 W, xi = 2.84, Gaussian pump times a seeded 5 % smooth
    perturbation, 20 checkpoints): time of the fused forward CWES and of the gradient pass
    (forward with checkpoints + reverse sweep) through the C ABI, CUDA events."""
    import torch
    from shg_focused_gaussian_beams_gb300.autograd import gaussian_pump
    from shg_focused_gaussian_beams_gb300.solver import Solver
    inst = W.plain_instance(256, 400, 20.0, 2.84, 50.0)
    g = torch.Generator().manual_seed(3)
    noise = torch.randn(256, 256, 2, generator=g, dtype=torch.float64)
    noise = torch.complex(noise[..., 0], noise[..., 1])
    k = torch.fft.fftfreq(256, dtype=torch.float64)
    lp = torch.exp(-0.5 * (k[:, None] ** 2 + k[None, :] ** 2) * (2 * 3.141592653589793 * 8 / 2.355) ** 2)
    noise = torch.fft.ifft2(torch.fft.fft2(noise) * lp)
    noise = noise / noise.abs().pow(2).mean().sqrt()
    pump = (gaussian_pump(256, 256, inst.lx, inst.ly, inst.power, inst.waist, inst.focal, inst.temp, device="cpu")
            * (1 + 0.05 * noise)).to(torch.complex64).cuda()
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=256, ny=256, nz=400, lx=inst.lx, ly=inst.ly)
    st = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 1)):
        s.cwes_device(inst.temp, pump)
        s.grad(inst.temp, pump, checkpoints=20)
    torch.cuda.synchronize()
    def timed(fn, reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    fwd = timed(lambda: s.cwes_device(inst.temp, pump), max(args.steps, 1))
    grd = timed(lambda: s.grad(inst.temp, pump, checkpoints=20), max(args.steps, 1))
    r = s.grad(inst.temp, pump, checkpoints=20)
    # every step stored (399 states of X_s, W_s, F_s: 1.2 GB), no replay
    s.grad(inst.temp, pump, checkpoints=399)
    torch.cuda.synchronize()
    grd_all = timed(lambda: s.grad(inst.temp, pump, checkpoints=399), max(args.steps, 1))
    r_all = s.grad(inst.temp, pump, checkpoints=399)
    print(json.dumps({"workload": "adjoint256: 256x256x400, P=20 W, xi=2.84",
                      "forward_ms": fwd, "gradient_ms_20_checkpoints": grd, "gradient_over_forward": grd / fwd,
                      "gradient_ms_store_all": grd_all, "store_all_over_forward": grd_all / fwd,
                      "loss_W": r["loss"], "dL_dT": r["dT"], "dL_dLambda": r["dLambda"],
                      "store_all_dT_rel_diff": abs(r_all["dT"] - r["dT"]) / abs(r["dT"])}), flush=True)


def run_thermal_adjoint(args, count=64, n=256, nz=400, design_steps=20):
    """Batched adjoint with THERMAL: 64 solves of 256x256x400 (P ~ U(5, 40) W, xi = 2.84,
    oven 50 C + U(-1, 1) K), Hermite-Gauss (m, n <= 3) admixtures |c| <= 0.2 on a Gaussian;
    each temperature field is solved once (Solver::run, THERMAL) and held fixed. Times the
    batched forward and gradient passes (CUDA events) and the 20-step design loop."""
    import torch
    from shg_focused_gaussian_beams_gb300 import inverse as I
    from shg_focused_gaussian_beams_gb300.solver import ThermalGradBatch
    insts = W.config_thermal_adjoint(count, n=n, nz=nz)
    i0 = insts[0]
    focal = float(np.float32(0.5 * W.CRYSTAL_QPM50.lz))
    tb = ThermalGradBatch(count, crystal=W.CRYSTAL_QPM50, nx=n, ny=n, nz=nz, lx=i0.lx, ly=i0.ly, bc=1)
    t0 = time.time()
    counts = [tb.solve_temperature(i, x.power, x.waist, focal, x.temp, 25.0, x.t1, x.t2) for i, x in enumerate(insts)]
    t_temp = time.time() - t0
    tcs = [float(tb.temperature(i)[0, n // 2, n // 2]) for i in range(count)]
    modes = torch.stack([I.hermite_gauss_modes(n, n, i0.lx, i0.ly, x.waist, focal, tc, mmax=3)[0]
                         for x, tc in zip(insts, tcs)])
    coef0 = I.seeded_admixtures(count, modes.shape[1], seed=77, cmax=0.2)
    power = torch.tensor([x.power for x in insts], dtype=torch.float64, device="cuda")
    pumps = I.pumps_from_coefficients(coef0.cuda(), modes, power).to(torch.complex64).contiguous()
    st = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 1)):
        tb.forward(pumps)
        tb.gradient(pumps, checkpoints=20)
    torch.cuda.synchronize()

    def timed(fn, reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    reps = max(args.steps, 1)
    fwd = timed(lambda: tb.forward(pumps), reps)
    n_fwd = tb.launch_count()
    grd = timed(lambda: tb.gradient(pumps, checkpoints=20), reps)
    n_grd = tb.launch_count()
    mem20 = tb.device_bytes()
    tb.gradient(pumps, checkpoints=nz - 1)
    grd_all = timed(lambda: tb.gradient(pumps, checkpoints=nz - 1), reps)
    mem_all = tb.device_bytes()
    t0 = time.time()
    _, hist = I.optimize_inputs(tb, coef0, modes, power, steps=design_steps, lr=0.05, checkpoints=nz - 1)
    torch.cuda.synchronize()
    t_design = time.time() - t0
    units = count * n * n * (nz - 1)
    print(json.dumps({
        "workload": f"thermal_adjoint: {count} solves {n}x{n}x{nz}, P~U(5,40) W, xi=2.84, oven 50+U(-1,1) C, "
                    "HG(m,n<=3) admixtures |c|<=0.2, T solved once then fixed",
        "temperature_solves_s": t_temp, "jacobi_counts_first": counts[0],
        "forward_ms": fwd, "forward_launches": n_fwd,
        "forward_grid_pt_steps_per_s": units / (fwd * 1e-3),
        "gradient_ms_20_checkpoints": grd, "gradient_launches": n_grd, "gradient_over_forward": grd / fwd,
        "gradient_ms_store_all": grd_all, "store_all_over_forward": grd_all / fwd,
        "device_gb_20_checkpoints": mem20 / 1e9, "device_gb_store_all": mem_all / 1e9,
        "design_loop_s": t_design, "design_steps": design_steps,
        "eta_mean_before": float(hist[0].mean()), "eta_mean_after": float(hist[-1].mean()),
        "eta_improved_solves": int((hist[-1] > hist[0]).sum()),
    }), flush=True)


def run_heat(args):
    """Heat sweeps alone on the 256x256x400 THERMAL grid: one sweep per launch and K = 2, 3,
    4 sweeps per launch (temporal blocking); algorithmic bytes 12 per voxel and sweep."""
    inst = W.config_thermal_256()
    vox = inst.nx * inst.ny * inst.nz
    peak, kind = measured_hbm()
    out = {"workload": "heat256: Jacobi sweeps on 256x256x400, oven-surrounded", "peak": peak, "peak_source": kind}
    for spec in args.heat_kinds.split(","):
        kind, _, zc = spec.partition(":")  # "tma:50" = TMA-staged sweep with 50-plane chunks
        os.environ["SHG_HEAT"] = kind
        if zc:
            os.environ["SHG_HEAT_ZC"] = zc
        for lv in args.heat_levels.split(","):
            os.environ["SHG_HEAT_TB"] = lv
            per = heat_sweep_time(inst, max(args.steps, 1) * 96)
            out[f"{spec}_levels_{lv}"] = {"ms_per_sweep": 1e3 * per, "GBps_algorithmic": 12.0 * vox / per / 1e9,
                                          "frac": 12.0 * vox / per / 1e9 / peak}
        os.environ.pop("SHG_HEAT_ZC", None)
    os.environ.pop("SHG_HEAT_TB")
    os.environ.pop("SHG_HEAT")
    print(json.dumps(out), flush=True)


def run_thermal(args):
    """THERMAL 256x256x400 (oven surrounded, seeded oven temperature): one step = one full
    Solver::run with -DTHERMAL semantics (Jacobi to the reference's stop rule, five outer
    iterations). Reports grid-pt*z-steps/s of the z-marches, Jacobi voxel-sweeps/s and the
    heat-sweep kernel's roofline from live CUDA events."""
    import torch
    from shg_focused_gaussian_beams_gb300.solver import Solver, heat_sweeps
    inst = W.config_thermal_256()
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=inst.nx, ny=inst.ny, nz=inst.nz, lx=inst.lx, ly=inst.ly, thermal=True,
               bc=inst.bc)
    times = []
    with Clocks(0) as clk:
        for k in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.run(inst.power, inst.waist, inst.focal, inst.temp, inst.t_inf, inst.t1, inst.t2)
            torch.cuda.synchronize()
            if k >= args.warmup:
                times.append(time.perf_counter() - t0)
    counts = s.jacobi_counts()
    outer = sum(1 for c in counts if c >= 0)
    sweeps = sum(c for c in counts if c >= 0)
    t = statistics.median(times)
    vox = inst.nx * inst.ny * inst.nz
    per_sweep = heat_sweep_time(inst, 400)
    peak, peak_kind = measured_hbm()
    ach = 12.0 * vox / per_sweep / 1e9
    line = {"metric": "THERMAL 256x256x400 solve: grid-pt·z-steps/s of the z-marches", "impl": "ours",
            "value": vox * outer / t, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "thermal256: 256x256x400, P=30 W, xi=2.84, 2000x1000 um cross-section, "
                                   "oven-surrounded faces at a seeded U(45,55) C", "t_oven": inst.temp},
            "jacobi_counts": counts, "voxel_sweeps_per_s": vox * sweeps / t,
            "roofline": {"bound": "hbm", "kernel": "k_heat_tma<1,4> (one Jacobi sweep: TMA plane ring, 4 rows per "
                                                   "consumer warp, 8-plane chunks)",
                         "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak, "peak_source": peak_kind, "ms_per_launch": 1e3 * per_sweep,
                         "algorithmic_bytes_per_launch": 12.0 * vox, "traffic": heat_traffic(vox),
                         "note": "CUDA events around 400 back-to-back sweeps on the launching stream"},
            "clocks": clk.summary(), "efficiency": s.efficiency()}
    # the workload's relative-residual stop rule (||dT|| / ||T|| < 1e-6, checked every 100 sweeps)
    s.set_jacobi_rule(1e-6, check_every=100)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.run(inst.power, inst.waist, inst.focal, inst.temp, inst.t_inf, inst.t1, inst.t2)
    torch.cuda.synchronize()
    line["relative_residual_mode"] = {"ms": 1e3 * (time.perf_counter() - t0), "jacobi_counts": s.jacobi_counts(),
                                      "last_relative_residual": s.jacobi_residual(), "efficiency": s.efficiency()}
    # CPU: the restatement's Jacobi sweep (the reference's loop) on this grid, one core
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, inst.nx, inst.ny, inst.nz, inst.lx, inst.ly))
    T0 = o.init_temperature(inst.temp, inst.t1, inst.t2, inst.bc)
    Q = np.full_like(T0, 1e-9)
    t0 = time.perf_counter()
    o.heat_sweeps(T0, Q, inst.t_inf, 3, inst.bc)
    cpu = 3 * vox / (time.perf_counter() - t0)
    line["cpu_baseline"] = {"value": cpu, "unit": "voxel-sweeps/s", "cores": 1, "kind": "port",
                            "sample": "3 Jacobi sweeps of the 256x256x400 grid (the oracle restatement of "
                                      "Tfield.h's sweep, single-threaded like the reference)"}
    line["gpu_over_cpu_voxel_sweeps"] = vox / per_sweep / cpu
    print(json.dumps(line), flush=True)


CPU_KIND = ("oracle restatement of the reference's z-march (FP32, the reference's operation order) with the "
            "radix-2 FFTW stand-in of oracle/dft_ref.h, not FFTW (no libfftw3f on the host)")


def sweep_classes(insts):
    """Stratification of a sweep by (N, Nz) class: {(n, nz): (count, first solve of the class)}."""
    out = {}
    for i in insts:
        c, first = out.get((i.nx, i.nz), (0, i))
        out[(i.nx, i.nz)] = (c + 1, first)
    return dict(sorted(out.items()))


def class_times(classes, copies):
    """Wall time of `copies` full-length solves of each class run at once on `copies` host
    threads (the SHG.sh one-process-per-point loop on that many cores): {(n, nz): seconds}."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cfg = O.make_cfg(W.CRYSTAL_QPM50, 64, 64, 100)
    out = {}
    for key, (_, inst) in classes.items():
        t0 = time.perf_counter()
        O.sweep_plain(cfg, [inst] * copies, threads=copies)
        out[key] = time.perf_counter() - t0
    return out


def stratified_rate(classes, per_class_s, cores):
    """Sweep rate on `cores` host cores from the class times: the 512 solves spread over the
    cores, so the sweep takes sum over classes of count x (time of one solve) / cores, with one
    solve's time taken as the wall time of `cores` concurrent solves of its class."""
    work = sum(c * i.nx * i.ny * i.nz for c, i in classes.values())
    sweep_s = sum(classes[k][0] * per_class_s[k] for k in classes) / cores
    return work / sweep_s, sweep_s, work


def oracle_rate(insts, cores):
    """cpu_baseline of the sweep: one full-length solve of each of the (N, Nz) classes, all
    classes at once on the host cores (bounded: the wall time is the 256x256x400 solve)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    classes = sweep_classes(insts)
    cfg = O.make_cfg(W.CRYSTAL_QPM50, 64, 64, 100)
    O.sweep_plain(cfg, [next(iter(classes.values()))[1]], threads=1)  # load / warm
    reps = [i for _, i in classes.values()]
    # each class's solve on its own thread, all at once; per-solve time from a timed pass of
    # each class alone would take longer, so each thread times its own solve
    import threading as th
    per = {}

    def one(key, inst):
        t0 = time.perf_counter()
        O.sweep_plain(cfg, [inst], threads=1)
        per[key] = time.perf_counter() - t0
    t0 = time.perf_counter()
    ts = [th.Thread(target=one, args=(k, i)) for k, (_, i) in classes.items()]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    wall = time.perf_counter() - t0
    value, sweep_s, _ = stratified_rate(classes, per, cores)
    sample = (f"one full-length solve of each of the {len(reps)} (N, Nz) classes of the sweep, all at once on "
              f"{len(reps)} of {cores} host threads ({wall:.1f} s wall); sweep time = sum over classes of count x "
              f"solve time / {cores} cores = {sweep_s:.1f} s; weights (N, Nz: count) "
              + ", ".join(f"{k[0]}x{k[1]}: {c}" for k, (c, _) in classes.items()))
    return value, sample


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.rows and time.time() - t0 < 3.0:  # sampler running before timing starts
                time.sleep(0.05)
            self.rows.clear()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel):
    """Measured DRAM traffic of `kernel` from the committed ncu summaries
    (profiles/ncu_traffic.json): a dict with bytes per solve or per grid point, or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def heat_traffic(vox):
    """DRAM bytes of one TMA-staged sweep over `vox` voxels from the committed ncu capture
    (bytes per voxel of a 256x256x400 launch), or None."""
    t = ncu_traffic("heat_tma<4>")
    return None if t is None else t["bytes_per_voxel"] * vox


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    from shg_focused_gaussian_beams_gb300.parallel import world_max
    return world_max(v) if world > 1 else v


def run_reference(args):
    """The reference's CPU algorithm on the sweep, stratified by (N, Nz) class: step k runs
    full-length solves of the classes assigned to it (every class at least once over the K
    steps), `cores` copies at once on `cores` host threads, the SHG.sh process-per-point loop.
    value = the sweep rate derived from the per-class times (stratified_rate)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    insts, desc = workload(args.workload)
    cores = os.cpu_count() or 1
    classes = sweep_classes(insts)
    keys = list(classes)
    steps = max(args.steps, 1)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cfg = O.make_cfg(W.CRYSTAL_QPM50, 64, 64, 100)
    smallest = min(keys, key=lambda k: k[0] * k[0] * k[1])
    for _ in range(args.warmup):
        O.sweep_plain(cfg, [classes[smallest][1]] * cores, threads=cores)
    per = {k: [] for k in keys}
    wall = []
    for k in range(steps):
        # classes of step k: round robin, so K >= 9 steps cover each class at least once and
        # fewer steps take several classes each
        if steps >= len(keys):
            mine = [keys[k % len(keys)]]
        else:
            mine = [keys[j] for j in range(len(keys)) if j % steps == k]
        t0 = time.perf_counter()
        for key, t in class_times({q: classes[q] for q in mine}, cores).items():
            per[key].append(t)
        wall.append(time.perf_counter() - t0)
    per_s = {k: statistics.median(v) for k, v in per.items() if v}
    missing = [k for k in keys if k not in per_s]
    if missing:  # cannot happen with the assignment above; measured here rather than guessed
        per_s.update(class_times({q: classes[q] for q in missing}, cores))
    value, sweep_s, work = stratified_rate(classes, per_s, cores)
    total = sum(wall)
    sample = (f"each step: full-length solves of its (N, Nz) classes, {cores} copies at once on {cores} host "
              f"threads; all {len(keys)} classes over the {steps} steps; sweep time on {cores} cores = sum over "
              f"classes of count x solve time / {cores} = {sweep_s:.1f} s for {len(insts)} solves; weights "
              "(N x Nz: count) " + ", ".join(f"{k[0]}x{k[1]}: {classes[k][0]}" for k in keys))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": desc | {"stratified": {f"{k[0]}x{k[1]}": {"count": classes[k][0],
                                                                 "solve_s": per_s[k]} for k in keys},
                              "sweep_s_on_host": sweep_s, "same_config": True},
            "solves_per_s": len(insts) / sweep_s,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample + "; " + CPU_KIND},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def per_instance_rate(sample, device):
    """Solves one at a time through the single-solve API (shg_run: graph launch, sync)."""
    from shg_focused_gaussian_beams_gb300.solver import Solver
    hs = [Solver(crystal=W.CRYSTAL_QPM50, nx=i.nx, ny=i.ny, nz=i.nz, lx=i.lx, ly=i.ly, device=device)
          for i in sample]
    for h, i in zip(hs, sample):
        h.run(i.power, i.waist, i.focal, i.temp)
    t0 = time.perf_counter()
    for h, i in zip(hs, sample):
        h.run(i.power, i.waist, i.focal, i.temp)
    dt = time.perf_counter() - t0
    for h in hs:
        h.close()
    return {"solves_per_s": len(sample) / dt, "pt_steps_per_s": pt_steps(sample) / dt, "sample_solves": len(sample),
            "note": "the first 64 solves of the same workload, one Solver::run each (single-solve graph, "
                    "synchronised), handles created and warmed outside the timed region"}


def run_ours(args):
    import torch
    from shg_focused_gaussian_beams_gb300.solver import Sweep

    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    insts, desc = workload(args.workload, rank, world)
    sw = Sweep(insts, crystal=W.CRYSTAL_QPM50, device=local)
    if args.workload == "resident256":
        sw.set_schedule(256, True, 16, 2)
    stream = torch.cuda.Stream()
    for _ in range(max(args.warmup, 3)):
        sw.run_async(stream.cuda_stream)
    stream.synchronize()
    launches = sw.launch_count()

    # device-resident timed region; warm-up runs again once the clock sampler is up, so the
    # GPU is at its working clocks (not ramping from idle) when timing starts
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for _ in range(max(args.warmup, 3)):
            sw.run_async(stream.cuda_stream)
        stream.synchronize()
        barrier(world)
        ev0.record(stream)
        for _ in range(args.steps):
            sw.run_async(stream.cuda_stream)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = allmax(world, ev0.elapsed_time(ev1))
    work = desc["pt_steps_per_step"]
    value = work * world * args.steps / (ms * 1e-3)
    solves_s = len(insts) * world * args.steps / (ms * 1e-3)
    eta = sw.results()

    # end to end through the C ABI: parameters in (pinned), efficiencies + the SH and pump
    # output fields of every solve out (pinned)
    off = sw.field_offsets()
    eta_h = torch.empty(len(insts), dtype=torch.float64, pin_memory=True)
    fld_h = torch.empty(int(off[-1]) * 2, dtype=torch.float32, pin_memory=True)
    pmp_h = torch.empty(int(off[-1]) * 2, dtype=torch.float32, pin_memory=True)
    eta_np = eta_h.numpy()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sw.set_instances(insts)
        sw.run(eta_out=eta_np, sh_out_all=fld_h.data_ptr())
        sw.pump_fields_into(pmp_h.data_ptr())
    torch.cuda.synchronize()
    e2e_s = allmax(world, time.perf_counter() - t0)
    h2d, d2h_fields = sw.io_bytes()
    e2e = {"value": work * world * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": len(insts) * 8 + 2 * d2h_fields,
           "solves_per_s": len(insts) * world * args.steps / e2e_s,
           "outputs": "efficiencies, SH and pump output fields of every solve"}

    # the plain per-instance GPU path on a sample of the same solves: one solve at a time
    # through Solver::run (handles created and warmed outside the timed region)
    per = per_instance_rate(insts[:64], local) if rank == 0 else None

    # roofline of the dominant kernel from an instrumented run (per-launch CUDA events)
    prof = sw.profile()
    dom = max(prof, key=lambda k: prof[k][1])
    n_l, ms_k, bytes_k = prof[dom]
    peak, peak_kind = measured_hbm()
    achieved = bytes_k / (ms_k * 1e-3) / 1e9
    tr = ncu_traffic(dom)
    traffic = None
    if tr and "bytes_per_solve" in tr and dom.startswith("resident<"):
        # the resident march moves each solve's fields in and out once (and reads its
        # propagators from L2): traffic scales with the solves of the launch, not the steps
        n_dom = int(dom[len("resident<"):-1])
        traffic = tr["bytes_per_solve"] * sum(1 for i in insts if i.nx == n_dom)
    elif tr and "bytes_per_point" in tr:
        traffic = tr["bytes_per_point"] * bytes_k / n_l / (32.0 if dom.startswith("rows") else 48.0)
    issue = None
    if tr and "thread_inst_per_pt_step" in tr:
        # the resident march keeps its fields on chip, so its bound is FP32 instruction issue:
        # thread-instructions per second (ncu count per pt.step x the launch's pt.steps from
        # its algorithmic bytes, 32 B per pt.step) against the issue peak of 4 schedulers x
        # 32 lanes per SM at the sampled SM clock
        props = torch.cuda.get_device_properties(local)
        pt_steps = bytes_k / n_l / 32.0
        inst_s = tr["thread_inst_per_pt_step"] * pt_steps / (ms_k / n_l * 1e-3)
        sm_mhz = clk.summary().get("sm_mhz") or 2070.0
        peak_inst = props.multi_processor_count * 128 * sm_mhz * 1e6
        issue = {"achieved": inst_s, "peak": peak_inst, "unit": "thread-instructions/s", "frac": inst_s / peak_inst,
                 "thread_inst_per_pt_step": tr["thread_inst_per_pt_step"], "source": tr.get("inst_source"),
                 "peak_note": f"{props.multi_processor_count} SMs x 128 lanes x {sm_mhz:.0f} MHz (nominal issue rate)"}
    fp32 = None
    if dom.startswith(("resident<", "cluster<", "coop<")):  # the whole march in one kernel
        # flops of the method per grid-pt.z-step: 4 2D FFTs at 5 N log2 N, 2 propagator
        # products, 2 RK4 calls (20 log2(N^2) + 456; sincos not counted), against the nominal
        # FP32 rate (no measured FP32 peak exists): SMs x 128 lanes x 2 flop x SM clock
        props = torch.cuda.get_device_properties(local)
        n_dom = int(dom[dom.index("<") + 1:-1])
        flop_pt = 20.0 * math.log2(n_dom * n_dom) + 456.0
        pt_steps = bytes_k / n_l / 32.0
        fl_s = flop_pt * pt_steps / (ms_k / n_l * 1e-3)
        sm_mhz = clk.summary().get("sm_mhz") or 2070.0
        peak_fl = props.multi_processor_count * 128 * 2 * sm_mhz * 1e6
        fp32 = {"achieved": fl_s / 1e12, "peak": peak_fl / 1e12, "unit": "TFLOP/s", "frac": fl_s / peak_fl,
                "flop_per_pt_step": flop_pt, "peak_note": "nominal FP32 rate at the sampled SM clock"}
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "launches": n_l, "issue": issue, "fp32": fp32,
            "ms_per_launch": ms_k / n_l, "algorithmic_bytes_per_launch": bytes_k / n_l,
            "traffic": traffic,
            "traffic_source": None if tr is None else tr.get("source"),
            "share_of_step": ms_k / sum(v[1] for v in prof.values()),
            "kernels": {k: {"launches": v[0], "ms": v[1], "GBps": v[2] / (v[1] * 1e-3) / 1e9} for k, v in prof.items()}}

    if rank == 0:
        cores = os.cpu_count() or 1
        cpu_value, cpu_sample_text = oracle_rate(insts, cores)
        metric = METRIC if args.workload == "sweep" else f"grid-pt·z-steps/s ({desc['workload']})"
        line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"l2": "inputs larger than L2 (fields + propagators of 512 solves ~0.7 GB resident)"} | desc | {
                                  "parallelism": f"dp{world} (independent solves per GPU)",
                                  "crystal": "MgO:sPPLT, L=30 mm, QPM at 50 C, d_eff 6.75 pm/V"},
                "solves_per_s": solves_s, "e2e": e2e, "gpu_launches": launches * args.steps,
                "roofline": roof, "clocks": clk.summary(),
                "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": cpu_sample_text + "; " + CPU_KIND},
                "eta_mean": float(np.mean(eta)),
                "per_instance_gpu": per,
                "batched_over_per_instance": {"solves_per_s": solves_s / world / per["solves_per_s"],
                                              "pt_steps_per_s": value / world / per["pt_steps_per_s"]},
                "schedule": sw.schedule(),
                "class_timeline_ms": sw.timeline()}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--heat-levels", default="1", help="heat256: sweeps per launch to time (1 = no blocking)")
    ap.add_argument("--heat-kinds", default="tma,ws4",
                    help="heat256: single-sweep kernels to time (tma, tma:<planes per block>, ws4, ws8, 25)")
    ap.add_argument("--workload", choices=["sweep", "plain128", "rows256", "thermal256", "heat256", "adjoint256", "thermal_adjoint",
                                              "resident256"],
                    default="sweep")
    args = ap.parse_args()
    if args.workload == "thermal256":
        run_thermal(args)
    elif args.workload == "heat256":
        run_heat(args)
    elif args.workload == "adjoint256":
        run_adjoint(args)
    elif args.workload == "thermal_adjoint":
        run_thermal_adjoint(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
