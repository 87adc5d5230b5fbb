"""SHG.sh-style sweep front-end (src/SHG.sh:31-101) on the GB300 library.

    python -m shg_focused_gaussian_beams_gb300.sweep --power 30 --waist 29 --t1 55.66 \
        [--t2 55.66] [--sols 1] [--stmp 1] [--thermal] [--bc 0|1] [--nx 64 --ny 64 --nz 200 ...] \
        [--foldersim Simulations] [--workdir .]

ARG1..ARG4 of SHG.sh become --power, --waist, --t1, --t2; each accepts several values
and every combination of power x waist x t1 is run (SHG.sh's nested loops, with the second
Peltier temperature equal to the first unless --t2 is given). SOLS / STMP keep their
meaning (save only the last slice / save the temperature tensor). Each point writes its
outputs (Files.h formats) into sPPLT_P_<P>_W_T1_<T1>_WAIST_<waist>/ together with the log
<folder>.txt, and the folders are gathered under --foldersim, as SHG.sh:73-101 does.

Plain points with SOLS=1 run together as one batch (one device schedule); THERMAL points
and SOLS=0 points run one solve at a time through Solver::run.
"""
from __future__ import annotations

import argparse
import itertools
import os
import shutil
import time

from . import workloads as W
from .files import save_matrix_complex


def _crystal(args):
    base = W.CRYSTAL_REFERENCE if args.crystal == "reference" else W.CRYSTAL_QPM50
    c = dict(base.__dict__)
    for k in ("lx", "ly", "lz", "deff", "lambda_qpm", "alpha_p", "alpha_s", "beta_s"):
        v = getattr(args, k)
        if v is not None:
            c[k] = v
    return c


def _folder(p, t1, w):
    return f"sPPLT_P_{p}_W_T1_{t1}_WAIST_{w}"


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--power", nargs="+", required=True, help="ARG1: pump power(s) [W]")
    ap.add_argument("--waist", nargs="+", required=True, help="ARG2: beam waist(s) [um]")
    ap.add_argument("--t1", nargs="+", required=True, help="ARG3: first Peltier / phase-matching temperature(s) [C]")
    ap.add_argument("--t2", nargs="+", default=None, help="ARG4: second Peltier temperature(s) [C] (default: = t1)")
    ap.add_argument("--sols", type=int, default=1)
    ap.add_argument("--stmp", type=int, default=0)
    ap.add_argument("--thermal", action="store_true")
    ap.add_argument("--bc", type=int, default=0)
    ap.add_argument("--nx", type=int, default=64)
    ap.add_argument("--ny", type=int, default=64)
    ap.add_argument("--nz", type=int, default=200)
    for k in ("lx", "ly", "lz", "deff", "lambda_qpm", "alpha_p", "alpha_s", "beta_s"):
        ap.add_argument("--" + k.replace("_", "-"), dest=k, type=float, default=None)
    ap.add_argument("--crystal", choices=["reference", "qpm50"], default="reference")
    ap.add_argument("--foldersim", default="Simulations")
    ap.add_argument("--workdir", default=".")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)

    from .solver import Solver, Sweep

    cr = _crystal(args)
    points = []
    for p, w, t1 in itertools.product(args.power, args.waist, args.t1):
        t2 = t1 if args.t2 is None else (args.t2[args.t1.index(t1)] if len(args.t2) == len(args.t1) else args.t2[0])
        points.append((p, w, t1, t2))
    work = os.path.abspath(args.workdir)
    sim = os.path.join(work, args.foldersim)
    os.makedirs(sim, exist_ok=True)
    focal = 0.5 * cr["lz"]
    t0 = time.time()
    logs = {}
    if not args.thermal and args.sols == 1:
        insts = [W.Instance(nx=args.nx, ny=args.ny, nz=args.nz, lx=cr["lx"], ly=cr["ly"], power=float(p),
                            waist=float(w), temp=float(t1), focal=focal) for p, w, t1, _ in points]
        sw = Sweep(insts, crystal=cr, device=args.device)
        eta = sw.run()
        pumps, shs = sw.fields()
        for k, (p, w, t1, t2) in enumerate(points):
            folder = os.path.join(sim, _folder(p, t1, w))
            os.makedirs(folder, exist_ok=True)
            save_matrix_complex(folder, "Pump_out", pumps[k])
            save_matrix_complex(folder, "Signal_out", shs[k])
            logs[folder] = (p, w, t1, t2, eta[k])
    else:
        for p, w, t1, t2 in points:
            folder = os.path.join(sim, _folder(p, t1, w))
            os.makedirs(folder, exist_ok=True)
            s = Solver(crystal=cr, nx=args.nx, ny=args.ny, nz=args.nz, lx=cr["lx"], ly=cr["ly"],
                       thermal=args.thermal, bc=args.bc, device=args.device)
            s.set_output_dir(folder)
            s.run(float(p), float(w), focal, float(t1), 25.0, float(t1), float(t2), bool(args.sols), bool(args.stmp))
            logs[folder] = (p, w, t1, t2, s.efficiency())
            s.close()
    for folder, (p, w, t1, t2, e) in logs.items():
        with open(folder + ".txt", "w") as fh:
            fh.write(f"Pump power =  {p} W\nBeam waist = {w} um\nPeltier 1 temperature =  {t1} C\n"
                     f"Peltier 2 temperature =  {t2} C\nConversion efficiency = {e:.9g}\n")
        shutil.move(folder + ".txt", os.path.join(folder, os.path.basename(folder) + ".txt"))
    print(f"{len(points)} points in {time.time() - t0:.3f} s -> {sim}")
    return logs


if __name__ == "__main__":
    main()
