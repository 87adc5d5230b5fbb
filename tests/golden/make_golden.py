"""Generates the committed golden fixtures from the reference's own build.

Runs the reference (alfredos84/SHG_Focused_Gaussian_Beams, compiled in place by
oracle/build_ref.py into oracle/_ref/) on small configurations and stores its outputs as
.npz files beside this script. Needs the reference sources (development container only);
the fixtures then travel with the repository.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import build_ref  # noqa: E402
from configs import REF_BUILDS  # noqa: E402
from ref import RefBuild  # noqa: E402

from shg_focused_gaussian_beams_gb300.workloads import waist_for_xi  # noqa: E402


def _read_dat_complex(d, name, ny, nx):
    re = np.loadtxt(os.path.join(d, name + "_r.dat"), dtype=np.float64).reshape(ny, nx)
    im = np.loadtxt(os.path.join(d, name + "_i.dat"), dtype=np.float64).reshape(ny, nx)
    return (re.astype(np.float32) + 1j * im.astype(np.float32)).astype(np.complex64)


def crystal_meta(tag):
    c = REF_BUILDS[tag]
    out = {}
    for k, v in c.items():
        if k in ("name", "thermal"):
            continue
        out["cfg_" + k] = np.float64(v) if isinstance(v, float) else np.int64(v)
    out["cfg_thermal"] = np.int64(bool(c.get("thermal")))
    return out


def plain_case(tag, power, waist, temp, name):
    r = RefBuild(tag)
    focal = np.float32(0.5 * r.lz)
    pump = r.set_pump(power, focal, waist, temp)
    hp, hs = r.propagators(temp)
    zero = np.zeros_like(pump)
    po, so, pe, se = r.cwes_plain(pump, zero, temp)
    out = dict(pump_in=pump, pump_out=po, sh_out=so, dk=r.dk_constant(temp), n_p=r.n(1.064, temp),
               n_s=r.n(np.float32(0.532), temp), power=np.float32(power), waist=np.float32(waist),
               temp=np.float32(temp), focal=focal, dx=r.dx, dy=r.dy, dz=r.dz, **crystal_meta(tag))
    if r.nx <= 64:
        out["hp"] = hp
        out["hs"] = hs
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name, "eta-ish", float(np.sum(np.abs(so) ** 2) / np.sum(np.abs(pump) ** 2)))


def cli_case(tag, args, name):
    """SHG.cpp main exactly as shipped (clock-seeded SH noise), outputs read from .dat."""
    exe = os.path.join(build_ref.OUT, f"shg_ref_{tag}")
    r = RefBuild(tag)
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([exe] + [str(a) for a in args], cwd=d, check=True, stdout=subprocess.DEVNULL)
        po = _read_dat_complex(d, "Pump_out", r.ny, r.nx)
        so = _read_dat_complex(d, "Signal_out", r.ny, r.nx)
        with open(os.path.join(d, "Signal_out_r.dat")) as fh:  # the reference's own text, first rows
            head = [fh.readline() for _ in range(3)]
        with open(os.path.join(HERE, "stock_cli_signal_head.txt"), "w") as fh:
            fh.write("".join(head))
    np.savez_compressed(os.path.join(HERE, name), pump_out=po, sh_out=so, args=np.array(args, np.float64),
                        **crystal_meta(tag))
    print("wrote", name)


def dft_case(name):
    """The FFTW-API stand-in on a seeded field (both directions)."""
    import ctypes as C
    rng = np.random.default_rng(7)
    r = RefBuild("c0_small")
    a = (rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))).astype(np.complex64)
    # forward / backward through the reference's diffraction with unit propagator is not
    # exposed, so the fixture records the stand-in's transform of `a` via dft_ref in float.
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # noqa: E402
    np.savez_compressed(os.path.join(HERE, name), a=a, fwd=O.dft2d(a, -1), bwd=O.dft2d(a, +1))
    del r, C
    print("wrote", name)


def thermal_case(tag, power, waist, temp, t1, t2, bc, name):
    r = RefBuild(tag)
    res = r.thermal_run(power, waist, np.float32(0.5 * r.lz), temp, 25.0, t1, t2, bc=bc)
    rng = np.random.default_rng(11)
    T0 = r.init_temperature(temp, t1, t2, bc)
    Q = (rng.random(T0.shape) * 2e-10).astype(np.float32)
    T37 = r.heat_sweeps(T0, Q, 25.0, 37, bc)
    np.savez_compressed(os.path.join(HERE, name), pump_out=res["pump"], sh_out=res["sh"], T=res["T"],
                        counts=np.array(res["counts"]), outer=res["outer"], power=np.float32(power),
                        waist=np.float32(waist), temp=np.float32(temp), t1=np.float32(t1), t2=np.float32(t2),
                        bc=bc, T0=T0, Q=Q, T37=T37, dk_T=r.dk_thermal(res["T"]), **crystal_meta(tag))
    print("wrote", name, res["counts"])


def main():
    if not build_ref.available():
        print("reference sources not present; fixtures are committed already")
        return
    build_ref.build()
    w0 = waist_for_xi(2.84, 50.0)
    # SHG.sh:31-34 arguments on the stock build (64x64x200, 2000x1000 um, its crystal)
    plain_case("stock", 30.0, 29.0, 55.66, "stock_plain.npz")
    cli_case("stock", [30, 29, 55.66, 55.66, 1, 0], "stock_cli.npz")
    plain_case("c0_small", 10.0, w0, 50.0, "c0_small.npz")
    plain_case("c0", 10.0, w0, 50.0, "c0_128x200.npz")
    plain_case("walkoff", 10.0, w0, 50.0, "walkoff.npz")
    dft_case("dft64.npz")
    thermal_case("th_small", 30.0, w0, 50.0, 50.0, 50.0, 0, "thermal_topopen.npz")
    thermal_case("th_small", 30.0, w0, 52.0, 52.0, 52.0, 1, "thermal_oven.npz")


if __name__ == "__main__":
    main()
