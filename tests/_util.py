"""Shared helpers for the tests (not collected)."""
from __future__ import annotations

import math
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")

# Parity bar: output fields within relative L2 1e-4 and conversion
# efficiency within 1e-4 relative of the reference's FP32 build and of the FP64 run.
FIELD_RTOL = 1e-4
ETA_RTOL = 1e-4


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def eta(pump_in, sh_out, n_p, n_s):
    """P_SH(out)/P_pump(in) with P = 1/2 eps0 c n sum|A|^2 dx dy (dx dy cancel)."""
    return float(n_s) * float(np.sum(np.abs(np.asarray(sh_out, np.complex128)) ** 2)) / (
        float(n_p) * float(np.sum(np.abs(np.asarray(pump_in, np.complex128)) ** 2)))


def cfg_from_golden(g):
    import oracle as O
    return O.Cfg(int(g["cfg_nx"]), int(g["cfg_ny"]), int(g["cfg_nz"]), float(g["cfg_lx"]), float(g["cfg_ly"]),
                 float(g["cfg_lz"]), float(g["cfg_lp"]), float(g["cfg_deff"]), float(g["cfg_lambda_qpm"]),
                 float(g["cfg_alpha_p"]), float(g["cfg_alpha_s"]), float(g["cfg_beta_s"]), float(g["cfg_rho_p"]),
                 float(g["cfg_rho_s"]), float(g["cfg_kth"]), float(g["cfg_htc"]))


def crystal_from_golden(g):
    return {k[4:]: float(g[k]) for k in g if k.startswith("cfg_") and k not in
            ("cfg_nx", "cfg_ny", "cfg_nz", "cfg_thermal")}


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def smooth_noise(rng, n, cells=8):
    """Seeded complex Gaussian field smoothed over `cells` grid cells (FFT low-pass)."""
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    k = np.fft.fftfreq(n)
    g = np.exp(-0.5 * (k[:, None] ** 2 + k[None, :] ** 2) * (2 * math.pi * cells / 2.355) ** 2)
    b = np.fft.ifft2(np.fft.fft2(a) * g)
    return b / np.sqrt(np.mean(np.abs(b) ** 2))
