"""Crystal presets and the benchmark workloads (pure Python, no CUDA needed).

Units follow the reference (Crystal.h:19-21): micrometres, picoseconds, volts, watts.

* ``CRYSTAL_REFERENCE`` is the reference's compiled-in MgO:sPPLT crystal
  (Crystal.h:26-53), used by the stock ``SHG`` CLI.
* ``CRYSTAL_QPM50`` is the same crystal with the poling period set to quasi-phase-matching
  at a 50 C oven, d_eff = 6.75 pm/V and the absorption figures of the plain 128x128x200
  workload (alpha_p = 0.002 /cm, alpha_s = 0.04 /cm, beta_s = 1e-11 m/W).

``sellmeier_n`` reproduces the reference's Sellmeier routine bit for bit (float
arguments, double evaluation, float result; Crystal.h:116-132), which the workload
definitions need to place the poling period and the pump waist. ``crystal=1`` selects
periodically poled lithium niobate with the congruent-LiNbO3 Sellmeier fit of Jundt,
Opt. Lett. 22, 1553 (1997) (``ln_n``; the reference's README names an MgO:PPLN crystal,
whose index its code does not hold); ``CRYSTAL_PPLN_QPM50`` is the plain workload's
crystal with that index and its own poling period for phase matching at 50 C.
"""
from __future__ import annotations

import math
import random
from dataclasses import dataclass, field, asdict

import numpy as np

F32 = np.float32
LP_UM = 1.064          # pump wavelength, Crystal.h:26
LZ_UM = 30000.0        # crystal length, Crystal.h:33


def sellmeier_n(L: float, T: float) -> np.float32:
    """Extraordinary index of MgO:sPPLT (Bruner et al.), as Crystal.h:116-132 evaluates
    it: float coefficients, double pow/sqrt, result rounded to float."""
    L = F32(L)
    T = F32(T)
    A, B, C, D = F32(4.502483), F32(0.007294), F32(0.185087), F32(-0.02357)
    E, Fc, G, H = F32(0.073423), F32(0.199595), F32(0.001), F32(7.99724)
    tk = float(T) + 273.15
    tk2 = tk * tk
    b = F32(3.483933e-8 * tk2)
    c = F32(1.607839e-8 * tk2)
    L2 = float(L) * float(L)
    cc = float(F32(C + c))
    n2 = (float(A) + float(F32(B + b)) / (L2 - cc * cc) + float(E) / (L2 - float(Fc) * float(Fc))
          + float(G) / (L2 - float(H) * float(H)) + float(D) * L2)
    return F32(math.sqrt(n2))


def ln_n(L: float, T: float) -> np.float32:
    """Extraordinary index of congruent LiNbO3 (PPLN; Jundt, Opt. Lett. 22, 1553-1555
    (1997)): n^2 = a1 + b1 f + (a2 + b2 f)/(L^2 - (a3 + b3 f)^2) + (a4 + b4 f)/(L^2 - a5^2)
    - a6 L^2 with f = (T - 24.5)(T + 570.82); double, rounded to float."""
    a1, a2, a3, a4, a5, a6 = 5.35583, 0.100473, 0.20692, 100.0, 11.34927, 1.5334e-2
    b1, b2, b3, b4 = 4.629e-7, 3.862e-8, -0.89e-8, 2.657e-5
    t, L2 = float(F32(T)), float(F32(L)) ** 2
    f = (t - 24.5) * (t + 570.82)
    c3 = a3 + b3 * f
    n2 = a1 + b1 * f + (a2 + b2 * f) / (L2 - c3 * c3) + (a4 + b4 * f) / (L2 - a5 * a5) - a6 * L2
    return F32(math.sqrt(n2))


def index_n(L: float, T: float, crystal: int = 0) -> np.float32:
    """n(L, T) of the selected crystal: 0 MgO:sPPLT (the reference's), 1 PPLN."""
    return ln_n(L, T) if crystal == 1 else sellmeier_n(L, T)


def qpm_period(T: float, lp: float = LP_UM, crystal: int = 0) -> float:
    """Poling period that phase-matches 2*k_p = k_s at oven temperature T, rounded to
    float: Lambda = lp / (2 (n_s - n_p))."""
    n_p = float(index_n(lp, T, crystal))
    n_s = float(index_n(F32(0.5 * lp), T, crystal))
    return float(F32(lp / (2.0 * (n_s - n_p))))


def waist_for_xi(xi: float, T: float, lz: float = LZ_UM, lp: float = LP_UM, crystal: int = 0) -> float:
    """Pump waist radius giving focusing parameter xi = L / (2 z_R), z_R = pi n_p w0^2 / lp."""
    n_p = float(index_n(lp, T, crystal))
    zr = lz / (2.0 * xi)
    return float(F32(math.sqrt(zr * lp / (math.pi * n_p))))


@dataclass
class Crystal:
    name: str
    lx: float = 2000.0
    ly: float = 1000.0
    lz: float = LZ_UM
    lp: float = LP_UM
    deff: float = 11.00e-6
    lambda_qpm: float = 7.97
    alpha_p: float = 0.17e-6
    alpha_s: float = 1.57e-6
    beta_s: float = 5e-5
    rho_p: float = 0.0
    rho_s: float = 0.0
    kth: float = 8.4e-6
    htc: float = 10e-12
    crystal: int = 0                 # refractive index: 0 MgO:sPPLT (Crystal.h), 1 PPLN (LiNbO3)


CRYSTAL_REFERENCE = Crystal(name="MgO:sPPLT (reference defaults)")
PM_TEMP_C = 50.0
CRYSTAL_QPM50 = Crystal(name="MgO:sPPLT QPM@50C", deff=6.75e-6, lambda_qpm=qpm_period(PM_TEMP_C),
                        alpha_p=2e-7, alpha_s=4e-6, beta_s=1e-5)
CRYSTAL_PPLN_QPM50 = Crystal(name="PPLN QPM@50C", deff=6.75e-6, lambda_qpm=qpm_period(PM_TEMP_C, crystal=1),
                             alpha_p=2e-7, alpha_s=4e-6, beta_s=1e-5, crystal=1)


@dataclass
class Instance:
    """One solve: grid, window and run parameters (argument list of Solver::run)."""
    nx: int
    ny: int
    nz: int
    lx: float
    ly: float
    power: float
    waist: float
    temp: float
    focal: float = 0.5 * LZ_UM
    t_inf: float = 25.0
    t1: float | None = None
    t2: float | None = None
    thermal: bool = False
    bc: int = 0                      # 0 = open top (Tfield.h:113), 1 = oven surrounded (Tfield.h:224)

    def as_dict(self):
        return asdict(self)

    @property
    def pt_steps(self) -> int:
        return self.nx * self.ny * self.nz


def plain_instance(n: int, nz: int, power: float, xi: float, temp: float,
                   window_waists: float = 16.0) -> Instance:
    w0 = waist_for_xi(xi, temp)
    win = float(F32(window_waists * w0))
    return Instance(nx=n, ny=n, nz=nz, lx=win, ly=win, power=power, waist=w0, temp=temp)


def config_plain_128() -> Instance:
    """Plain method, 128x128 complex64, Nz = 200, P = 10 W, xi = 2.84, 50 C, window 16 w0."""
    return plain_instance(128, 200, 10.0, 2.84, PM_TEMP_C)


def config_thermal_256(seed: int = 1234, n: int = 256, nz: int = 400) -> Instance:
    """THERMAL: 256x256x400, P = 30 W, xi = 2.84, crystal cross-section 2000x1000 um,
    faces held at an oven temperature drawn from U(45, 55) C (oven-surrounded mode)."""
    rng = random.Random(seed)
    t_oven = float(F32(rng.uniform(45.0, 55.0)))
    w0 = waist_for_xi(2.84, PM_TEMP_C)
    return Instance(nx=n, ny=n, nz=nz, lx=2000.0, ly=1000.0, power=30.0, waist=w0, temp=t_oven,
                    t1=t_oven, t2=t_oven, thermal=True, bc=1)


def config_thermal_adjoint(count: int = 64, seed: int = 4242, n: int = 256, nz: int = 400) -> list[Instance]:
    """Batched THERMAL gradient workload: `count` solves of n x n x nz, pump power U(5, 40) W,
    xi = 2.84 (waist at 50 C), window 16 w0, oven-surrounded faces at 50 C + U(-1, 1) K;
    each solve's temperature field is solved once and then held fixed."""
    rng = random.Random(seed)
    w0 = waist_for_xi(2.84, PM_TEMP_C)
    win = float(F32(16.0 * w0))
    out = []
    for _ in range(count):
        p = float(F32(rng.uniform(5.0, 40.0)))
        t = float(F32(PM_TEMP_C + rng.uniform(-1.0, 1.0)))
        out.append(Instance(nx=n, ny=n, nz=nz, lx=win, ly=win, power=p, waist=w0, temp=t, t1=t, t2=t,
                            thermal=True, bc=1))
    return out


def config_sweep(count: int = 512, seed: int = 2024) -> list[Instance]:
    """Batched sweep: per instance P log-U(1, 50) W, xi U(0.5, 5), T = 50 C + U(-2, 2) K,
    N in {64, 128, 256}, Nz in {100, 200, 400}; window 16 w0."""
    rng = random.Random(seed)
    out = []
    for _ in range(count):
        p = float(F32(math.exp(rng.uniform(math.log(1.0), math.log(50.0)))))
        xi = rng.uniform(0.5, 5.0)
        t = float(F32(PM_TEMP_C + rng.uniform(-2.0, 2.0)))
        n = rng.choice([64, 128, 256])
        nz = rng.choice([100, 200, 400])
        out.append(plain_instance(n, nz, p, xi, t))
    return out


def crystal_dict(c: Crystal) -> dict:
    return asdict(c)
