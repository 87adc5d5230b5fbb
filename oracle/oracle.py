"""ORACLE — test infrastructure only.

ctypes access to the oracle restatement (``oracle/_build/liboracle.so``). Only tests/,
``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it, as the checker.
Arrays: numpy complex64/complex128 of shape (NY, NX) for fields, float32 (NZ, NY, NX)
for temperature tensors (reference layout IDX(x,y,z) = z*NX*NY + y*NX + x).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_f, _d, _i = C.c_float, C.c_double, C.c_int
_pf, _pd, _pi = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int)


class Cfg(C.Structure):
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i), ("lx", _f), ("ly", _f), ("lz", _f), ("lp", _f),
                ("deff", _f), ("lambda_qpm", _f), ("alpha_p", _f), ("alpha_s", _f), ("beta_s", _f),
                ("rho_p", _f), ("rho_s", _f), ("kth", _f), ("htc", _f), ("crystal", _i)]


class Inst(C.Structure):
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i), ("lx", _f), ("ly", _f), ("power", _f),
                ("waist", _f), ("temp", _f), ("focal", _f)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        import sys
        sys.path.insert(0, HERE)
        from build import build  # noqa: E402
        L = C.CDLL(build())
        L.oracle_n_f32.restype = _f
        L.oracle_n_f32.argtypes = [_f, _f]
        L.oracle_n_f64.restype = _d
        L.oracle_n_f64.argtypes = [_d, _d]
        L.oracle_index_f32.restype = _f
        L.oracle_index_f32.argtypes = [_i, _f, _f]
        L.oracle_index_f64.restype = _d
        L.oracle_index_f64.argtypes = [_i, _d, _d]
        P = C.POINTER(Cfg)
        L.oracle_set_pump_f32.argtypes = [P, _f, _f, _f, _f, _pf]
        L.oracle_set_pump_f64.argtypes = [P, _d, _d, _d, _d, _pd]
        L.oracle_propagators_f32.argtypes = [P, _f, _pf, _pf]
        L.oracle_propagators_f64.argtypes = [P, _d, _pd, _pd]
        L.oracle_dk_constant_f32.restype = _f
        L.oracle_dk_constant_f32.argtypes = [P, _f]
        L.oracle_dk_constant_f64.restype = _d
        L.oracle_dk_constant_f64.argtypes = [P, _d]
        L.oracle_diffraction_f32.argtypes = [P, _f, _pf, _pf]
        L.oracle_dft2d_f32.argtypes = [_i, _i, _i, _pf, _pf]
        L.oracle_dft2d_f64.argtypes = [_i, _i, _i, _pd, _pd]
        L.oracle_cwes_plain_f32.argtypes = [P, _pf, _pf, _f, _f, _pf, _pf, _pf, _pf]
        L.oracle_cwes_plain_f64.argtypes = [P, _pd, _pd, _d, _d, _pd, _pd, _pd, _pd]
        L.oracle_run_plain_f32.argtypes = [P, _f, _f, _f, _f, _i, _pf, _pf]
        L.oracle_init_temperature.argtypes = [P, _f, _f, _f, _i, _pf]
        L.oracle_heat_sweeps.argtypes = [P, _pf, _pf, _f, _i, _i]
        L.oracle_set_threads.argtypes = [_i]
        L.oracle_reduced_sum.restype = _f
        L.oracle_reduced_sum.argtypes = [P, _pf, _pf]
        L.oracle_dk_thermal.argtypes = [P, _pf, _pf]
        L.oracle_set_q.argtypes = [P, _pf, _pf, _pf, _i, _pf]
        L.oracle_cwes_thermal_f32.argtypes = [P, _pf, _pf, _pf, _pf, _f, _pf, _pf]
        L.oracle_cwes_thermal_f64.argtypes = [P, _pd, _pd, _pd, _pd, _d, _pd, _pd]
        L.oracle_thermal_run.restype = _i
        L.oracle_thermal_run.argtypes = [P, _f, _f, _f, _f, _f, _f, _f, _i, _i, _pf, _pf, _pf, _pi]
        L.oracle_sweep_plain.argtypes = [P, C.POINTER(Inst), _i, _i, _pd]
        L.oracle_power_f32.restype = _d
        L.oracle_power_f32.argtypes = [P, _pf, _f]
        _lib = L
    return _lib


def set_threads(threads: int):
    """Host threads of the restatement's heat sweeps (results do not depend on it)."""
    lib().oracle_set_threads(int(threads))


def _pF(a):
    return a.ctypes.data_as(_pf)


def _pD(a):
    return a.ctypes.data_as(_pd)


def make_cfg(crystal, nx, ny, nz, lx=None, ly=None) -> Cfg:
    """crystal: a workloads.Crystal (or dict with the same keys)."""
    g = crystal if isinstance(crystal, dict) else crystal.__dict__
    return Cfg(nx, ny, nz, g["lx"] if lx is None else lx, g["ly"] if ly is None else ly, g["lz"], g["lp"],
               g["deff"], g["lambda_qpm"], g["alpha_p"], g["alpha_s"], g["beta_s"], g["rho_p"], g["rho_s"],
               g["kth"], g["htc"], int(g.get("crystal", 0)))


class Oracle:
    """The restatement bound to one grid/crystal configuration."""

    def __init__(self, cfg: Cfg):
        self.cfg = cfg
        self.L = lib()
        self.nx, self.ny, self.nz = cfg.nx, cfg.ny, cfg.nz

    def _c2(self, dt=np.complex64):
        return np.zeros((self.ny, self.nx), dt)

    # Crystal.h:116 (or the PPLN fit for crystal 1)
    def n(self, L, T):
        return np.float32(self.L.oracle_index_f32(self.cfg.crystal, L, T))

    def n64(self, L, T):
        return float(self.L.oracle_index_f64(self.cfg.crystal, L, T))

    def set_pump(self, power, focal, waist, tc):
        a = self._c2()
        self.L.oracle_set_pump_f32(C.byref(self.cfg), power, focal, waist, tc, _pF(a))
        return a

    def set_pump64(self, power, focal, waist, tc):
        a = self._c2(np.complex128)
        self.L.oracle_set_pump_f64(C.byref(self.cfg), power, focal, waist, tc, _pD(a))
        return a

    def propagators(self, tc):
        hp, hs = self._c2(), self._c2()
        self.L.oracle_propagators_f32(C.byref(self.cfg), tc, _pF(hp), _pF(hs))
        return hp, hs

    def propagators64(self, tc):
        hp, hs = self._c2(np.complex128), self._c2(np.complex128)
        self.L.oracle_propagators_f64(C.byref(self.cfg), tc, _pD(hp), _pD(hs))
        return hp, hs

    def dk_constant(self, temp):
        return np.float32(self.L.oracle_dk_constant_f32(C.byref(self.cfg), temp))

    def dk_constant64(self, temp):
        return float(self.L.oracle_dk_constant_f64(C.byref(self.cfg), temp))

    def diffraction(self, pump, sh, tc):
        p = np.ascontiguousarray(pump, np.complex64).copy()
        s = np.ascontiguousarray(sh, np.complex64).copy()
        self.L.oracle_diffraction_f32(C.byref(self.cfg), tc, _pF(p), _pF(s))
        return p, s

    def cwes_plain(self, pump, sh, temp, dk=float("nan")):
        p = np.ascontiguousarray(pump, np.complex64)
        s = np.ascontiguousarray(sh, np.complex64)
        po, so, pe, se = self._c2(), self._c2(), self._c2(), self._c2()
        self.L.oracle_cwes_plain_f32(C.byref(self.cfg), _pF(p), _pF(s), temp, dk, _pF(po), _pF(so), _pF(pe),
                                     _pF(se))
        return po, so, pe, se

    def cwes_plain64(self, pump, sh, temp, dk=float("nan")):
        p = np.ascontiguousarray(pump, np.complex128)
        s = np.ascontiguousarray(sh, np.complex128)
        po, so, pe, se = (self._c2(np.complex128) for _ in range(4))
        self.L.oracle_cwes_plain_f64(C.byref(self.cfg), _pD(p), _pD(s), temp, dk, _pD(po), _pD(so), _pD(pe),
                                     _pD(se))
        return po, so, pe, se

    def run_plain(self, power, waist, focal, temp, sh_seed=-1):
        po, so = self._c2(), self._c2()
        self.L.oracle_run_plain_f32(C.byref(self.cfg), power, waist, focal, temp, sh_seed, _pF(po), _pF(so))
        return po, so

    def init_temperature(self, temp, t1, t2, bc):
        T = np.zeros((self.nz, self.ny, self.nx), np.float32)
        self.L.oracle_init_temperature(C.byref(self.cfg), temp, t1, t2, bc, _pF(T))
        return T

    def heat_sweeps(self, T, Q, t_inf, nsweeps, bc):
        Tn = np.ascontiguousarray(T, np.float32).copy()
        Qn = np.ascontiguousarray(Q, np.float32)
        self.L.oracle_heat_sweeps(C.byref(self.cfg), _pF(Tn), _pF(Qn), t_inf, nsweeps, bc)
        return Tn

    def reduced_sum(self, Tf, Ti):
        return np.float32(self.L.oracle_reduced_sum(C.byref(self.cfg), _pF(np.ascontiguousarray(Tf, np.float32)),
                                                    _pF(np.ascontiguousarray(Ti, np.float32))))

    def dk_thermal(self, T):
        D = np.zeros((self.nz, self.ny, self.nx), np.float32)
        self.L.oracle_dk_thermal(C.byref(self.cfg), _pF(np.ascontiguousarray(T, np.float32)), _pF(D))
        return D

    def set_q(self, Q, T, pump, sh, s):
        Qn = np.ascontiguousarray(Q, np.float32).copy()
        self.L.oracle_set_q(C.byref(self.cfg), _pF(np.ascontiguousarray(T, np.float32)),
                            _pF(np.ascontiguousarray(pump, np.complex64)),
                            _pF(np.ascontiguousarray(sh, np.complex64)), s, _pF(Qn))
        return Qn

    def cwes_thermal(self, T, pump, sh, tc, dk3=None):
        """THERMAL CWES with T held fixed (float); returns the fields at the top of slice NZ-1."""
        Tn = np.ascontiguousarray(T, np.float32)
        dk = None if dk3 is None else np.ascontiguousarray(dk3, np.float32)
        po, so = self._c2(), self._c2()
        self.L.oracle_cwes_thermal_f32(C.byref(self.cfg), _pF(Tn), _pF(dk) if dk is not None else None,
                                       _pF(np.ascontiguousarray(pump, np.complex64)),
                                       _pF(np.ascontiguousarray(sh, np.complex64)), tc, _pF(po), _pF(so))
        return po, so

    def cwes_thermal64(self, T, pump, sh, tc, dk3=None):
        """Same in double; dk3 (e.g. the float delta-k table) pins delta-k."""
        Tn = np.ascontiguousarray(T, np.float64)
        dk = None if dk3 is None else np.ascontiguousarray(dk3, np.float64)
        po, so = self._c2(np.complex128), self._c2(np.complex128)
        self.L.oracle_cwes_thermal_f64(C.byref(self.cfg), _pD(Tn), _pD(dk) if dk is not None else None,
                                       _pD(np.ascontiguousarray(pump, np.complex128)),
                                       _pD(np.ascontiguousarray(sh, np.complex128)), tc, _pD(po), _pD(so))
        return po, so

    def thermal_run(self, power, waist, focal, temp, t_inf, t1, t2, bc=0, sh_seed=-1):
        po, so = self._c2(), self._c2()
        T = np.zeros((self.nz, self.ny, self.nx), np.float32)
        counts = (C.c_int * 5)()
        outer = self.L.oracle_thermal_run(C.byref(self.cfg), power, waist, focal, temp, t_inf, t1, t2, bc,
                                          sh_seed, _pF(po), _pF(so), _pF(T), counts)
        return dict(pump=po, sh=so, T=T, counts=list(counts), outer=outer)

    def power(self, field, n_index):
        f = np.ascontiguousarray(field, np.complex64)
        return float(self.L.oracle_power_f32(C.byref(self.cfg), _pF(f), n_index))


def dft2d(a: np.ndarray, sign: int) -> np.ndarray:
    """FFTW-convention unnormalised 2D DFT of a (n0, n1) array (float32 or float64 complex)."""
    a = np.ascontiguousarray(a)
    out = np.empty_like(a)
    if a.dtype == np.complex64:
        lib().oracle_dft2d_f32(a.shape[0], a.shape[1], sign, _pF(a), _pF(out))
    else:
        a = a.astype(np.complex128)
        out = np.empty_like(a)
        lib().oracle_dft2d_f64(a.shape[0], a.shape[1], sign, _pD(a), _pD(out))
    return out


def sweep_plain(crystal_cfg: Cfg, instances, threads: int) -> np.ndarray:
    n = len(instances)
    arr = (Inst * n)()
    for k, it in enumerate(instances):
        arr[k] = Inst(it.nx, it.ny, it.nz, it.lx, it.ly, it.power, it.waist, it.temp, it.focal)
    eta = np.zeros(n, np.float64)
    lib().oracle_sweep_plain(C.byref(crystal_cfg), arr, n, threads, _pD(eta))
    return eta
