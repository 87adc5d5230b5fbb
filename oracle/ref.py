"""ORACLE — test infrastructure only.

ctypes access to the reference build (``oracle/_ref/libshg_ref_<tag>.so``, made by
``build_ref.py`` from the reference's own headers). Every function here calls the
reference's code; arrays are numpy complex64 in the reference layout
IDX(x, y, z) = z*NX*NY + y*NX + x (Common.h:27-29), i.e. shape (NZ, NY, NX) / (NY, NX).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_f = C.c_float
_pf = C.POINTER(C.c_float)
_pi = C.POINTER(C.c_int)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_pf)


def lib_path(tag: str) -> str:
    return os.path.join(REF_DIR, f"libshg_ref_{tag}.so")


def have(tag: str) -> bool:
    return os.path.isfile(lib_path(tag))


class RefBuild:
    """One compiled configuration of the reference."""

    def __init__(self, tag: str):
        self.tag = tag
        self.lib = L = C.CDLL(lib_path(tag))
        L.ref_n.restype = _f
        L.ref_n.argtypes = [_f, _f]
        L.ref_dk_constant.restype = _f
        L.ref_dk_constant.argtypes = [_f]
        L.ref_reduced_sum.restype = _f
        L.ref_set_pump.argtypes = [_pf, _f, _f, _f, _f]
        L.ref_propagators.argtypes = [_pf, _pf, _f]
        L.ref_diffraction.argtypes = [_pf, _pf, _f]
        L.ref_cwes_plain.argtypes = [_pf, _pf, _f, _pf, _pf, _pf, _pf]
        L.ref_init_temperature.argtypes = [_pf, _f, _f, _f, C.c_int]
        L.ref_heat_sweeps.argtypes = [_pf, _pf, _f, C.c_int, C.c_int]
        L.ref_dk_thermal.argtypes = [_pf, _pf]
        L.ref_set_q.argtypes = [_pf, _pf, _pf, _pf, C.c_int]
        L.ref_noise.argtypes = [_pf, C.c_uint]
        L.ref_thermal_run.restype = C.c_int
        L.ref_thermal_run.argtypes = [_f, _f, _f, _f, _f, _f, _f, C.c_int, C.c_int, _pf, _pf, _pf, _pi]
        nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
        L.ref_grid(C.byref(nx), C.byref(ny), C.byref(nz))
        self.nx, self.ny, self.nz = nx.value, ny.value, nz.value
        consts = np.zeros(12, np.float32)
        L.ref_constants(_ptr(consts))
        (self.dx, self.dy, self.dz, self.dQ, self.deff, self.lambda_qpm, self.alpha_p,
         self.alpha_s, self.beta_s, self.lx, self.ly, self.lz) = [np.float32(v) for v in consts]
        self.thermal = bool(L.ref_is_thermal())

    # -- helpers
    def _c2(self):
        return np.zeros((self.ny, self.nx), np.complex64)

    def _r3(self):
        return np.zeros((self.nz, self.ny, self.nx), np.float32)

    # -- wrappers (reference file:line in ref_driver.cpp)
    def n(self, L, T):
        return np.float32(self.lib.ref_n(L, T))

    def set_pump(self, power, focal, waist, tc):
        a = self._c2()
        self.lib.ref_set_pump(_ptr(a), power, focal, waist, tc)
        return a

    def noise(self, seed):
        a = self._c2()
        self.lib.ref_noise(_ptr(a), seed)
        return a

    def propagators(self, tc):
        hp, hs = self._c2(), self._c2()
        self.lib.ref_propagators(_ptr(hp), _ptr(hs), tc)
        return hp, hs

    def dk_constant(self, temp):
        return np.float32(self.lib.ref_dk_constant(temp))

    def diffraction(self, pump, sh, tc):
        p = np.ascontiguousarray(pump, np.complex64).copy()
        s = np.ascontiguousarray(sh, np.complex64).copy()
        self.lib.ref_diffraction(_ptr(p), _ptr(s), tc)
        return p, s

    def cwes_plain(self, pump, sh, temp):
        p = np.ascontiguousarray(pump, np.complex64)
        s = np.ascontiguousarray(sh, np.complex64)
        po, so, pe, se = self._c2(), self._c2(), self._c2(), self._c2()
        self.lib.ref_cwes_plain(_ptr(p), _ptr(s), temp, _ptr(po), _ptr(so), _ptr(pe), _ptr(se))
        return po, so, pe, se

    def init_temperature(self, temp, t1, t2, bc):
        T = self._r3()
        self.lib.ref_init_temperature(_ptr(T), temp, t1, t2, bc)
        return T

    def heat_sweeps(self, T, Q, t_inf, nsweeps, bc):
        Tn = np.ascontiguousarray(T, np.float32).copy()
        Qn = np.ascontiguousarray(Q, np.float32)
        self.lib.ref_heat_sweeps(_ptr(Tn), _ptr(Qn), t_inf, nsweeps, bc)
        return Tn

    def reduced_sum(self, Tf, Ti):
        Tf = np.ascontiguousarray(Tf, np.float32)
        Ti = np.ascontiguousarray(Ti, np.float32)
        return np.float32(self.lib.ref_reduced_sum(_ptr(Tf), _ptr(Ti)))

    def dk_thermal(self, T):
        T = np.ascontiguousarray(T, np.float32)
        D = self._r3()
        self.lib.ref_dk_thermal(_ptr(D), _ptr(T))
        return D

    def set_q(self, Q, T, pump, sh, s):
        Qn = np.ascontiguousarray(Q, np.float32).copy()
        self.lib.ref_set_q(_ptr(Qn), _ptr(np.ascontiguousarray(T, np.float32)),
                           _ptr(np.ascontiguousarray(pump, np.complex64)),
                           _ptr(np.ascontiguousarray(sh, np.complex64)), s)
        return Qn

    def thermal_run(self, power, waist, focal, temp, t_inf, t1, t2, bc=0, sh_seed=-1):
        po, so, T = self._c2(), self._c2(), self._r3()
        counts = (C.c_int * 5)()
        outer = self.lib.ref_thermal_run(power, waist, focal, temp, t_inf, t1, t2, bc, sh_seed,
                                         _ptr(po), _ptr(so), _ptr(T), counts)
        return dict(pump=po, sh=so, T=T, counts=list(counts), outer=outer)
