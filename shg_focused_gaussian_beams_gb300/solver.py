"""Python mirror of the reference's solver interface over the C ABI.

``Solver`` follows ``class Solver`` of Solver.h:120-153 (``run`` with the arguments of
Solver::run, Solver.h:279) plus the set-up calls of Efields (Efields.h:174-192) and the
plain CWES (Solver.h:245). ``Sweep`` runs many independent solves in one device schedule
(the SHG.sh one-process-per-point loop, SHG.sh:39-90). Host arrays are numpy complex64
of shape (NY, NX) in the reference layout IDX(x, y) = y*NX + x.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import asdict, is_dataclass

import numpy as np

from . import _lib
from ._lib import check, lib


def _cfg_from(crystal=None, **kw) -> _lib.Config:
    cfg = _lib.default_config()
    if crystal is not None:
        src = asdict(crystal) if is_dataclass(crystal) else dict(crystal)
        for k in ("lx", "ly", "lz", "lp", "deff", "lambda_qpm", "alpha_p", "alpha_s", "beta_s", "rho_p",
                  "rho_s", "kth", "htc"):
            if k in src:
                setattr(cfg, k, float(src[k]))
        if "crystal" in src:
            cfg.crystal = int(src["crystal"])
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def _pf(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _device_field(t, numel, what, device=None):
    """`t` if it is a contiguous complex64 CUDA tensor of `numel` elements (on CUDA device
    `device` when given: the handle's), else ValueError: the C ABI reads or writes exactly
    that many elements through the raw pointer, on the handle's device."""
    import torch
    if (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.complex64 and t.is_contiguous()
            and t.numel() == numel):
        if device is not None and t.device.index != device:
            raise ValueError(f"{what}: tensor on cuda:{t.device.index}, the handle's device is cuda:{device}")
        return t
    if isinstance(t, torch.Tensor):
        got = (f"a {t.dtype} {t.device.type} tensor of shape {tuple(t.shape)}"
               + ("" if t.is_contiguous() else ", not contiguous"))
    else:
        got = type(t).__name__
    raise ValueError(f"{what}: expected a contiguous complex64 CUDA tensor of {numel} elements, got {got}")


class Solver:
    """One solve on the device (Solver.h:120-153)."""

    def __init__(self, crystal=None, nx=64, ny=64, nz=200, lx=None, ly=None, thermal=False, bc=0, sh_seed=-1,
                 device=0):
        kw = dict(nx=nx, ny=ny, nz=nz, thermal=int(thermal), bc=bc, sh_seed=sh_seed, device=device)
        if lx is not None:
            kw["lx"] = float(lx)
        if ly is not None:
            kw["ly"] = float(ly)
        self.cfg = _cfg_from(crystal, **kw)
        h = C.c_void_p()
        check(lib().shg_create(C.byref(self.cfg), C.byref(h)), "shg_create")
        self._h = h
        self.nx, self.ny, self.nz = nx, ny, nz

    def close(self):
        if getattr(self, "_h", None):
            lib().shg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # Solver::run (Solver.h:279)
    def run(self, power, waist, focalpoint, temp, t_inf=25.0, t_peltier1=None, t_peltier2=None,
            save_only_last=True, save_temperature=False):
        t1 = temp if t_peltier1 is None else t_peltier1
        t2 = t1 if t_peltier2 is None else t_peltier2
        check(lib().shg_run(self._h, power, waist, focalpoint, temp, t_inf, t1, t2, int(save_only_last),
                            int(save_temperature)), "shg_run")
        return self

    def set_output_dir(self, path):
        """Directory for the reference's text outputs of run() (Files.h formats)."""
        check(lib().shg_set_output_dir(self._h, None if path is None else str(path).encode()), "shg_set_output_dir")

    # Efields::setInputPump (Efields.h:174)
    def set_input_pump(self, power, focalpoint, waist, tc):
        check(lib().shg_set_input_pump(self._h, power, focalpoint, waist, tc), "shg_set_input_pump")

    def set_input_fields(self, pump: np.ndarray, sh: np.ndarray | None = None):
        p = np.ascontiguousarray(pump, np.complex64)
        s = None if sh is None else np.ascontiguousarray(sh, np.complex64)
        for name, a in (("pump", p), ("sh", s)):
            if a is not None and a.size != self.nx * self.ny:
                raise ValueError(f"{name}: {a.size} points, expected NX*NY = {self.nx * self.ny}")
        check(lib().shg_set_input_fields(self._h, _pf(p), None if s is None else _pf(s)), "shg_set_input_fields")

    # Solver::CWES (Solver.h:245), plain
    def cwes(self, temp):
        check(lib().shg_cwes(self._h, temp), "shg_cwes")
        return self

    def cwes_device(self, temp, pump_in, sh_in=None, pump_out=None, sh_out=None, stream=None):
        """Device-pointer CWES on torch tensors (complex64, (NY, NX), contiguous)."""
        import torch
        n, dv = self.nx * self.ny, self.cfg.device
        _device_field(pump_in, n, "pump_in", dv)
        if sh_in is not None:
            _device_field(sh_in, n, "sh_in", dv)
        pump_out = torch.empty_like(pump_in) if pump_out is None else _device_field(pump_out, n, "pump_out", dv)
        sh_out = torch.empty_like(pump_in) if sh_out is None else _device_field(sh_out, n, "sh_out", dv)
        st = torch.cuda.current_stream(pump_in.device).cuda_stream if stream is None else stream
        check(lib().shg_cwes_device(self._h, temp, pump_in.data_ptr(),
                                    None if sh_in is None else sh_in.data_ptr(), pump_out.data_ptr(),
                                    sh_out.data_ptr(), st), "shg_cwes_device")
        return pump_out, sh_out

    def set_poling_period(self, lambda_qpm):
        check(lib().shg_set_poling_period(self._h, float(lambda_qpm)), "shg_set_poling_period")
        self.cfg.lambda_qpm = float(lambda_qpm)

    def grad(self, temp, pump_in, sh_in=None, checkpoints=20, stream=None):
        """Adjoint pass: L = SH output power and its gradients with respect to the input
        fields (torch complex64 CUDA tensors, dL/dRe + i dL/dIm), the oven temperature
        (fields held fixed) and the poling period. Returns a dict."""
        import torch
        _device_field(pump_in, self.nx * self.ny, "pump_in", self.cfg.device)
        if sh_in is not None:
            _device_field(sh_in, self.nx * self.ny, "sh_in", self.cfg.device)
        gp = torch.empty_like(pump_in)
        gs = torch.empty_like(pump_in)
        out = (C.c_double * 4)()
        st = torch.cuda.current_stream(pump_in.device).cuda_stream if stream is None else stream
        check(lib().shg_grad_device(self._h, temp, pump_in.data_ptr(), None if sh_in is None else sh_in.data_ptr(),
                                    int(checkpoints), gp.data_ptr(), gs.data_ptr(), out, st), "shg_grad_device")
        return {"loss": out[0], "grad_pump": gp, "grad_sh": gs, "dT": out[1], "dLambda": out[2], "ddk": out[3]}

    def grad_run(self, power, waist, focalpoint, temp, pump_factor=None, checkpoints=20, stream=None, device=None):
        """Adjoint pass of Solver::run's plain path (Gaussian pump of setPump at `temp`, times
        the optional complex64 CUDA tensor pump_factor; SH from zero): L = SH output power and
        its gradients with respect to the input pump field, the oven temperature (input field
        held fixed, and in total through the pump's index), the poling period, the focal
        point, the waist and the pump power. Returns a dict."""
        import torch
        dev = pump_factor.device if pump_factor is not None else torch.device(device or f"cuda:{self.cfg.device}")
        gp = torch.empty((self.ny, self.nx), dtype=torch.complex64, device=dev)
        out = (C.c_double * 8)()
        st = torch.cuda.current_stream(dev).cuda_stream if stream is None else stream
        # the factor's contiguous copy, if one is made, stays referenced through the call
        fac = None if pump_factor is None else _device_field(pump_factor.contiguous(), self.nx * self.ny,
                                                            "pump_factor", self.cfg.device)
        check(lib().shg_grad_run(self._h, power, waist, focalpoint, temp, None if fac is None else fac.data_ptr(),
                                 int(checkpoints), gp.data_ptr(), out, st), "shg_grad_run")
        return {"loss": out[0], "grad_pump": gp, "dT": out[1], "dLambda": out[2], "ddk": out[3], "dfocal": out[4],
                "dwaist": out[5], "dpower": out[6], "dT_total": out[7]}

    def fields(self):
        p = np.zeros((self.ny, self.nx), np.complex64)
        s = np.zeros((self.ny, self.nx), np.complex64)
        check(lib().shg_get_fields(self._h, _pf(p), _pf(s)), "shg_get_fields")
        return p, s

    def powers(self):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        check(lib().shg_get_powers(self._h, C.byref(a), C.byref(b), C.byref(c)), "shg_get_powers")
        return a.value, b.value, c.value

    def efficiency(self) -> float:
        e = C.c_double()
        check(lib().shg_efficiency(self._h, C.byref(e)), "shg_efficiency")
        return e.value

    # THERMAL results (Tfield::Tfinal and the Jacobi sweep counts of Solver.h:295-338)
    def temperature(self):
        T = np.zeros((self.nz, self.ny, self.nx), np.float32)
        check(lib().shg_get_temperature(self._h, _pf(T)), "shg_get_temperature")
        return T

    def set_jacobi_rule(self, rel_tol=0.0, check_every=100, max_sweeps=1000000):
        """rel_tol <= 0: the reference's stop rule; else ||dT||/||T|| < rel_tol."""
        check(lib().shg_set_jacobi_rule(self._h, float(rel_tol), int(check_every), int(max_sweeps)),
              "shg_set_jacobi_rule")

    def jacobi_residual(self) -> float:
        r = C.c_double()
        check(lib().shg_get_jacobi_residual(self._h, C.byref(r)), "shg_get_jacobi_residual")
        return r.value

    def jacobi_counts(self):
        c = (C.c_int * 5)()
        check(lib().shg_get_jacobi_counts(self._h, c), "shg_get_jacobi_counts")
        return list(c)


class Sweep:
    """Independent plain solves run together (one device schedule, CUDA graph)."""

    def __init__(self, instances, crystal=None, device=0):
        self.cfg = _cfg_from(crystal, device=device)
        n = len(instances)
        arr = (_lib.Instance * n)()
        for k, it in enumerate(instances):
            arr[k] = _lib.Instance(it.nx, it.ny, it.nz, it.lx, it.ly, it.power, it.waist, it.temp, it.focal)
        self._arr = arr
        self.instances = list(instances)
        b = C.c_void_p()
        check(lib().shg_batch_create(C.byref(self.cfg), arr, n, C.byref(b)), "shg_batch_create")
        self._b = b
        self.n = n

    def close(self):
        if getattr(self, "_b", None):
            lib().shg_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field_offsets(self):
        off = np.zeros(self.n + 1, np.int64)
        check(lib().shg_batch_field_offsets(self._b, off.ctypes.data_as(C.POINTER(C.c_longlong))),
              "shg_batch_field_offsets")
        return off

    def run(self, with_fields=False, eta_out=None, sh_out_all=None):
        """Run every solve. Returns efficiencies, and the SH output fields (list of (n, n)
        complex64 views into one contiguous buffer) when with_fields is set.
        eta_out / sh_out_all may be caller-owned (e.g. pinned) host buffers: eta_out a
        contiguous float64 array of one value per solve, sh_out_all a contiguous complex64
        array of every solve's points or the integer address of such a buffer."""
        eta = np.zeros(self.n, np.float64) if eta_out is None else eta_out
        if not (isinstance(eta, np.ndarray) and eta.dtype == np.float64 and eta.flags.c_contiguous
                and eta.size == self.n):
            raise ValueError(f"eta_out: expected a contiguous float64 array of {self.n} values")
        buf = sh_out_all
        if isinstance(buf, np.ndarray):
            total = int(self.field_offsets()[-1])
            if not (buf.dtype == np.complex64 and buf.flags.c_contiguous and buf.size == total):
                raise ValueError(f"sh_out_all: expected a contiguous complex64 array of {total} points")
        elif buf is not None and with_fields:
            raise ValueError("with_fields needs sh_out_all as an array (or None), not an address")
        if with_fields and buf is None:
            buf = np.zeros(int(self.field_offsets()[-1]), np.complex64)
        ptr = None if buf is None else C.c_void_p(buf.ctypes.data if isinstance(buf, np.ndarray) else buf)
        check(lib().shg_batch_run(self._b, eta.ctypes.data_as(C.POINTER(C.c_double)), ptr), "shg_batch_run")
        if not with_fields:
            return eta
        off = self.field_offsets()
        fields = [np.asarray(buf)[off[i]:off[i + 1]].reshape(it.ny, it.nx) for i, it in enumerate(self.instances)]
        return eta, fields

    def fields(self):
        """Output (pump, SH) fields of every solve after a run: two lists of (n, n) arrays."""
        off = self.field_offsets()
        p = np.zeros(int(off[-1]), np.complex64)
        s = np.zeros(int(off[-1]), np.complex64)
        check(lib().shg_batch_fields(self._b, C.c_void_p(p.ctypes.data), C.c_void_p(s.ctypes.data)),
              "shg_batch_fields")
        sh = [(it.ny, it.nx) for it in self.instances]
        return ([p[off[i]:off[i + 1]].reshape(sh[i]) for i in range(self.n)],
                [s[off[i]:off[i + 1]].reshape(sh[i]) for i in range(self.n)])

    def pump_fields_into(self, ptr):
        """Copy the output pump fields of every solve (contiguous, solve order) to a
        caller-owned host buffer at address ptr (e.g. pinned memory)."""
        check(lib().shg_batch_fields(self._b, C.c_void_p(ptr), None), "shg_batch_fields")

    def set_instances(self, instances):
        arr = (_lib.Instance * self.n)()
        for k, it in enumerate(instances):
            arr[k] = _lib.Instance(it.nx, it.ny, it.nz, it.lx, it.ly, it.power, it.waist, it.temp, it.focal)
        check(lib().shg_batch_set_instances(self._b, arr, self.n), "shg_batch_set_instances")
        self._arr = arr
        self.instances = list(instances)

    def profile(self):
        """Per-kernel totals of one instrumented run: {name: (launches, ms, algorithmic bytes)}."""
        stats = (_lib.KernelStat * 64)()
        n = C.c_int()
        check(lib().shg_batch_profile(self._b, stats, 64, C.byref(n)), "shg_batch_profile")
        return {stats[i].name.decode(): (stats[i].launches, stats[i].ms, stats[i].bytes) for i in range(n.value)}

    def run_async(self, stream):
        check(lib().shg_batch_run_async(self._b, stream), "shg_batch_run_async")

    def results(self):
        eta = np.zeros(self.n, np.float64)
        check(lib().shg_batch_results(self._b, eta.ctypes.data_as(C.POINTER(C.c_double))), "shg_batch_results")
        return eta

    def io_bytes(self):
        """(host->device bytes per re-parameterised run, device->host bytes of all SH fields)."""
        a, b = C.c_longlong(), C.c_longlong()
        check(lib().shg_batch_io_bytes(self._b, C.byref(a), C.byref(b)), "shg_batch_io_bytes")
        return a.value, b.value

    def autotune(self, stream=None):
        """Time the schedules of every grid-size class now (outside any capture)."""
        check(lib().shg_batch_autotune(self._b, stream), "shg_batch_autotune")

    def set_schedule(self, n, resident=True, cluster_size=1, ctas_per_sm=1, threads_per_line=None):
        """Fix the schedule of the grid-n class: streaming (resident=False), a resident variant
        (optionally with its line-FFT split), resident="coop", the persistent cooperative
        grid of a batch of one solve, or resident="cluster", one thread-block cluster per solve
        with one thread per point in the pointwise phase."""
        if resident in ("coop", "cluster"):
            mode = 2 if resident == "coop" else 3
            check(lib().shg_batch_set_schedule(self._b, int(n), mode, 0, 0), "shg_batch_set_schedule")
            return
        if resident and threads_per_line:
            check(lib().shg_batch_set_schedule_split(self._b, int(n), int(cluster_size), int(ctas_per_sm),
                                                     int(threads_per_line)), "shg_batch_set_schedule_split")
            return
        check(lib().shg_batch_set_schedule(self._b, int(n), int(bool(resident)), int(cluster_size),
                                           int(ctas_per_sm)), "shg_batch_set_schedule")

    def timeline(self, stream=None):
        """[(start_ms, end_ms)] per grid-size class of one concurrent run (diagnostic)."""
        out = (C.c_double * 64)()
        n = C.c_int()
        check(lib().shg_batch_timeline(self._b, out, 32, C.byref(n), stream), "shg_batch_timeline")
        return [(out[2 * k], out[2 * k + 1]) for k in range(n.value)]

    def schedule(self) -> str:
        """The schedule chosen per grid-size class, with the autotuner's trial times."""
        buf = C.create_string_buffer(8192)
        check(lib().shg_batch_schedule(self._b, buf, len(buf)), "shg_batch_schedule")
        return buf.value.decode()

    def launch_count(self) -> int:
        v = C.c_int()
        check(lib().shg_batch_launch_count(self._b, C.byref(v)), "shg_batch_launch_count")
        return v.value


class ThermalGradBatch:
    """Batched gradient of the THERMAL z-march with each solve's temperature field held
    fixed (``shg_thgrad_*``). Solve i's temperature comes from Solver::run (THERMAL) with a
    Gaussian pump (``solve_temperature``) or is given (``set_temperature``); its loss is the
    SH output power, differentiated with respect to its input pump. Pumps are torch
    complex64 CUDA tensors of shape (count, NY, NX)."""

    def __init__(self, count, crystal=None, nx=64, ny=64, nz=200, lx=None, ly=None, bc=0, device=0):
        kw = dict(nx=nx, ny=ny, nz=nz, thermal=1, bc=bc, device=device)
        if lx is not None:
            kw["lx"] = float(lx)
        if ly is not None:
            kw["ly"] = float(ly)
        self.cfg = _cfg_from(crystal, **kw)
        h = C.c_void_p()
        check(lib().shg_thgrad_create(C.byref(self.cfg), int(count), C.byref(h)), "shg_thgrad_create")
        self._h = h
        self.count, self.nx, self.ny, self.nz = int(count), nx, ny, nz
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            lib().shg_thgrad_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve_temperature(self, i, power, waist, focal, temp, t_inf=25.0, t_peltier1=None, t_peltier2=None):
        """Solver::run (THERMAL, Solver.h:287-340) for solve i; returns its Jacobi counts."""
        t1 = temp if t_peltier1 is None else t_peltier1
        t2 = t1 if t_peltier2 is None else t_peltier2
        c = (C.c_int * 5)()
        check(lib().shg_thgrad_solve_temperature(self._h, int(i), power, waist, focal, temp, t_inf, t1, t2, c),
              "shg_thgrad_solve_temperature")
        return list(c)

    def set_temperature(self, i, T: np.ndarray, power, waist, focal):
        Tn = np.ascontiguousarray(T, np.float32)
        if Tn.size != self.nx * self.ny * self.nz:
            raise ValueError(f"temperature field of {Tn.size} values, expected NX*NY*NZ = "
                             f"{self.nx * self.ny * self.nz}")
        check(lib().shg_thgrad_set_temperature(self._h, int(i), _pf(Tn), power, waist, focal),
              "shg_thgrad_set_temperature")

    def temperature(self, i):
        T = np.zeros((self.nz, self.ny, self.nx), np.float32)
        check(lib().shg_thgrad_get_temperature(self._h, int(i), _pf(T)), "shg_thgrad_get_temperature")
        return T

    def _stream(self, t, stream):
        import torch
        return torch.cuda.current_stream(t.device).cuda_stream if stream is None else stream

    def gaussian_pumps(self, stream=None):
        import torch
        out = torch.empty((self.count, self.ny, self.nx), dtype=torch.complex64, device=f"cuda:{self.device}")
        check(lib().shg_thgrad_gaussian_pumps(self._h, out.data_ptr(), self._stream(out, stream)),
              "shg_thgrad_gaussian_pumps")
        return out

    def _check_pump(self, pump, what="pump"):
        _device_field(pump, self.count * self.ny * self.nx, what, self.device)

    def forward(self, pump, with_fields=False, stream=None):
        """Returns dict(p_sh, p_in [W] as numpy arrays, and with_fields: pump_out, sh_out)."""
        import torch
        self._check_pump(pump)
        po = torch.empty_like(pump) if with_fields else None
        so = torch.empty_like(pump) if with_fields else None
        psh = np.zeros(self.count)
        pin = np.zeros(self.count)
        check(lib().shg_thgrad_forward(self._h, pump.data_ptr(), None if po is None else po.data_ptr(),
                                       None if so is None else so.data_ptr(), psh.ctypes.data_as(C.POINTER(C.c_double)),
                                       pin.ctypes.data_as(C.POINTER(C.c_double)), self._stream(pump, stream)),
              "shg_thgrad_forward")
        r = {"p_sh": psh, "p_in": pin}
        if with_fields:
            r.update(pump_out=po, sh_out=so)
        return r

    def gradient(self, pump, checkpoints=20, grad=None, stream=None):
        """Returns dict(p_sh, p_in, grad) with grad[i] = dP_SH,i / dA_in,i (dL/dRe + i dL/dIm)."""
        import torch
        self._check_pump(pump)
        if grad is not None:
            self._check_pump(grad, "grad")
        g = torch.empty_like(pump) if grad is None else grad
        psh = np.zeros(self.count)
        pin = np.zeros(self.count)
        check(lib().shg_thgrad_gradient(self._h, pump.data_ptr(), int(checkpoints), g.data_ptr(),
                                        psh.ctypes.data_as(C.POINTER(C.c_double)),
                                        pin.ctypes.data_as(C.POINTER(C.c_double)), self._stream(pump, stream)),
              "shg_thgrad_gradient")
        return {"p_sh": psh, "p_in": pin, "grad": g}

    def launch_count(self) -> int:
        return int(lib().shg_thgrad_launch_count(self._h))

    def device_bytes(self) -> float:
        return float(lib().shg_thgrad_device_bytes(self._h))


def _grid_cfg(crystal, nx, ny, nz, lx=None, ly=None):
    kw = dict(nx=nx, ny=ny, nz=nz)
    if lx is not None:
        kw["lx"] = float(lx)
    if ly is not None:
        kw["ly"] = float(ly)
    return _cfg_from(crystal, **kw)


def init_temperature(crystal, nx, ny, nz, temp, t1, t2, bc, lx=None, ly=None):
    """Tfield.h:31-110 on the device."""
    cfg = _grid_cfg(crystal, nx, ny, nz, lx, ly)
    T = np.zeros((nz, ny, nx), np.float32)
    check(lib().shg_init_temperature(C.byref(cfg), temp, t1, t2, bc, _pf(T)), "shg_init_temperature")
    return T


def heat_sweeps(crystal, T, Q, t_inf, nsweeps, bc, lx=None, ly=None):
    """`nsweeps` Jacobi sweeps of Tfield.h:113 (bc 0) / 224 (bc 1) on the device."""
    nz, ny, nx = T.shape
    if np.shape(Q) != T.shape:
        raise ValueError(f"heat source of shape {np.shape(Q)}, expected the temperature's {T.shape}")
    cfg = _grid_cfg(crystal, nx, ny, nz, lx, ly)
    Tn = np.ascontiguousarray(T, np.float32).copy()
    Qn = np.ascontiguousarray(Q, np.float32)
    check(lib().shg_heat_sweeps(C.byref(cfg), _pf(Tn), _pf(Qn), t_inf, nsweeps, bc), "shg_heat_sweeps")
    return Tn


def dk_thermal(crystal, T, lx=None, ly=None):
    """PhaseMatching.h:41-54 on the device: (delta-k, n_p, n_s) per voxel."""
    nz, ny, nx = T.shape
    cfg = _grid_cfg(crystal, nx, ny, nz, lx, ly)
    D, NP, NS = (np.zeros(T.shape, np.float32) for _ in range(3))
    check(lib().shg_dk_thermal(C.byref(cfg), _pf(np.ascontiguousarray(T, np.float32)), _pf(D), _pf(NP), _pf(NS)),
          "shg_dk_thermal")
    return D, NP, NS


def dft2d_device(x, sign: int, out=None, stream=None):
    """Unnormalised 2D DFT of a square (n, n) complex64 CUDA tensor (FFTW sign convention)."""
    import torch
    if x.dim() != 2 or x.shape[0] != x.shape[1]:
        raise ValueError(f"expected a square (n, n) tensor, got shape {tuple(x.shape)}")
    n = int(x.shape[0])
    _device_field(x, n * n, "x")
    out = torch.empty_like(x) if out is None else _device_field(out, n * n, "out")
    st = torch.cuda.current_stream(x.device).cuda_stream if stream is None else stream
    check(lib().shg_dft2d_device(n, sign, x.data_ptr(), out.data_ptr(), st), "shg_dft2d_device")
    return out
