"""Failure paths of the device API, made on the host (GB300 only; no GPU fault, trap or hang).

* Non-finite inputs: a NaN or infinite input field gives SHG_ERR_NONFINITE from the
  efficiency, and a solve with a NaN parameter makes the batch report SHG_ERR_NONFINITE
  while every other solve's efficiency is still stored.
* Device memory: a batch whose buffers exceed the free device memory is refused on the host
  with SHG_ERR_NOMEM before any allocation, and the process carries on.
* Bounded waits: with the TMA heat sweep's producer starved (SHG_HEAT_TMA_STARVE=1, every
  consumer wait runs out after its poll limit), a THERMAL run under the reference's stop rule
  and under the relative-residual rule ends at its first residual check with the error, and
  the device-buffer sweep call reports it through its own error word; runs afterwards are
  exact again.
"""
import time

import numpy as np
import pytest

import oracle as O
from _util import bits_equal

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import solver as S  # noqa: E402
from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402
from shg_focused_gaussian_beams_gb300._lib import ShgError  # noqa: E402


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_nonfinite_input_field(bad):
    inst = W.plain_instance(32, 12, 10.0, 2.84, 50.0)
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, 32, 32, 12, inst.lx, inst.ly))
    pump = o.set_pump(inst.power, inst.focal, inst.waist, inst.temp)
    pump[16, 16] = np.complex64(complex(bad, 0.0))
    s = S.Solver(crystal=W.CRYSTAL_QPM50, nx=32, ny=32, nz=12, lx=inst.lx, ly=inst.ly)
    s.set_input_fields(pump)
    s.cwes(inst.temp)
    with pytest.raises(ShgError, match="NONFINITE"):
        s.efficiency()
    # the handle stays usable
    s.set_input_fields(o.set_pump(inst.power, inst.focal, inst.waist, inst.temp))
    s.cwes(inst.temp)
    assert np.isfinite(s.efficiency())


def test_batch_with_a_nan_parameter_reports_nonfinite():
    insts = [W.plain_instance(32, 12, p, 2.84, 50.0) for p in (5.0, 10.0, 20.0)]
    insts[1] = W.Instance(**{**insts[1].as_dict(), "power": float("nan")})
    sw = S.Sweep(insts, crystal=W.CRYSTAL_QPM50)
    eta = np.zeros(3)
    with pytest.raises(ShgError, match="NONFINITE.*solve 1"):
        sw.run(eta_out=eta)
    assert np.isnan(eta[1]) and np.isfinite(eta[0]) and np.isfinite(eta[2])
    sw.close()


def test_batch_past_free_memory_is_refused_on_the_host():
    free, _ = torch.cuda.mem_get_info()
    per_solve = 48 * 256 * 256  # six complex64 fields of 256 x 256
    count = int(free // per_solve) + 64
    inst = W.plain_instance(256, 100, 10.0, 2.84, 50.0)
    t0 = time.time()
    with pytest.raises(ShgError, match="NOMEM"):
        S.Sweep([inst] * count, crystal=W.CRYSTAL_QPM50)
    assert time.time() - t0 < 60
    # nothing was allocated and the device is fine
    sw = S.Sweep([inst], crystal=W.CRYSTAL_QPM50)
    assert np.isfinite(sw.run()[0])
    sw.close()


@pytest.mark.parametrize("rule", ["reference", "relative"])
def test_starved_heat_pipeline_ends_the_jacobi_solve_promptly(rule, monkeypatch):
    monkeypatch.setenv("SHG_HEAT", "tma")
    monkeypatch.setenv("SHG_HEAT_TB", "1")
    inst = W.plain_instance(32, 24, 20.0, 2.84, 50.0)
    s = S.Solver(crystal=W.CRYSTAL_QPM50, nx=32, ny=32, nz=24, lx=inst.lx, ly=inst.ly, thermal=True, bc=1)
    if rule == "relative":
        s.set_jacobi_rule(1e-9, check_every=5, max_sweeps=100000)
    monkeypatch.setenv("SHG_HEAT_TMA_STARVE", "1")
    t0 = time.time()
    with pytest.raises(ShgError, match="TMA pipeline wait gave up"):
        s.run(20.0, inst.waist, inst.focal, 50.0, 25.0, 50.0, 50.0)
    # one residual check: at most check_every sweeps of about a second each, not the
    # 5000-sweep blocks of the reference's rule (or the relative rule's sweep cap)
    assert time.time() - t0 < 60
    monkeypatch.delenv("SHG_HEAT_TMA_STARVE")
    s.run(20.0, inst.waist, inst.focal, 50.0, 25.0, 50.0, 50.0)
    ref = S.Solver(crystal=W.CRYSTAL_QPM50, nx=32, ny=32, nz=24, lx=inst.lx, ly=inst.ly, thermal=True, bc=1)
    if rule == "relative":
        ref.set_jacobi_rule(1e-9, check_every=5, max_sweeps=100000)
    ref.run(20.0, inst.waist, inst.focal, 50.0, 25.0, 50.0, 50.0)
    assert bits_equal(s.temperature(), ref.temperature())
    assert s.jacobi_counts() == ref.jacobi_counts()


def test_starved_device_sweeps_report_through_their_own_error_word(monkeypatch):
    monkeypatch.setenv("SHG_HEAT", "tma")
    monkeypatch.setenv("SHG_HEAT_TB", "1")
    import ctypes as C
    from shg_focused_gaussian_beams_gb300 import _lib
    from shg_focused_gaussian_beams_gb300.solver import _cfg_from
    n, nz = 40, 33
    cfg = _cfg_from(W.CRYSTAL_QPM50, nx=n, ny=n, nz=nz, lx=600.0, ly=600.0)
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, n, n, nz, 600.0, 600.0))
    T0 = o.init_temperature(48.0, 50.0, 46.5, 1)
    Q = (np.random.default_rng(2).random(T0.shape) * 5e-9).astype(np.float32)
    QK = torch.from_numpy(Q / np.float32(W.CRYSTAL_QPM50.kth)).cuda()
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    monkeypatch.setenv("SHG_HEAT_TMA_STARVE", "1")
    Ta = torch.from_numpy(T0).cuda()
    Tb = Ta.clone()
    rc = L.shg_heat_sweeps_device(C.byref(cfg), Ta.data_ptr(), Tb.data_ptr(), QK.data_ptr(), 25.0, 1, 1, st)
    assert rc == 3 and b"TMA pipeline wait gave up" in L.shg_last_error()
    monkeypatch.delenv("SHG_HEAT_TMA_STARVE")
    Ta = torch.from_numpy(T0).cuda()
    Tb = Ta.clone()
    _lib.check(L.shg_heat_sweeps_device(C.byref(cfg), Ta.data_ptr(), Tb.data_ptr(), QK.data_ptr(), 25.0, 4, 1, st),
               "shg_heat_sweeps_device")
    torch.cuda.synchronize()
    assert bits_equal(Ta.cpu().numpy(), o.heat_sweeps(T0, Q, 25.0, 4, 1))
