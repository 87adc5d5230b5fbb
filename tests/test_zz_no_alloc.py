"""The allocation-free plain CWES (shg_cwes_noalloc) against the allocating entry point.

Some callers cannot call cudaMalloc (their device memory belongs to another allocator, or
their loop must not allocate); shg_cwes_noalloc keeps all working memory in a fixed device
array instead. This file is collected last so that a stop-at-first-failure run has run
every other test before it; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from _util import FIELD_RTOL, crystal_from_golden, golden, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import _lib  # noqa: E402
from shg_focused_gaussian_beams_gb300.solver import Solver, _cfg_from  # noqa: E402


def _noalloc(cfg, temp, pump, sh=None):
    po = torch.empty_like(pump)
    so = torch.empty_like(pump)
    eta = C.c_double()
    st = torch.cuda.current_stream().cuda_stream
    rc = _lib.lib().shg_cwes_noalloc(C.byref(cfg), temp, pump.data_ptr(), None if sh is None else sh.data_ptr(),
                                     po.data_ptr(), so.data_ptr(), C.byref(eta), st)
    _lib.check(rc, "shg_cwes_noalloc")
    torch.cuda.synchronize()
    return po.cpu().numpy(), so.cpu().numpy(), eta.value


def test_noalloc_matches_allocating_entry_point_twice():
    g = golden("c0_small.npz")
    crystal = crystal_from_golden(g)
    nx, nz = int(g["cfg_nx"]), int(g["cfg_nz"])
    temp = float(g["temp"])
    cfg = _cfg_from(crystal, nx=nx, ny=nx, nz=nz)
    rng = np.random.default_rng(9)
    pump1 = g["pump_in"]
    pump2 = (g["pump_in"] * (1 + 0.05 * rng.standard_normal(pump1.shape))).astype(np.complex64)
    sh2 = (0.01 * pump2).astype(np.complex64)
    ref = Solver(crystal=crystal, nx=nx, ny=nx, nz=nz, lx=float(g["cfg_lx"]), ly=float(g["cfg_ly"]))
    for pump, sh in ((pump1, None), (pump2, sh2)):
        p = torch.from_numpy(pump).cuda()
        s = None if sh is None else torch.from_numpy(sh).cuda()
        po_a, so_a = ref.cwes_device(temp, p, s)
        torch.cuda.synchronize()
        eta_a = ref.efficiency()
        po_n, so_n, eta_n = _noalloc(cfg, temp, p, s)
        assert rel_l2(so_n, so_a.cpu().numpy()) < FIELD_RTOL
        assert rel_l2(po_n, po_a.cpu().numpy()) < FIELD_RTOL
        assert abs(eta_n - eta_a) / eta_a < 1e-4


def test_noalloc_rejects_sizes_beyond_its_scratch():
    cfg = _cfg_from(None, nx=256, ny=256, nz=10)
    p = torch.zeros((256, 256), dtype=torch.complex64, device="cuda")
    rc = _lib.lib().shg_cwes_noalloc(C.byref(cfg), 50.0, p.data_ptr(), None, p.data_ptr(), p.data_ptr(), None,
                                     None)
    assert rc == 1 and b"scratch" in _lib.lib().shg_last_error()
    cfg = _cfg_from(None, nx=64, ny=64, nz=5000)
    rc = _lib.lib().shg_cwes_noalloc(C.byref(cfg), 50.0, p.data_ptr(), None, p.data_ptr(), p.data_ptr(), None,
                                     None)
    assert rc == 1
