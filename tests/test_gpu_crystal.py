"""The PPLN crystal option on the device against the oracle (GB300 only).

The oracle restates the same published LiNbO3 fit (Jundt 1997) as the device, so the
device path with crystal = 1 is checked like the reference crystal: plain CWES fields and
efficiency within the parity bar, delta-k(T) and both index tables bit for bit, and a small
THERMAL run with the reference's stop rule (counts equal, fields within the bar).
"""
import numpy as np
import pytest

import oracle as O
from _util import ETA_RTOL, FIELD_RTOL, bits_equal, eta, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import solver as S  # noqa: E402
from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402

CR = W.CRYSTAL_PPLN_QPM50


def test_ppln_plain_run_vs_oracle():
    w0 = W.waist_for_xi(2.84, 50.0, crystal=1)
    win = float(np.float32(16 * w0))
    n, nz = 64, 60
    o = O.Oracle(O.make_cfg(CR, n, n, nz, win, win))
    po_r, so_r = o.run_plain(10.0, w0, float(np.float32(15000.0)), 50.0)
    s = S.Solver(crystal=CR, nx=n, ny=n, nz=nz, lx=win, ly=win)
    s.run(10.0, w0, float(np.float32(15000.0)), 50.0)
    po, so = s.fields()
    assert rel_l2(so, so_r) < FIELD_RTOL and rel_l2(po, po_r) < FIELD_RTOL
    pin = o.set_pump(10.0, float(np.float32(15000.0)), w0, 50.0)
    e_ref = eta(pin, so_r, o.n(1.064, 50.0), o.n(np.float32(0.532), 50.0))
    assert abs(s.efficiency() - e_ref) / e_ref < ETA_RTOL
    assert e_ref > 1e-3  # phase matched near 50 C by construction


def test_ppln_thermal_tables_and_run_vs_oracle():
    n, nz = 32, 24
    cfg = O.make_cfg(CR, n, n, nz, 600.0, 600.0)
    o = O.Oracle(cfg)
    rng = np.random.default_rng(9)
    T = (o.init_temperature(50.0, 50.0, 50.0, 1) + rng.normal(0, 0.3, (nz, n, n))).astype(np.float32)
    D, NP, NS = S.dk_thermal(CR, T, lx=600.0, ly=600.0)
    assert bits_equal(D, o.dk_thermal(T))
    w0 = W.waist_for_xi(2.84, 50.0, crystal=1)
    ref = o.thermal_run(20.0, w0, float(np.float32(15000.0)), 50.0, 25.0, 50.0, 50.0, bc=1)
    s = S.Solver(crystal=CR, nx=n, ny=n, nz=nz, lx=600.0, ly=600.0, thermal=True, bc=1)
    s.run(20.0, w0, float(np.float32(15000.0)), 50.0, 25.0, 50.0, 50.0)
    assert s.jacobi_counts() == ref["counts"]
    po, so = s.fields()
    assert rel_l2(so, ref["sh"]) < FIELD_RTOL
    assert np.max(np.abs(s.temperature() - ref["T"])) < 1e-4
