"""Reference-format outputs on the device path (GB300 only): shg_run's Files.h files
(SOLS=1 / SOLS=0, STMP=1), the `shg` CLI with SHG.cpp's argv, and the SHG.sh-style sweep."""
import os
import subprocess

import numpy as np
import pytest

from _util import FIELD_RTOL, ROOT, crystal_from_golden, golden, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import workloads as W  # noqa: E402
from shg_focused_gaussian_beams_gb300.files import load_matrix_complex, save_matrix_complex  # noqa: E402
from shg_focused_gaussian_beams_gb300.solver import Solver  # noqa: E402


def test_sols1_files_match_fields_and_format(tmp_path):
    inst = W.plain_instance(64, 30, 10.0, 2.84, 50.0)
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=64, ny=64, nz=30, lx=inst.lx, ly=inst.ly)
    s.set_output_dir(str(tmp_path))
    s.run(inst.power, inst.waist, inst.focal, inst.temp, save_only_last=True)
    po, so = s.fields()
    assert np.array_equal(load_matrix_complex(str(tmp_path), "Pump_out"), po)
    assert np.array_equal(load_matrix_complex(str(tmp_path), "Signal_out"), so)
    ours = open(tmp_path / "Signal_out_i.dat").read()
    os.makedirs(tmp_path / "py", exist_ok=True)
    save_matrix_complex(str(tmp_path / "py"), "Signal_out", so)
    assert ours == open(tmp_path / "py" / "Signal_out_i.dat").read()


def test_sols0_writes_every_slice(tmp_path):
    inst = W.plain_instance(32, 12, 10.0, 2.84, 50.0)
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=32, ny=32, nz=12, lx=inst.lx, ly=inst.ly)
    s.set_output_dir(str(tmp_path))
    s.run(inst.power, inst.waist, inst.focal, inst.temp, save_only_last=False)
    po, so = s.fields()
    for k in range(12):
        assert (tmp_path / f"Pump_{k}_r.dat").exists() and (tmp_path / f"Signal_{k}_i.dat").exists()
    assert np.array_equal(load_matrix_complex(str(tmp_path), "Pump_11"), po)
    assert np.array_equal(load_matrix_complex(str(tmp_path), "Signal_11"), so)
    assert np.all(load_matrix_complex(str(tmp_path), "Signal_0") == 0)
    import oracle as O
    o = O.Oracle(O.make_cfg(W.CRYSTAL_QPM50, 32, 32, 12, inst.lx, inst.ly))
    p0 = o.set_pump(inst.power, inst.focal, inst.waist, inst.temp)
    assert rel_l2(load_matrix_complex(str(tmp_path), "Pump_0"), p0) < 1e-6


def test_thermal_files_with_temperature(tmp_path):
    g = golden("thermal_topopen.npz")
    nz, ny, nx = g["T"].shape
    s = Solver(crystal=crystal_from_golden(g), nx=nx, ny=ny, nz=nz, lx=float(g["cfg_lx"]), ly=float(g["cfg_ly"]),
               thermal=True, bc=0)
    s.set_output_dir(str(tmp_path))
    s.run(float(g["power"]), float(g["waist"]), 15000.0, float(g["temp"]), 25.0, float(g["t1"]), float(g["t2"]),
          save_only_last=True, save_temperature=True)
    T = s.temperature()
    for z in (0, nz // 2, nz - 1):
        rows = [[float(v) for v in line.rstrip("\n").split("\t") if v] for line in open(tmp_path / f"Tfinal_{z}.dat")]
        assert np.allclose(np.array(rows), T[z], rtol=1e-5, atol=0)
    assert rel_l2(load_matrix_complex(str(tmp_path), "Signal_out"), g["sh_out"]) < FIELD_RTOL


def test_cli_runs_with_reference_argv(tmp_path):
    g = golden("stock_cli.npz")
    exe = os.path.join(ROOT, "shg_focused_gaussian_beams_gb300", "_build", "shg")
    r = subprocess.run([exe, "30", "29", "55.66", "55.66", "1", "0", "--outdir", str(tmp_path)], capture_output=True,
                       text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert "Conversion efficiency" in r.stdout and "Nonlinear crystal = MgO:sPPLT" in r.stdout
    # SHG.cpp:85-97: the elapsed seconds appended to the per-grid timing file in the working directory
    assert float(open(tmp_path / "CPUTime_NZ_200_N_64_T.txt").read().split()[-1]) > 0
    so = load_matrix_complex(str(tmp_path), "Signal_out")
    assert rel_l2(so, g["sh_out"]) < FIELD_RTOL


def test_sweep_front_end(tmp_path):
    from shg_focused_gaussian_beams_gb300 import sweep
    logs = sweep.main(["--power", "10", "20", "30", "--waist", "28", "31", "--t1", "50.0", "--crystal", "qpm50",
                       "--nx", "64", "--ny", "64", "--nz", "40", "--lx", "463.26", "--ly", "463.26",
                       "--workdir", str(tmp_path)])
    assert len(logs) == 6
    folder = tmp_path / "Simulations" / "sPPLT_P_20_W_T1_50.0_WAIST_31"
    assert (folder / "Signal_out_r.dat").exists()
    assert (folder / "sPPLT_P_20_W_T1_50.0_WAIST_31.txt").exists()
    s = Solver(crystal=W.CRYSTAL_QPM50, nx=64, ny=64, nz=40, lx=463.26, ly=463.26)
    s.run(20.0, 31.0, 15000.0, 50.0)
    e = [v[4] for k, v in logs.items() if k.endswith("sPPLT_P_20_W_T1_50.0_WAIST_31")][0]
    assert abs(e - s.efficiency()) / s.efficiency() < 1e-6
    assert rel_l2(load_matrix_complex(str(folder), "Signal_out"), s.fields()[1]) < 1e-6
