"""Files.h output formats (CPU): the writer renders values exactly as the reference's
std::setprecision(20) / default-precision streams do, checked against text the reference
itself wrote (tests/golden/stock_cli_signal_head.txt, made by make_golden.py)."""
import os

import numpy as np

from _util import GOLDEN
from shg_focused_gaussian_beams_gb300.files import load_matrix_complex, save_matrix_complex, save_tensor_real


def test_matrix_writer_reproduces_reference_text(tmp_path):
    ref = open(os.path.join(GOLDEN, "stock_cli_signal_head.txt")).read().splitlines(keepends=True)
    # the reference's first rows, parsed and re-rendered by the writer
    rows = [[float(x) for x in line.rstrip("\n").split("\t") if x] for line in ref]
    field = np.array(rows, np.float32) + 0j
    save_matrix_complex(str(tmp_path), "X", field)
    ours = open(tmp_path / "X_r.dat").read().splitlines(keepends=True)
    assert ours == ref


def test_round_trip_and_tensor(tmp_path):
    rng = np.random.default_rng(1)
    f = (rng.standard_normal((5, 7)) + 1j * rng.standard_normal((5, 7))).astype(np.complex64) * 1e-3
    save_matrix_complex(str(tmp_path), "F", f)
    assert np.array_equal(load_matrix_complex(str(tmp_path), "F"), f)
    T = (50 + rng.standard_normal((3, 4, 5))).astype(np.float32)
    save_tensor_real(str(tmp_path), "Tfinal", T)
    line = open(tmp_path / "Tfinal_2.dat").readline()
    assert line == "".join(format(float(x), "g") + "\t" for x in T[2, 0]) + "\n"


def test_sweep_folder_names_follow_shg_sh():
    """SHG.sh:76 names each point's folder from the raw argument text:
    sPPLT_P_${ARG1}_W_T1_${ARG3}_WAIST_${ARG2}."""
    from shg_focused_gaussian_beams_gb300.sweep import _folder
    assert _folder("30", "55.66", "29") == "sPPLT_P_30_W_T1_55.66_WAIST_29"
    assert _folder("2.5", "50", "31.25") == "sPPLT_P_2.5_W_T1_50_WAIST_31.25"
