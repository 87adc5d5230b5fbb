"""The shg CLI's argument handling (SHG.cpp:37-50 argv plus options) on paths that end
before any device call, so no GPU is needed."""
import os
import subprocess

import pytest

from _util import ROOT

EXE = os.path.join(ROOT, "shg_focused_gaussian_beams_gb300", "_build", "shg")


def _run(args, tmp_path):
    if not os.path.isfile(EXE):
        pytest.skip("shg CLI not built")
    return subprocess.run([EXE] + args, capture_output=True, text=True, timeout=60, cwd=str(tmp_path))


@pytest.mark.parametrize("args", [[], ["30", "29"], ["30", "29", "50", "50", "1"]])
def test_too_few_arguments_print_the_usage(args, tmp_path):
    r = _run(args, tmp_path)
    assert r.returncode == 2 and "usage: shg P waist T1 T2 SOLS STMP" in r.stderr


@pytest.mark.parametrize("opt,msg", [(["--nx"], "missing value for --nx"), (["--bogus", "1"], "unknown option --bogus"),
                                     (["--crystal", "bbo"], "unknown crystal bbo")])
def test_bad_options_are_refused(opt, msg, tmp_path):
    r = _run(["30", "29", "50", "50", "1", "0"] + opt, tmp_path)
    assert r.returncode == 2 and msg in r.stderr
    # refused before the run: no timing file was written
    assert not list(tmp_path.glob("CPUTime_*"))
