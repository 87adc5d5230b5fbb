"""The library's host code under AddressSanitizer and UBSan, on the paths that need no GPU
(crystal indices, argument checking), in a child process with the sanitizer runtime
preloaded. The GPU paths run under the same build in tests/test_gpu_check.py."""
import os
import shutil

import pytest

from _diag import asan_runtime, run_child


@pytest.mark.skipif(not shutil.which(os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")) or asan_runtime() is None,
                    reason="needs nvcc and the AddressSanitizer runtime")
def test_host_paths_clean_under_asan_ubsan():
    from shg_focused_gaussian_beams_gb300 import build as B
    lib = B.build(variant="sanitize")
    rc, report, err = run_child("host", lib, sanitize=True, timeout=600)
    assert "ERROR: AddressSanitizer" not in err and "runtime error:" not in err, err[-3000:]
    assert rc == 0 and report is not None, err[-3000:]
    assert all(c["ok"] for c in report["cases"].values()), report
