"""Diagnostic builds on the GPU (GB300 only), each in a child process (tests/_check_run.py):

* the SHG_CHECK build: device-side index checks (descriptors, stages, field, propagator,
  slice and voxel indices, distributed-shared-memory ranks, TMA box coordinates) that record
  a failure site instead of faulting. Its reporting path is shown by a self-test kernel
  that records a failure without touching memory; then every kernel family runs at 16-64
  point grids against the oracle, and no check may fail;
* the host code under AddressSanitizer and UBSan (runtime preloaded), on plain and THERMAL
  runs with file outputs, the batch schedules and the heat components.
"""
import concurrent.futures as cf

import pytest

from _diag import asan_runtime, run_child

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("no CUDA device", allow_module_level=True)

from shg_focused_gaussian_beams_gb300 import build as B  # noqa: E402


@pytest.fixture(scope="module")
def diag_libs():
    variants = ["check"] + (["sanitize"] if asan_runtime() else [])
    with cf.ThreadPoolExecutor(max_workers=len(variants)) as ex:
        futs = {v: ex.submit(B.build, False, 8, False, v) for v in variants}
        return {v: f.result() for v, f in futs.items()}


def test_check_build_reports_and_small_solves_pass_every_check(diag_libs):
    rc, report, err = run_child("check", diag_libs["check"], sanitize=False)
    assert report is not None, err[-3000:]
    bad = {k: v for k, v in report["cases"].items() if not v["ok"]}
    assert rc == 0 and not bad, (bad, err[-2000:])
    assert report["cases"]["selftest_reported"]["ok"] and report["cases"]["no_failed_check"]["ok"]


def test_host_code_clean_under_asan_ubsan_on_gpu_paths(diag_libs):
    if "sanitize" not in diag_libs:
        pytest.skip("no AddressSanitizer runtime on this machine")
    rc, report, err = run_child("sanitize", diag_libs["sanitize"], sanitize=True)
    assert "ERROR: AddressSanitizer" not in err and "runtime error:" not in err, err[-3000:]
    assert report is not None, err[-3000:]
    bad = {k: v for k, v in report["cases"].items() if not v["ok"]}
    assert rc == 0 and not bad, (bad, err[-2000:])


def test_check_build_at_the_benchmarked_sizes(diag_libs):
    """The SHG_CHECK build on the workloads as benchmarked: the 512-solve sweep with every
    schedule the autotuner tries, lone 128x128x200 and 256x256x400 solves on the persistent
    grid, and a THERMAL 256x256x400 run; no check may fail."""
    rc, report, err = run_child("fullsize", diag_libs["check"], sanitize=False)
    assert report is not None, err[-3000:]
    bad = {k: v for k, v in report["cases"].items() if not v["ok"]}
    assert rc == 0 and not bad, (bad, err[-2000:])
