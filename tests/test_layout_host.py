"""Host-side checks of the device data layouts (no GPU needed).

The propagators are stored in the order the column transforms read them
(`hprop_index_rt` / `hprop_index` in csrc/shg_fft.cuh): the value of spectral row k and
column x must land exactly once in [0, N^2), at the slot that thread t reads into register r
where spec_index(t, r) == k, with registers 2j and 2j + 1 forming one 16-byte word and
the words of consecutive columns adjacent. A small host program built with nvcc from the
header checks this for every supported line length.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "shg_focused_gaussian_beams_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "shg_fft.cuh"
using namespace shg;

static int spec_index_host(int n, int t, int r) {   // spec_index<N, G> of shg_fft.cuh
    const int G = line_threads(n), E = n / G, Q = E / G;
    const int m = r / G, k1 = r % G;
    return (t * Q + m) + E * k1;
}

int main() {
    const int sizes[] = {16, 32, 64, 128, 256};
    for (int n : sizes) {
        const int G = line_threads(n), E = n / G;
        std::vector<int> seen((size_t)n * n, 0);
        for (int k = 0; k < n; ++k)
            for (int x = 0; x < n; ++x) {
                const size_t i = hprop_index_rt(n, k, x);
                if (i >= (size_t)n * n || seen[i]++) { std::printf("n=%d not a bijection at k=%d x=%d\n", n, k, x); return 1; }
            }
        for (int t = 0; t < G; ++t)
            for (int r = 0; r < E; ++r)
                for (int x = 0; x < n; ++x) {
                    const size_t i = hprop_index_rt(n, spec_index_host(n, t, r), x);
                    const size_t word = ((size_t)t * (E / 2) + r / 2) * n + x;   // the 16-byte word thread t loads
                    if (i != 2 * word + (r & 1)) { std::printf("n=%d t=%d r=%d x=%d: slot %zu\n", n, t, r, x, i); return 1; }
                }
    }
    std::printf("ok\n");
    return 0;
}
"""


def test_propagator_order_is_the_column_transform_order():
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout.cu")
        exe = os.path.join(d, "layout")
        with open(src, "w") as f:
            f.write(PROGRAM)
        subprocess.run([nvcc, "-std=c++17", "-I", CSRC, "-o", exe, src], check=True, capture_output=True)
        run = subprocess.run([exe], capture_output=True, text=True)
    assert run.returncode == 0 and run.stdout.strip() == "ok", run.stdout
