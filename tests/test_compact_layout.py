"""The compact plan's order layout helpers (tsg_internal.cuh), compiled for the
host with nvcc: every span's padded order stride, the chunks of 64 rows of 32
depth-first positions, and the chunk a sample-range endpoint belongs to.

The rows pass and the seek rely on three properties checked here for every
sample count a compact plan allows (at most 65,535) at the chunk and row
boundaries:
* a span has at most 32 chunks (the seek keeps one chunk offset per lane);
* an endpoint's row within its chunk is at most the chunk's row count (the
  row after the last only for position = number of samples), so the rows
  pass's shared-memory rows are never indexed past the chunk;
* the order stride is the sample count rounded up to a multiple of 8
  (16-byte copies start on 16-byte boundaries)."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include "tsg_internal.cuh"
// prints n, chunks, stride and the worst violations over the endpoints
// tried: 0 when every property holds
int main() {
    long long bad = 0, worst_chunks = 0;
    for (long long n = 1; n <= 65535; n++) {
        const bool edge = n <= 4200 || n % 32 <= 1 || n % 32 == 31 || n % 2048 <= 1
            || n % 2048 == 2047 || n >= 65000;
        if (!edge) {
            continue;
        }
        const long long CH = tsg::compact_row_chunks(n);
        const long long nrows = (n + 31) / 32;
        if (CH > worst_chunks) worst_chunks = CH;
        if (CH < 1 || CH > 32 || (CH - 1) * 64 >= nrows + (nrows == 0)) bad++;
        const long long st = tsg::compact_order_stride(n);
        if (st % 8 != 0 || st < n || st >= n + 8) bad++;
        for (long long x = 0; x <= n; x++) {
            const bool near = x % 32 <= 1 || x % 32 == 31 || x == n;
            if (!near) continue;
            const long long c = tsg::compact_chunk_of(x, n);
            const long long rb = c * 64;
            const long long nr = rb + 64 < nrows ? 64 : nrows - rb;
            const long long l = (x >> 5) - rb;
            if (c < 0 || c >= CH || l < 0 || l > nr) bad++;
            if (l == nr && !(x == n && n % 32 == 0)) bad++;
        }
    }
    std::printf("%lld %lld\n", bad, worst_chunks);
    return 0;
}
"""


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def test_compact_layout_helpers(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = tmp_path / "layout.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "layout"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                    "-I", os.path.join(REPO, "tskit_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    bad, worst_chunks = int(out[0]), int(out[1])
    assert bad == 0
    assert worst_chunks == 32  # 65,535 samples: 2,048 rows, 32 chunks
