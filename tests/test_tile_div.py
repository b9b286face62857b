"""The multi-grid kernels' tile numbering: the multiply-shift quotient of
gmes_internal.cuh (tile_div_of / tile_quot) against integer division, for
divisors and dividends across [1, 2^31), on the host.  The helper is
compiled from the library's own header with nvcc into a small host program
(no GPU is touched)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cstdio>
#include <cstdint>
#include "gmes_internal.cuh"

static uint64_t rng = 88172645463325252ull;
static uint32_t next() {  // xorshift64
  rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;
  return (uint32_t)(rng >> 16);
}

static long check(uint32_t d, uint32_t n) {
  uint32_t m; int32_t s;
  gmes::tile_div_of(d, m, s);
  const uint32_t q = (uint32_t)(((uint64_t)n * m) >> s);  // tile_quot's arithmetic
  return q == n / d ? 0 : 1;
}

int main() {
  long bad = 0, tried = 0;
  const uint32_t lim = 0x7fffffffu;  // n, d < 2^31
  for (uint32_t d = 1; d < 4096; ++d)
    for (uint32_t n : {0u, 1u, d - 1, d, d + 1, 2 * d - 1, lim - 1, lim - d})
      if (n < lim) { bad += check(d, n); ++tried; }
  for (int b = 1; b < 31; ++b)
    for (uint32_t d : {(1u << b) - 1, 1u << b, (1u << b) + 1})
      for (int t = 0; t < 200; ++t) {
        const uint32_t n = next() & lim;
        const uint32_t k = n / d;
        bad += check(d, n); ++tried;
        if (k > 0) { bad += check(d, k * d - 1); bad += check(d, k * d); tried += 2; }
      }
  for (int t = 0; t < 200000; ++t) {
    const uint32_t d = (next() & lim) | 1u, n = next() & lim;
    bad += check(d, n); ++tried;
  }
  std::printf("%ld %ld\n", tried, bad);
  return bad != 0;
}
'''


def test_tile_quotient_is_exact(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "tile_div.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "tile_div"
    subprocess.run([nvcc, "-std=c++17", "-O2", f"-I{ROOT / 'include'}",
                    f"-I{ROOT / 'gmes_gb300' / 'csrc'}", str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    tried, bad = map(int, out.stdout.split())
    assert tried > 200000 and bad == 0, out.stdout
