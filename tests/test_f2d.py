"""The integer-pipe float -> double conversion of the FP64 reductions
(``f2d`` in csrc/common.cuh) against the host's own conversion, bit for bit:
every subnormal, both zeros and infinities, NaNs, and 2^16 mantissas at each
exponent.  The function is compiled as host code, so no GPU is needed."""
import os
import subprocess

import pytest

from prtcl_gb300 import build

PROGRAM = r'''
#include "common.cuh"
#include <cmath>
#include <cstdio>
#include <cstring>
static long n = 0, bad = 0;
static void check(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  double a = prtcl_gpu::f2d(f), b = double(f);
  uint64_t x, y;
  std::memcpy(&x, &a, 8);
  std::memcpy(&y, &b, 8);
  bool ok = std::isnan(f) ? (std::isnan(a) && (x >> 63) == (y >> 63)) : x == y;
  bad += !ok;
  ++n;
}
int main() {
  for (uint32_t m = 0; m < (1u << 23); ++m) {  // zeros and subnormals
    check(m);
    check(m | 0x80000000u);
  }
  for (uint32_t e = 1; e < 256; ++e)            // normals, infinities, NaNs
    for (uint32_t k = 0; k < 65536; ++k) {
      uint32_t m = (k * 2654435761u) & 0x7FFFFFu;
      check((e << 23) | m);
      check((e << 23) | m | 0x80000000u);
    }
  std::printf("%ld %ld\n", n, bad);
  return bad != 0;
}
'''


def test_f2d_matches_the_host_conversion(tmp_path):
    try:
        nvcc = build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    src = tmp_path / "f2d_check.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "f2d_check"
    r = subprocess.run([nvcc, "-O2", "-I", build.CSRC, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    n, bad = map(int, out.stdout.split())
    assert n == 2 * (1 << 23) + 2 * 255 * 65536 and bad == 0, out.stdout
    assert os.path.exists(exe)
