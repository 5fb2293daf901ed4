"""The fast division the cell kernels use for cell coordinates (FastDiv in
csrc/mf_common.cuh: n / d = (umulhi(n, mul) + n) >> shift with per-level
multipliers) agrees with integer division for every divisor a level can
have (cell counts per direction and plane, up to 70000) and for random
large divisors up to 2^31, with dividends below 2^31 (cell counts are
checked to stay below it).
Host code compiled by nvcc and run on the CPU; the device path computes the
same expression with __umulhi."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "matrix-free-dealii-precice_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include "mf_common.cuh"
using namespace mfgpu;
int main()
{
  uint64_t state = 0x9e3779b97f4a7c15ull, checked = 0;
  auto next = [&] { state ^= state << 13; state ^= state >> 7; state ^= state << 17; return state; };
  for (unsigned d = 1; d <= 70000; d += (d < 4096 ? 1 : 97))
    {
      const FastDiv f = make_fastdiv(d);
      const unsigned edge[] = {0u, 1u, d - 1, d, d + 1, 2 * d - 1, 2 * d, 0x7fffffffu, 0x7ffffffeu,
                               0x7fffffffu / d * d, 0x7fffffffu / d * d - 1};
      for (unsigned n : edge)
        {
          if (n > 0x7fffffffu)
            continue;
          if (f.div(n) != n / d || f.mod(n) != n % d)
            {
              std::printf("FAIL d=%u n=%u\n", d, n);
              return 1;
            }
          ++checked;
        }
      for (int i = 0; i < 64; ++i)
        {
          const unsigned n = unsigned(next() & 0x7fffffffu);
          if (f.div(n) != n / d || f.mod(n) != n % d)
            {
              std::printf("FAIL d=%u n=%u\n", d, n);
              return 1;
            }
          ++checked;
        }
    }
  // large divisors up to 2^31: random ones and the powers of two and
  // their neighbours
  for (int t = 0; t < 20000 + 3 * 31; ++t)
    {
      unsigned d;
      if (t < 20000)
        d = 1u + unsigned(next() % 0x7fffffffull);
      else
        {
          const int k = (t - 20000) % 31, v = (t - 20000) / 31;
          d = (1u << k) + (v == 0 ? 0u : (v == 1 ? 1u : (k > 0 ? 0xffffffffu : 0u)));
          if (d == 0u)
            continue;
        }
      const FastDiv f = make_fastdiv(d);
      for (int i = 0; i < 16; ++i)
        {
          const unsigned n = i == 0 ? 0x7fffffffu : (i == 1 ? d - 1 : (i == 2 && d < 0x7fffffffu ? d : unsigned(next() & 0x7fffffffu)));
          if (n > 0x7fffffffu)
            continue;
          if (f.div(n) != n / d || f.mod(n) != n % d)
            {
              std::printf("FAIL d=%u n=%u\n", d, n);
              return 1;
            }
          ++checked;
        }
    }
  std::printf("ok %llu\n", (unsigned long long)checked);
  return 0;
}
"""


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    return None


@pytest.mark.skipif(_nvcc() is None, reason="needs nvcc")
def test_fast_division_matches_integer_division(tmp_path):
    src = tmp_path / "fastdiv.cu"
    exe = tmp_path / "fastdiv"
    src.write_text(PROGRAM)
    r = subprocess.run([_nvcc(), "-std=c++17", "-O2", "-I", CSRC, str(src), "-o", str(exe)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")
