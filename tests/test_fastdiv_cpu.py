"""The ensemble kernel's division by a channel's width (FastDiv in tlbm_gb300/csrc/ensemble.h:
Granlund and Montgomery's division by an invariant integer) against exact division, on the
host: every divisor up to 4096 for the numerators below 2^16 and random ones up to 2^31 - 1,
and widths up to 65535 at the ends of the range.  The same constants drive the device code."""

import os
import subprocess

import pytest

from tlbm_gb300 import build as B

SRC = r"""
#include <cstdio>
#include <cstdint>
#include "ensemble.h"
using namespace tlbm;
static uint32_t div_fast(uint32_t n, FastDiv d) {
  const uint32_t hi = static_cast<uint32_t>((uint64_t(n) * d.m) >> 32);
  return (hi + n) >> d.l;
}
int main() {
  uint64_t state = 0x9E3779B97F4A7C15ull, bad = 0, checks = 0;
  auto next = [&]() { state = state * 6364136223846793005ull + 1442695040888963407ull;
                      return static_cast<uint32_t>(state >> 33); };
  for (uint32_t d = 1; d <= 65535; d += (d < 4096 ? 1 : 251)) {
    const FastDiv f = make_fast_div(d);
    const uint32_t lim = d <= 4096 ? (1u << 16) : 4096u;
    for (uint32_t n = 0; n < lim; ++n, ++checks) bad += div_fast(n, f) != n / d;
    for (int k = 0; k < 2000; ++k, ++checks) {
      const uint32_t n = next() & 0x7FFFFFFFu;
      bad += div_fast(n, f) != n / d;
    }
    const uint32_t ends[] = {0x7FFFFFFFu, 0x7FFFFFFEu, d - 1, d, 2 * d - 1};
    for (uint32_t n : ends) { ++checks; bad += div_fast(n, f) != n / d; }
  }
  std::printf("%llu %llu\n", (unsigned long long)checks, (unsigned long long)bad);
  return bad != 0;
}
"""


def test_fast_division_constants(tmp_path):
    try:
        nvcc = B.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    cu = tmp_path / "fastdiv.cu"
    cu.write_text(SRC)
    exe = str(tmp_path / "fastdiv")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I" + B.CSRC, "-I" + os.path.join(B.REPO, "include"),
                        str(cu), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    checks, bad = map(int, r.stdout.split())
    assert checks > 200_000_000 and bad == 0 and r.returncode == 0
