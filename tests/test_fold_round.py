"""The split GEMM's integer rounding of int64 level sums to FP64 (csrc/fold_round.h),
compiled for the host with g++ and checked against an independent int128 rounding:

* to_double_exact: bit-identical to the correctly rounded (nearest, ties to even)
  value of (H 2^28 + Lo) 2^(ee-63), random and exact-tie cases;
* to_double_window (the C M epilogue): |error| <= 2^(s+ee-63) + 1 ulp of the
  result, over the level-sum ranges one to 128 K-chunks produce.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

DRIVER = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "fold_round.h"
using gbcp::fold::to_double_exact;
using gbcp::fold::to_double_window;
using gbcp::fold::window_drop_bits;

static unsigned long long bits_of(double d) { unsigned long long b; memcpy(&b, &d, 8); return b; }
static double of_bits(unsigned long long b) { double d; memcpy(&d, &b, 8); return d; }

// independent reference: the int128 value rounded to 53 bits, ties to even
static double ref(long long H, long long Lo, int ee) {
  __int128 v = (__int128)H * ((__int128)1 << 28) + (__int128)Lo;
  if (v == 0) return 0.0;
  const bool neg = v < 0;
  unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  int top = 127;
  while (!((m >> top) & 1)) --top;
  unsigned long long mant;
  if (top > 52) {
    const int sh = top - 52;
    mant = (unsigned long long)(m >> sh);
    const unsigned __int128 rem = m & ((((unsigned __int128)1) << sh) - 1);
    const unsigned __int128 half = ((unsigned __int128)1) << (sh - 1);
    if (rem > half || (rem == half && (mant & 1))) ++mant;
    if (mant >> 53) { mant >>= 1; ++top; }
  } else {
    mant = (unsigned long long)m << (52 - top);
  }
  const int be = top + ee - 63 + 1023;
  const unsigned long long sg = neg ? (1ull << 63) : 0ull;
  if (be <= 0) return of_bits(sg);
  if (be >= 2047) return of_bits(sg | 0x7FF0000000000000ull);
  return of_bits(sg | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

int main() {
  std::mt19937_64 g(2024);
  long long bad_exact = 0, bad_window = 0, n = 0;
  for (int it = 0; it < 2000000; ++it) {
    const int bh = 1 + (int)(g() % 61), bl = 1 + (int)(g() % 61);
    long long H = (long long)(g() >> (64 - bh)), Lo = (long long)(g() >> (64 - bl));
    if (g() & 1) H = -H;
    if (g() & 1) Lo = -Lo;
    if (it % 5 == 0) Lo = -(H % (1ll << 20)) * (1ll << 28) + (long long)(g() % 9) - 4;  // cancellation
    if (it % 7 == 0) Lo = (long long)(g() % 3) << (g() % 30);                           // ties
    const int ee = (int)(g() % 200) - 100;
    ++n;
    if (bits_of(to_double_exact(H, Lo, ee)) != bits_of(ref(H, Lo, ee))) ++bad_exact;
  }
  for (int it = 0; it < 2000000; ++it) {
    const int chunks = 1 << (g() % 8);
    const int s = window_drop_bits(chunks);
    const unsigned long long hmax = (unsigned long long)(4.3e12 * chunks), lmax = (unsigned long long)(2.3e13 * chunks);
    long long H = (long long)(g() % hmax), Lo = (long long)(g() % lmax);
    if (g() & 1) H = -H;
    if (g() & 1) Lo = -Lo;
    if (it % 3 == 0) H >>= (g() % 40);
    if (it % 11 == 0) { H = 0; Lo >>= (g() % 40); }
    const int ee = (int)(g() % 120) - 60;
    const double a = ref(H, Lo, ee), b = to_double_window(H, Lo, ee, s);
    const double bound = std::ldexp(1.0, s - 63 + ee) + (a != 0.0 ? std::ldexp(1.0, std::ilogb(a) - 52) : 0.0);
    ++n;
    if (!(std::fabs(a - b) <= bound)) ++bad_window;
  }
  printf("%lld %lld %lld\n", n, bad_exact, bad_window);
  return 0;
}
"""


def test_fold_round_host(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "fold_round_check.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "fold_round_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "cpmd_gb300" / "csrc"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    n, bad_exact, bad_window = (int(x) for x in out)
    assert n == 4000000
    assert bad_exact == 0
    assert bad_window == 0
