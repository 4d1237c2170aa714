"""The split GEMM's arithmetic, run on the host with the device code's own
digit split and rounding (csrc/fold_round.h, compiled with g++), against exact
rational dot products (fractions.Fraction):

* x and y are cut into eight signed 7-bit digits on the scales 2^Ex, 2^Ey of
  their largest elements (fixed56 / digit);
* per K-chunk of 128 the 36 digit pairs with s + t <= 7 are summed per level
  d = s + t -- the bound the kernel relies on, |level sum| <= 128 (d + 1) 127^2
  < 2^24 (exact in FP32), is asserted, and so is the 32-bit pair combine
  v_2k 2^7 + v_2k+1 of its fold;
* the levels are folded into int64 H (levels 0-3) and Lo (4-7) and rounded by
  to_double_exact (the overlap finalizers) and to_double_window (the C M
  epilogue).

Error bound per dot product of length K: every product term loses the digit
pairs s + t >= 8 (at most 7 127^2 2^-70 + ... < 2^-53 of 2^(Ex+Ey)) and the
truncation below 2^(E-56) of each operand (< 2^-55 of the scale), so
|result - exact| <= K 2^-52 2^(Ex+Ey) + the final rounding (within an ulp, and
for the window form 2^(s-63) 2^(Ex+Ey) more).
"""
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

DRIVER = r"""
#include <cstdio>
#include <cstring>
#include <vector>
#include "fold_round.h"
using namespace gbcp::fold;

int main(int argc, char** argv) {
  FILE* f = fopen(argv[1], "rb");
  int nvec = 0, K = 0;
  if (fread(&nvec, 4, 1, f) != 1 || fread(&K, 4, 1, f) != 1) return 2;
  std::vector<double> x((size_t)nvec * K), y((size_t)nvec * K);
  if (fread(x.data(), 8, x.size(), f) != x.size() || fread(y.data(), 8, y.size(), f) != y.size()) return 2;
  fclose(f);
  for (int v = 0; v < nvec; ++v) {
    const double* a = x.data() + (size_t)v * K;
    const double* b = y.data() + (size_t)v * K;
    unsigned long long ma = 0, mb = 0;
    for (int k = 0; k < K; ++k) {
      const unsigned long long ba = to_bits(a[k]) & ~(1ull << 63), bb = to_bits(b[k]) & ~(1ull << 63);
      ma = ba > ma ? ba : ma;
      mb = bb > mb ? bb : mb;
    }
    const int ea = exp_of_max(ma), eb = exp_of_max(mb);
    long long H = 0, Lo = 0;
    int chunks = 0;
    for (int k0 = 0; k0 < K; k0 += 128, ++chunks) {
      long long lev[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int k = k0; k < K && k < k0 + 128; ++k) {
        bool na, nb;
        const unsigned long long fa = fixed56(a[k], ea, na), fb = fixed56(b[k], eb, nb);
        for (int s = 0; s < 8; ++s)
          for (int t = 0; s + t < 8; ++t) lev[s + t] += (long long)digit(fa, na, s) * digit(fb, nb, t);
      }
      for (int d = 0; d < 8; ++d)
        if (lev[d] > 128ll * (d + 1) * 16129 || -lev[d] > 128ll * (d + 1) * 16129 || lev[d] >= (1 << 24) ||
            -lev[d] >= (1 << 24)) {
          printf("LEVEL_BOUND %d %d %lld\n", v, d, lev[d]);
          return 3;
        }
      for (int g = 0; g < 8; g += 2) {
        const long long pr = lev[g] * 128 + lev[g + 1];
        if (pr > 2147483647ll || pr < -2147483648ll) {
          printf("PAIR_BOUND %d %d %lld\n", v, g, pr);
          return 3;
        }
      }
      H += (lev[0] * 128 + lev[1]) * 16384 + (lev[2] * 128 + lev[3]);
      Lo += (lev[4] * 128 + lev[5]) * 16384 + (lev[6] * 128 + lev[7]);
    }
    const int s = window_drop_bits(chunks);
    printf("%d %d %d %.17g %.17g\n", ea, eb, s, to_double_exact(H, Lo, ea + eb), to_double_window(H, Lo, ea + eb, s));
  }
  return 0;
}
"""


def cases(rng):
    out = []
    for K in (1, 7, 128, 129, 1000, 4096):
        for kind in ("normal", "wide", "cancel", "sparse"):
            x = rng.standard_normal(K)
            y = rng.standard_normal(K)
            if kind == "wide":  # magnitudes over 40 binades
                x *= 2.0 ** rng.integers(-40, 1, K)
                y *= 2.0 ** rng.integers(-40, 1, K)
            elif kind == "cancel" and K > 1:  # the dot product nearly cancels
                y[-1] = -(x[:-1] @ y[:-1]) / x[-1]
            elif kind == "sparse":
                x[rng.random(K) < 0.7] = 0.0
            out.append((x, y))
    out.append((np.array([3.0, -2.5, 1e-300]), np.array([1e-5, 7.0, 1e300])))  # extreme spread
    out.append((np.zeros(64), rng.standard_normal(64)))
    return out


def test_split_gemm_model_against_exact(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    rng = np.random.default_rng(11)
    cs = cases(rng)
    K = max(len(x) for x, _ in cs)
    X = np.zeros((len(cs), K))
    Y = np.zeros((len(cs), K))
    for i, (x, y) in enumerate(cs):
        X[i, :len(x)] = x
        Y[i, :len(y)] = y
    src = tmp_path / "model.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "model"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "cpmd_gb300" / "csrc"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    inp = tmp_path / "in.bin"
    inp.write_bytes(np.array([len(cs), K], np.int32).tobytes() + X.tobytes() + Y.tobytes())
    run = subprocess.run([str(exe), str(inp)], capture_output=True, text=True)
    assert run.returncode == 0, run.stdout + run.stderr
    lines = run.stdout.split("\n")
    for i, (x, y) in enumerate(cs):
        ea, eb, s, exact_form, window_form = lines[i].split()
        ea, eb, s = int(ea), int(eb), int(s)
        ref = sum((Fraction(float(a)) * Fraction(float(b)) for a, b in zip(X[i], Y[i])), Fraction(0))
        scale = Fraction(2) ** (ea + eb)
        n = len(x)
        for val, extra in ((float(exact_form), 0), (float(window_form), Fraction(2) ** (s - 63))):
            ulp = Fraction(2) ** (int(np.frexp(val)[1]) - 53) if val != 0.0 else Fraction(0)
            bound = n * Fraction(2) ** -52 * scale + ulp + extra * scale
            assert abs(Fraction(val) - ref) <= bound, (i, val, float(ref))
