// The integer arithmetic of the split GEMM shared by the device code and host
// tests (the file compiles as plain C++ too): splitting an FP64 value into
// signed 7-bit digits, and rounding the int64 level sums back to FP64.
//
// A split GEMM output is v 2^(ee-63) with v = H 2^28 + Lo: H holds levels 0-3
// and Lo levels 4-7 of the digit-pair sums (7 bits apart), ee = E_i + E_j the sum
// of the row and column scale exponents.  Both conversions use 64-bit integer
// instructions only: on GB300 the FP64 pipe (1/58 of FP32) would bound the
// epilogues that call them.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define GBCP_FOLD_FN __host__ __device__ __forceinline__
#else
#define GBCP_FOLD_FN inline
#endif

namespace gbcp {
namespace fold {

GBCP_FOLD_FN int clz64(unsigned long long x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

GBCP_FOLD_FN double from_bits(unsigned long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

GBCP_FOLD_FN unsigned long long to_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

// exponent E with |x| < 2^E from the bit pattern of max |x| (-1021 for zero and subnormals)
GBCP_FOLD_FN int exp_of_max(unsigned long long bits) {
  const int ex = (int)((bits >> 52) & 0x7FF);
  return (ex == 0) ? -1021 : ex - 1022;
}

// Fixed-point magnitude trunc(|x| 2^(56-E)) (< 2^56) and the sign, integer ops
// only; zero and subnormal values give 0.  x = 2^E sum_s d_s 2^(-7(s+1)) up to
// 2^(E-56), with the digits d_s of digit().
GBCP_FOLD_FN unsigned long long fixed56(double x, int E, bool& neg) {
  const unsigned long long b = to_bits(x);
  neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0) return 0ull;
  const unsigned long long M = (b & ((1ull << 52) - 1)) | (1ull << 52);
  int sh = ex - 1019 - E;  // = (ex - 1023) + 4 - E
  if (sh > 3) sh = 3;      // cannot happen when |x| < 2^E; keeps v < 2^56
  if (sh >= 0) return M << sh;
  return (sh <= -64) ? 0ull : (M >> (-sh));
}

// signed digit s (0 = most significant, s < 8) of a fixed56 magnitude: |d| <= 127
GBCP_FOLD_FN int digit(unsigned long long f, bool neg, int s) {
  const int d = (int)((f >> (7 * (7 - s))) & 127ull);
  return neg ? -d : d;
}

// v 2^(ee-63) correctly rounded (nearest, ties to even), valid for |H| < 2^62.
// v is rewritten as T 2^28 + r with T = H + floor(Lo / 2^28) and 0 <= r < 2^28;
// its magnitude |T'| 2^28 + r' is cut to a 64-bit window W (the bits below it
// only matter as a sticky bit) and W is rounded to 53 bits.  Results below the
// normal range flush to signed zero.
GBCP_FOLD_FN double to_double_exact(long long H, long long Lo, int ee) {
  const long long T = H + (Lo >> 28);
  const unsigned long long r = (unsigned long long)Lo & 0xFFFFFFFull;
  const bool neg = T < 0;
  const unsigned long long Tm = neg ? (unsigned long long)(-T) - (r != 0 ? 1ull : 0ull) : (unsigned long long)T;
  const unsigned long long rm = neg ? ((0x10000000ull - r) & 0xFFFFFFFull) : r;
  if ((Tm | rm) == 0) return 0.0;
  const int msbT = 63 - clz64(Tm);           // -1 when Tm == 0
  const int sh0 = msbT > 35 ? msbT - 35 : 0;  // bits of rm below the window
  const unsigned long long W = (Tm << (28 - sh0)) | (rm >> sh0);
  const bool sticky = (rm & ((1ull << sh0) - 1)) != 0;
  const int lz = clz64(W);
  const unsigned long long Wn = W << lz;
  int top = 63 - lz + sh0;  // index of the leading bit of the magnitude
  unsigned long long mant = Wn >> 11;
  const unsigned long long low = Wn & 0x7FFull;
  mant += (low > 0x400ull || (low == 0x400ull && (sticky || (mant & 1ull)))) ? 1ull : 0ull;
  if (mant >> 53) {
    mant >>= 1;
    ++top;
  }
  const int be = top + ee - 63 + 1023;
  const unsigned long long sg = neg ? (1ull << 63) : 0ull;
  if (be <= 0) return from_bits(sg);
  if (be >= 2047) return from_bits(sg | 0x7FF0000000000000ull);
  return from_bits(sg | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

// v 2^(ee-63) to within 2^(s+ee-63) plus half an ulp, in about a third of the
// instructions: the low s bits of Lo are dropped, so x = H 2^(28-s) +
// floor(Lo 2^-s) fits in 64 bits, and x is rounded to nearest even.  One K-chunk
// of 128 gives |H| < 2^42.03 and |Lo| < 2^44.4; with m chunks s = 9 +
// ceil(log2 m) keeps |x| < 2^62.  Branch-free (zero, underflow and overflow by
// selects), so that a thread's conversions can interleave.
GBCP_FOLD_FN double to_double_window(long long H, long long Lo, int ee, int s) {
  const long long x = (long long)((unsigned long long)H << (28 - s)) + (Lo >> s);
  const unsigned long long sg = (unsigned long long)x & (1ull << 63);
  const unsigned long long a = x < 0 ? (unsigned long long)(-x) : (unsigned long long)x;
  const int lz = clz64(a);                      // 64 when a == 0
  const unsigned long long m = a << (lz & 63);  // leading bit at 63 (0 when a == 0)
  const unsigned long long q = m >> 11;         // 53 bits
  const unsigned long long low = m & 0x7FFull;
  const unsigned long long r = q + ((low > 0x400ull || (low == 0x400ull && (q & 1ull))) ? 1ull : 0ull);
  const int be = (63 - lz) + s + ee - 63 + 1023;  // biased exponent of the leading bit
  // r in [2^52, 2^53]: its leading bit (and a rounding carry) lands in the exponent field
  unsigned long long bits = sg | (((unsigned long long)(be - 1) << 52) + r);
  bits = (a == 0 || be <= 0) ? sg : bits;
  bits = be >= 2046 ? (sg | 0x7FF0000000000000ull) : bits;
  return from_bits(bits);
}

// s for a unit of `chunks` K-chunks
GBCP_FOLD_FN int window_drop_bits(int chunks) {
  int s = 9;
  for (int m = 1; m < chunks; m *= 2) ++s;
  return s;
}

}  // namespace fold
}  // namespace gbcp
