// Blocked Cholesky factorisation S = U^T U and triangular inverse X = U^{-1}
// of the overlap matrix (the reference's uinv: dpotrf + dtrtri,
// rgs_utils.mod.F90:95-162), spread over many CTAs.
//
// On GB300 one FP64 warp instruction holds its SM sub-partition for about 64
// clocks whatever the number of active lanes, so these kernels (a) keep the
// pivot chain short, (b) give every warp as few FP64 instructions as the work
// allows and (c) spread each block product over many SMs, one row group of RG
// rows (one warp per row, lane = column) per CTA.
//
// 32 x 32 blocks, right-looking:
//   for each diagonal block k:
//     diag    one CTA factors A_kk = U_kk^T U_kk and, interleaved with it,
//             Y = U_kk^{-T} by forward substitution; X_kk = Y^T
//     panel   U_kj = X_kk^T A_kj for every block j > k           -> work copy Uw
//     update  A_ij -= U_ki^T U_kj for k < i <= j                  -> S
//   then V_ik = X_ii U_ik for every i < k (into S, no longer needed), and X
//   block-diagonal by block-diagonal: X_ij = -sum_{k=i+1..j} V_ik X_kj, j - i = 1, 2, ...
// Every kernel reads the ortho status word before it writes and writes nothing
// once a step has failed; diag sets it to (global pivot index + 1) at a pivot at or below
// 2^-46 of that row's original diagonal (an exactly dependent set of states,
// where dpotrf's info > 0 would depend on rounding) and to -1 at a NaN.  S is
// row-major n x n (symmetric, upper part used; scratch on return); X is row-major
// n x n, upper triangular, zero below.
#include <algorithm>
#include <functional>

#include "ctx.h"

namespace gbcp {

namespace {

constexpr int B = 32;
constexpr int RG = 4;  // rows per CTA of the block-product kernels

__device__ __forceinline__ bool failed(const int* status) { return *(volatile const int*)status != 0; }

// pivot test without FP64 instructions: 0 when d > thr, -1 when d is NaN, 1 otherwise
__device__ __forceinline__ long long order_key(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool is_nan_bits(double x) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
__device__ __forceinline__ int pivot_bad(double d, double thr) {
  if (is_nan_bits(d)) return -1;
  if (is_nan_bits(thr)) return 1;
  return order_key(d) > order_key(thr) ? 0 : 1;
}

// Factor + invert the diagonal block k: U_kk -> Uw (upper, zero below),
// U_kk^{-1} -> X (diagonal block).  Eight warps, lane = column.
// Row i of the shared array z holds the forward-substitution accumulators
// Y[i][c] of Y = U_kk^{-T} for c < i and the matrix entries A[i][c] for c >= i;
// after step q row q is final: Y[q][c] (c < q), Y[q][q] = d^{-1/2}, U[q][c] (c > q).
//   Step q: warp 0 applies row q-1 to row q (one FMA per lane), takes the pivot
//   d = A[q][q] and scales the row by d^{-1/2} (one multiply per lane).  The six
//   warps on the other three SM sub-partitions (warps 1-3 and 5-7; warp 4 shares
//   warp 0's FP64 unit and stays idle) meanwhile apply row q-1 to rows
//   i = q+1..31 round-robin, one predicated FMA per row: z[i][c] -= U[q-1][i]
//   z[q-1][c] for c >= i (matrix) and c < q (Y).  One barrier per step; the pivot
//   chain is one FMA, the rsqrt and one multiply, and no updater has more than
//   five rows.
__global__ void __launch_bounds__(8 * B) k_chol_diag(const double* __restrict__ S, double* __restrict__ Uw,
                                                     double* __restrict__ X, const double* __restrict__ diag0, int n,
                                                     int k, int* __restrict__ status) {
  pdl_entry();
  __shared__ double z[B][B + 1];
  __shared__ double udiag[B];
  __shared__ int bad_sh;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int base = k * B;
  // all global loads in flight together (rows r = w + 8 t, lane = column)
  double v[B / 8];
#pragma unroll
  for (int t = 0; t < B / 8; ++t) {
    const int r = w + 8 * t, i = base + r, j = base + lane;
    v[t] = (lane >= r && i < n && j < n) ? S[(size_t)i * n + j] : 0.0;
  }
  const double d0 = (w == 0 && base + lane < n) ? diag0[base + lane] : 1.0;
  if (failed(status)) return;
#pragma unroll
  for (int t = 0; t < B / 8; ++t) {
    const int r = w + 8 * t, i = base + r, j = base + lane;
    z[r][lane] = (i < n && j < n) ? v[t] : (r == lane ? 1.0 : 0.0);
  }
  const double thr = 0x1p-46 * d0;  // warp 0, lane r: pivot threshold of row r
  if (threadIdx.x == 0) bad_sh = 0;
  __syncthreads();
  for (int q = 0; q < B; ++q) {
    if (w == 0) {
      double tv = z[q][lane];
      if (q > 0) tv = fma(-z[q - 1][q], z[q - 1][lane], tv);
      const double d = __shfl_sync(0xffffffffu, tv, q);
      const double tq = __shfl_sync(0xffffffffu, thr, q);
      const int bad = pivot_bad(d, tq);
      if (bad) {
        if (lane == 0) bad_sh = (bad < 0) ? -1 : base + q + 1;
      } else {
        const double inv = rsqrt(d);
        const double o = tv * inv;
        z[q][lane] = (lane == q) ? inv : o;
        if (lane == q) udiag[q] = o;
      }
    } else if (q > 0 && w != 4) {
      // updater u = 0..5: rows i = q + 1 + u + 6 t (q+1 .. 31, at most 5 per warp):
      // loads first, then the FMAs
      const int u = (w < 4) ? w - 1 : w - 2;
      constexpr int T = (B - 2 + 5) / 6;
      const double rv = z[q - 1][lane];
      double cf[T], zv[T];
#pragma unroll
      for (int t = 0; t < T; ++t) {
        const int i = q + 1 + u + 6 * t;
        if (i < B) {
          cf[t] = z[q - 1][i];
          zv[t] = z[i][lane];
        }
      }
#pragma unroll
      for (int t = 0; t < T; ++t) {
        const int i = q + 1 + u + 6 * t;
        if (i < B && (lane >= i || lane < q)) z[i][lane] = fma(-cf[t], rv, zv[t]);
      }
    }
    __syncthreads();
    if (bad_sh) break;
  }
  if (bad_sh) {
    if (threadIdx.x == 0) atomicExch(status, bad_sh);
    return;
  }
  for (int e = threadIdx.x; e < B * B; e += 8 * B) {
    const int r = e / B, cc = e - r * B, i = base + r, j = base + cc;
    if (i < n && j < n) {
      Uw[(size_t)i * n + j] = (cc > r) ? z[r][cc] : (cc == r ? udiag[r] : 0.0);
      X[(size_t)i * n + j] = (cc >= r) ? z[cc][r] : 0.0;
    }
  }
}

// rows [r0, r0 + NROW) of block (bi, bj) of a row-major n x n matrix, into s[m][c]
// (m = row - r0); rows m >= nvalid and out-of-range entries -> 0.  All loads of a
// thread are issued before its shared-memory stores.
template <int NROW>
__device__ __forceinline__ void load_rows(const double* __restrict__ M, int n, int bi, int bj, int r0,
                                          double (*s)[B + 1], int nvalid = NROW) {
  constexpr int PER = (NROW * B + RG * B - 1) / (RG * B);
  double v[PER];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int e = threadIdx.x + p * RG * B, m = e / B, cc = e - m * B, i = bi * B + r0 + m, j = bj * B + cc;
    v[p] = (e < NROW * B && m < nvalid && i < n && j < n) ? M[(size_t)i * n + j] : 0.0;
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int e = threadIdx.x + p * RG * B, m = e / B, cc = e - m * B;
    if (e < NROW * B) s[m][cc] = v[p];
  }
}

// columns [c0, c0 + RG) of block (bi, bj), transposed into t[rl][m] = M_blk[m][c0 + rl]
__device__ __forceinline__ void load_cols_t(const double* __restrict__ M, int n, int bi, int bj, int c0,
                                            double (*t)[B + 1]) {
  for (int e = threadIdx.x; e < RG * B; e += RG * B) {
    const int m = e / RG, rl = e - m * RG, i = bi * B + m, j = bj * B + c0 + rl;
    t[rl][m] = (i < n && j < n) ? M[(size_t)i * n + j] : 0.0;
  }
}

// Uw_kj = X_kk^T A_kj, block column j = k + 1 + blockIdx.x, rows RG blockIdx.y ..
__global__ void __launch_bounds__(RG * B) k_chol_panel(const double* __restrict__ S, const double* __restrict__ X,
                                                       double* __restrict__ Uw, int n, int k,
                                                       const int* __restrict__ status) {
  pdl_entry();
  __shared__ double a[B][B + 1];
  __shared__ double xt[RG][B + 1];
  const int j = k + 1 + blockIdx.x, r0 = blockIdx.y * RG;
  load_rows<B>(S, n, k, j, 0, a, r0 + RG);
  load_cols_t(X, n, k, k, r0, xt);
  __syncthreads();
  const int rl = threadIdx.x / B, c = threadIdx.x % B, r = r0 + rl;
  double s = 0.0;
  for (int m = 0; m <= r; ++m) s = fma(xt[rl][m], a[m][c], s);
  const int i = k * B + r, jj = j * B + c;
  if (failed(status)) return;  // read late: its latency overlaps the loads
  if (i < n && jj < n) Uw[(size_t)i * n + jj] = s;
}

// A_ij -= Uw_ki^T Uw_kj for k < i <= j; blockIdx.x enumerates the upper block
// triangle, blockIdx.y the row group of block row i
__global__ void __launch_bounds__(RG * B) k_chol_update(double* __restrict__ S, const double* __restrict__ Uw, int n,
                                                        int nb, int k, const int* __restrict__ status) {
  pdl_entry();
  __shared__ double uj[B][B + 1];
  __shared__ double ui[RG][B + 1];
  const int m0 = nb - k - 1;  // trailing block count
  int t = blockIdx.x, ii = 0;
  while (ii < m0 && t >= m0 - ii) {
    t -= m0 - ii;
    ++ii;
  }
  const int bi = k + 1 + ii, bj = bi + t, r0 = blockIdx.y * RG;
  load_rows<B>(Uw, n, k, bj, 0, uj);
  load_cols_t(Uw, n, k, bi, r0, ui);
  __syncthreads();
  const int rl = threadIdx.x / B, c = threadIdx.x % B, r = r0 + rl;
  double s = 0.0;
#pragma unroll 8
  for (int m = 0; m < B; ++m) s = fma(ui[rl][m], uj[m][c], s);
  const int i = bi * B + r, jj = bj * B + c;
  if (failed(status)) return;
  if (i < n && jj < n && (bi < bj || c >= r)) S[(size_t)i * n + jj] -= s;
}

// V_ik = X_ii Uw_ik for i < k, into block (i, k) of S; blockIdx.x enumerates the
// strict upper block triangle (kcol < 0) or the blocks i = blockIdx.x of block
// column k = kcol, blockIdx.y the row group
__global__ void __launch_bounds__(RG * B) k_trtri_v(double* __restrict__ S, const double* __restrict__ Uw,
                                                    const double* __restrict__ X, int n, int nb, int kcol,
                                                    const int* __restrict__ status) {
  pdl_entry();
  __shared__ double u[B][B + 1];
  __shared__ double xi[RG][B + 1];
  int t = blockIdx.x, bi = 0;
  if (kcol >= 0) {
    bi = blockIdx.x;
    t = kcol - 1 - bi;
  } else {
    while (bi < nb - 1 && t >= nb - 1 - bi) {
      t -= nb - 1 - bi;
      ++bi;
    }
  }
  const int bk = bi + 1 + t, r0 = blockIdx.y * RG;
  load_rows<B>(Uw, n, bi, bk, 0, u);
  load_rows<RG>(X, n, bi, bi, r0, xi);
  __syncthreads();
  const int rl = threadIdx.x / B, c = threadIdx.x % B, r = r0 + rl;
  double s = 0.0;
  for (int m = r; m < B; ++m) s = fma(xi[rl][m], u[m][c], s);
  const int i = bi * B + r, jj = bk * B + c;
  if (failed(status)) return;
  if (i < n && jj < n) S[(size_t)i * n + jj] = s;
}

// X_ij = -sum_{k=i+1..j} V_ik X_kj for the block diagonal j - i = d (V in S);
// i = bi0 + blockIdx.x, blockIdx.y the row group
__global__ void __launch_bounds__(RG * B) k_trtri_diag(const double* __restrict__ S, double* __restrict__ X, int n,
                                                       int d, int bi0, const int* __restrict__ status) {
  pdl_entry();
  __shared__ double xk[B][B + 1];
  __shared__ double v[RG][B + 1];
  const int bi = bi0 + blockIdx.x, bj = bi + d, r0 = blockIdx.y * RG;
  const int rl = threadIdx.x / B, c = threadIdx.x % B, r = r0 + rl;
  double acc = 0.0;
  for (int bk = bi + 1; bk <= bj; ++bk) {
    load_rows<B>(X, n, bk, bj, 0, xk);
    load_rows<RG>(S, n, bi, bk, r0, v);
    __syncthreads();
#pragma unroll 8
    for (int m = 0; m < B; ++m) acc = fma(v[rl][m], xk[m][c], acc);
    __syncthreads();
  }
  const int i = bi * B + r, jj = bj * B + c;
  if (failed(status)) return;
  if (i < n && jj < n) X[(size_t)i * n + jj] = -acc;
}

// zero the strict lower triangle of X and keep the original diagonal of S
__global__ void k_zero_lower(double* __restrict__ X, const double* __restrict__ S, double* __restrict__ diag0, int n) {
  pdl_entry();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (j < i) X[e] = 0.0;
    if (j == i) diag0[i] = S[e];
  }
}

// ---- one-CTA Cholesky and inverse in double-float arithmetic (n <= 128) ----
//
// The blocked chain above spends most of its time in the FP64 pivot chain of
// k_chol_diag (GB300 issues FP64 at 1/64 of the FP32 rate).  For the overlap
// matrices of up to 128 states one CTA does the whole job instead, in
// double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers, kept by the error-free transformations TwoSum (Knuth) and
// TwoProduct by FMA (Dekker 1971) to about 2^-46 relative per operation; two
// slots go through each packed f32x2 instruction.  Against the FP64 chain the
// orthonormality of C U^-1 goes from a few 1e-16 to a few 1e-14 at n = 128.
//
// Scaling.  D = diag(2^k_i), k_i = -floor(e_i / 2) from the binary exponent e_i
// of S_ii, puts the diagonal of A = D S D in [1, 4) and (S being SPD) every
// entry below 4 in magnitude, inside FP32's range whatever the scale of S.
// A = L L^T gives U = L^T D^-1 and X = U^-1 = D L^-T.  Splitting S_ij into
// hi + lo, the scaling and the conversion back are integer operations on the
// bit patterns (the FP64 pipe also runs the F2F conversions).
//
// Elimination.  Slot (i, q), q <= i, lives in a register of warp i mod PR, lane
// q mod 32.  It holds A_iq (the Schur complement) up to step q and Z_iq after
// it, Z the inverse of the unit lower factor of A.  Step j, with d = A_jj and
// w_i = A_ij / d for the rows i > j:
//     A_iq -= w_i A_qj  (j < q <= i),   Z_ij = -w_i,   Z_iq -= w_i Z_jq  (q < j),
// so every slot of row i subtracts w_i times entry q of one vector, row j of Z
// followed by column j of A, which the owners of those slots publish in shared
// memory at the end of step j - 1 (double-buffered: one barrier per step).
// Then L^-1 = diag(d)^-1/2 Z: X_qi = 2^k_q d_i^-1/2 Z_iq (q < i), X_ii =
// 2^k_i d_i^-1/2.  A pivot at or below 2^-40 of its row's scaled original
// diagonal stops the factorisation with status (index + 1), a NaN pivot with
// -1: the rounding an exactly dependent set of states leaves in its pivot (a
// few 2^-46 of the diagonal) stays well inside that threshold.

typedef unsigned long long u64;

struct Dfl {
  float h, l;
};

__device__ __forceinline__ u64 p2(float a, float b) {
  u64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float p2lo(u64 r) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
  return a;
}
__device__ __forceinline__ float p2hi(u64 r) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
  return b;
}
__device__ __forceinline__ u64 padd(u64 a, u64 b) {
  u64 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ u64 psub(u64 a, u64 b) {
  u64 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ u64 pmul(u64 a, u64 b) {
  u64 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ u64 pfma(u64 a, u64 b, u64 c) {
  u64 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// TwoSum: s + e = a + b exactly
__device__ __forceinline__ Dfl df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// Fast2Sum (|a| >= |b|)
__device__ __forceinline__ Dfl df_fast(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ Dfl df_mul(Dfl a, Dfl b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_fast(p, e);
}
// 1 / d: the hardware reciprocal estimate, one Newton step r + r (1 - d r) in
// FP32 and one with the residual taken in double-float (no branch, no slow path)
__device__ __forceinline__ Dfl df_rcp(Dfl d) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d.h));
  r = __fmaf_rn(r, __fmaf_rn(-d.h, r, 1.0f), r);
  float e = __fmaf_rn(-d.h, r, 1.0f);
  e = __fmaf_rn(-d.l, r, e);
  return df_fast(r, __fmul_rn(r, e));
}
// d + 1
__device__ __forceinline__ Dfl df_add1(Dfl d) {
  const Dfl s = df_two_sum(d.h, 1.0f);
  return df_fast(s.h, __fadd_rn(s.l, d.l));
}
// d^-1/2: an FP32 estimate, one Newton step y (3 - d y^2) / 2 in FP32 and one
// y + y (1 - d y^2) / 2 with d y^2 in double-float (1 - d y^2 is exact there)
__device__ __forceinline__ Dfl df_rsqrt(Dfl d) {
  float y = rsqrtf(d.h);
  y = __fmul_rn(y, __fmaf_rn(__fmul_rn(-0.5f * d.h, y), y, 1.5f));
  const float p = __fmul_rn(y, y), pe = __fmaf_rn(y, y, -p);
  const float t = __fmul_rn(d.h, p);
  float te = __fmaf_rn(d.h, p, -t);
  te = __fmaf_rn(d.h, pe, te);
  te = __fmaf_rn(d.l, p, te);
  const float e = __fsub_rn(__fsub_rn(1.0f, t), te);
  return df_fast(y, __fmul_rn(__fmul_rn(0.5f, y), e));
}

// x 2^s as hi + lo: hi the leading 24 significand bits, lo the other 29 rounded
// to 24; magnitudes below FP32's normal range give 0, NaN and infinity NaN
__device__ __forceinline__ Dfl df_of_double(double x, int s) {
  const u64 b = (u64)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int E = (int)((b >> 52) & 0x7FF);
  if (E == 0x7FF) return {__uint_as_float(0x7FC00000u), 0.0f};
  const int e = E - 1023 + s;
  if (E == 0 || e < -126) return {__uint_as_float(sign), 0.0f};
  if (e > 127) return {__uint_as_float(sign | 0x7F800000u), 0.0f};
  const u64 m = b & 0xFFFFFFFFFFFFFull;
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29));
  float lo = 0.0f;
  if (e >= -74)
    lo = __fmul_rn(__uint2float_rn((unsigned)(m & 0x1FFFFFFFull)), __uint_as_float((unsigned)(e - 52 + 127) << 23));
  return {hi, __uint_as_float(__float_as_uint(lo) | sign)};
}

// (h + l) 2^s as a double.  After TwoSum the two significands lie 24 or more
// binades apart, so their sum fits the 53 bits of a double but for bits of l
// below 2^-52 of h; FP32 subnormal parts count as 0.
__device__ __forceinline__ double df_to_double(Dfl v, int s) {
  const Dfl t = df_two_sum(v.h, v.l);
  const unsigned bh = __float_as_uint(t.h), bl = __float_as_uint(t.l);
  const int eh = (int)((bh >> 23) & 0xFF), el = (int)((bl >> 23) & 0xFF);
  if (eh == 0xFF) return __longlong_as_double(0x7FF8000000000000LL);
  if (eh == 0) return 0.0;
  long long T = (long long)((u64)(0x800000u | (bh & 0x7FFFFFu)) << 29);  // units of 2^(eh - 127 - 52)
  if (el != 0) {
    const int sh = eh - el;
    const u64 ml = (u64)(0x800000u | (bl & 0x7FFFFFu));
    const long long lv = sh <= 29 ? (long long)(ml << (29 - sh)) : (sh < 53 ? (long long)(ml >> (sh - 29)) : 0LL);
    T += ((bh ^ bl) & 0x80000000u) ? -lv : lv;
  }
  int e = eh - 127 + s;
  if (T >= (1LL << 53)) {
    T >>= 1;
    ++e;
  } else if (T < (1LL << 52)) {
    T <<= 1;
    --e;
  }
  const u64 sign = (u64)(bh & 0x80000000u) << 32;
  if (e + 1023 <= 0) return __longlong_as_double((long long)sign);
  if (e + 1023 >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sign | ((u64)(e + 1023) << 52) | ((u64)T & 0xFFFFFFFFFFFFFull)));
}

// S row-major n x n (upper part used), X = U^-1 row-major, zero below the
// diagonal; NMAX / PR rows per warp, lanes over columns in pairs of 32-column
// blocks (q, q + 32) packed into one f32x2 register pair (hi parts, lo parts).
// The loops over the slots carry explicit unroll counts: without them the
// 128-state instance kept the slot arrays in local memory.
template <int NMAX, int PR>
__global__ void __launch_bounds__(32 * PR) k_chol_df(const double* __restrict__ S, double* __restrict__ X, int n,
                                                     int* __restrict__ status) {
  constexpr int RA = NMAX / PR, NP = NMAX / 64;
  static_assert(NMAX % 64 == 0 && NMAX % PR == 0, "layout");
  pdl_entry();
  __shared__ float2 buf[2][NMAX];  // the broadcast vector of the step (double-buffered)
  __shared__ float2 piv[NMAX];     // the pivots d_j
  __shared__ float thr[NMAX];      // 2^-40 of the scaled original diagonal
  __shared__ int kx[NMAX];         // k_i
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (failed(status)) return;
  for (int t = threadIdx.x; t < NMAX; t += 32 * PR) {
    int k = 0;
    if (t < n) {
      const int E = (int)((__double_as_longlong(S[(size_t)t * n + t]) >> 52) & 0x7FF);
      if (E != 0 && E != 0x7FF) k = -((E - 1023) >> 1);
    }
    kx[t] = k;
    buf[0][t] = buf[1][t] = make_float2(0.0f, 0.0f);
    thr[t] = 0.0f;
  }
  __syncthreads();
  u64 H[RA][NP], L[RA][NP];  // slots (i, q) and (i, q + 32): i = w + PR a, q = lane + 64 p
#pragma unroll 16
  for (int a = 0; a < RA; ++a) {
    const int i = w + PR * a;
#pragma unroll 16
    for (int p = 0; p < NP; ++p) {
      const int q0 = lane + 64 * p, q1 = q0 + 32;
      Dfl v0 = {0.0f, 0.0f}, v1 = {0.0f, 0.0f};
      if (i < n && q0 <= i) v0 = df_of_double(S[(size_t)q0 * n + i], kx[i] + kx[q0]);
      if (i < n && q1 <= i) v1 = df_of_double(S[(size_t)q1 * n + i], kx[i] + kx[q1]);
      H[a][p] = p2(v0.h, v1.h);
      L[a][p] = p2(v0.l, v1.l);
      if (i < n) {
        if (q0 == i) thr[i] = 0x1p-40f * v0.h;
        if (q1 == i) thr[i] = 0x1p-40f * v1.h;
        if (q0 == 0) buf[0][i] = make_float2(v0.h, v0.l);  // column 0, the first pivot included
      }
    }
  }
  for (int j = 0; j < n; ++j) {
    __syncthreads();
    const float2* b = buf[j & 1];
    float2* bn = buf[(j + 1) & 1];
    const float2 dv = b[j];
    if (!(dv.x > thr[j])) {  // every thread reads the same pivot: a uniform exit
      if (threadIdx.x == 0) atomicExch(status, dv.x != dv.x ? -1 : j + 1);
      return;
    }
    if (threadIdx.x == 0) piv[j] = dv;
    const Dfl rd = df_rcp({dv.x, dv.y});
    // entry j of the vector is d + 1: the generic update then turns A_ij = w_i d into
    // -w_i = Z_ij, and rows i <= j get w = 0, an exact no-op, so that all rows of a
    // warp update in one branch-free block (a row has slots in pair p only when
    // PR a >= 64 p, known at compile time)
    u64 vh[NP], vl[NP];
#pragma unroll 16
    for (int p = 0; p < NP; ++p) {
      float2 x0 = b[lane + 64 * p], x1 = b[lane + 64 * p + 32];
      if (lane == (j & 31) && (j >> 6) == p) {
        const Dfl d1 = df_add1({dv.x, dv.y});
        if (j & 32)
          x1 = make_float2(d1.h, d1.l);
        else
          x0 = make_float2(d1.h, d1.l);
      }
      vh[p] = p2(x0.x, x1.x);
      vl[p] = p2(x0.y, x1.y);
    }
    u64 wh[RA], wl[RA], nwh[RA];
#pragma unroll 16
    for (int a = 0; a < RA; ++a) {
      const int i = w + PR * a;
      const float2 bi = b[i];
      Dfl wi = df_mul({bi.x, bi.y}, rd);
      if (!(i > j && i < n)) wi = {0.0f, 0.0f};
      wh[a] = p2(wi.h, wi.h);
      wl[a] = p2(wi.l, wi.l);
      nwh[a] = p2(-wi.h, -wi.h);
    }
#pragma unroll 16
    for (int a = 0; a < RA; ++a) {
#pragma unroll 16
      for (int p = 0; p < NP; ++p) {
        if (64 * p <= PR * a) {
          // (H, L) -= w v: TwoProduct of the hi parts, TwoSum into H, the rest into L
          const u64 np = pmul(nwh[a], vh[p]);
          u64 pe = pfma(wh[a], vh[p], np);
          pe = pfma(wh[a], vl[p], pe);
          pe = pfma(wl[a], vh[p], pe);
          const u64 s = padd(H[a][p], np);
          const u64 bb = psub(s, H[a][p]);
          const u64 e = padd(psub(H[a][p], psub(s, bb)), psub(np, bb));
          H[a][p] = s;
          L[a][p] = padd(e, psub(L[a][p], pe));
        }
      }
    }
    if (j & 1) {  // renormalise every second step: the lo parts' own rounding stays at 2^-48 of hi
#pragma unroll 16
      for (int a = 0; a < RA; ++a)
#pragma unroll 16
        for (int p = 0; p < NP; ++p)
          if (64 * p <= PR * a) {
            const u64 s2 = padd(H[a][p], L[a][p]);
            const u64 b2 = psub(s2, H[a][p]);
            L[a][p] = padd(psub(H[a][p], psub(s2, b2)), psub(L[a][p], b2));
            H[a][p] = s2;
          }
    }
    // the vector of step j + 1: row j + 1 (Z part and pivot) from its warp, column
    // j + 1 from lane (j + 1) mod 32 of every warp
    const int j1 = j + 1;
    if (w == j1 % PR) {
#pragma unroll 16
      for (int a = 0; a < RA; ++a) {
        if (w + PR * a == j1) {
#pragma unroll 16
          for (int p = 0; p < NP; ++p) {
            const int q0 = lane + 64 * p;
            if (q0 <= j1) {
              const Dfl t = df_two_sum(p2lo(H[a][p]), p2lo(L[a][p]));
              bn[q0] = make_float2(t.h, t.l);
            }
            if (q0 + 32 <= j1) {
              const Dfl t = df_two_sum(p2hi(H[a][p]), p2hi(L[a][p]));
              bn[q0 + 32] = make_float2(t.h, t.l);
            }
          }
        }
      }
    }
    if (lane == (j1 & 31)) {
      const bool up = (j1 & 32) != 0;
#pragma unroll 16
      for (int a = 0; a < RA; ++a) {
        const int i = w + PR * a;
#pragma unroll 16
        for (int p = 0; p < NP; ++p) {
          if (64 * p <= PR * a && (j1 >> 6) == p && i > j1 && i < n) {
            const Dfl t = df_two_sum(up ? p2hi(H[a][p]) : p2lo(H[a][p]), up ? p2hi(L[a][p]) : p2lo(L[a][p]));
            bn[i] = make_float2(t.h, t.l);
          }
        }
      }
    }
  }
  __syncthreads();
  // X_qi = 2^k_q d_i^-1/2 Z_iq (q < i), X_ii = 2^k_i d_i^-1/2, zero below the diagonal
#pragma unroll 16
  for (int a = 0; a < RA; ++a) {
    const int i = w + PR * a;
    if (i < n) {
      const float2 pv = piv[i];
      const Dfl ri = df_rsqrt({pv.x, pv.y});
#pragma unroll 16
      for (int p = 0; p < NP; ++p) {
#pragma unroll 16
        for (int hf = 0; hf < 2; ++hf) {
          const int q = lane + 64 * p + 32 * hf;
          if (q == i) {
            X[(size_t)i * n + i] = df_to_double(ri, kx[i]);
          } else if (q < i) {
            const Dfl z = df_two_sum(hf ? p2hi(H[a][p]) : p2lo(H[a][p]), hf ? p2hi(L[a][p]) : p2lo(L[a][p]));
            X[(size_t)q * n + i] = df_to_double(df_mul(z, ri), kx[q]);
            X[(size_t)i * n + q] = 0.0;
          }
        }
      }
    }
  }
}

// ---- lean double-float elimination: one CTA, up to MMAX = 32 or 64 rows ----
//
// The elimination of k_chol_df with less work per step.  The vector of step j
// (row j of Z, the pivot d, column j of A) is scaled once per lane, u_q = v_q / d,
// with u_j = 1 + 1/d at the pivot entry; every slot (i, q) of an active row
// i > j then subtracts b_i u_q, b_i = A_ij taken from the same vector:
//     A_iq - A_ij A_qj / d   (q > j),   A_ij - A_ij (1 + 1/d) = -A_ij / d = Z_ij,
//     Z_iq - (A_ij / d) Z_jq (q < j).
// Finished rows (i <= j) are skipped by warp-uniform branches, 32-column blocks
// wholly above a warp's rows at compile time, and each update is one 15-operation
// double-float multiply-subtract, renormalised in place.  Serves the whole matrix
// up to MMAX states (diag0 == nullptr: thresholds from its own scaled diagonal) and
// the 32 x 32 diagonal blocks of the blocked chain (base = 32 k, the block's
// current Schur complement in S, thresholds from the original diagonal diag0);
// writes the (diagonal block of) X = U^-1, zero below its diagonal.

// m - b u: TwoProduct of the hi parts by FMA, TwoSum into hi, the low-order terms
// into lo, then Fast2Sum
__device__ __forceinline__ Dfl df_fms(Dfl m, Dfl b, Dfl u) {
  const float p = __fmul_rn(b.h, u.h);
  float pe = __fmaf_rn(b.h, u.h, -p);
  pe = __fmaf_rn(b.h, u.l, pe);
  pe = __fmaf_rn(b.l, u.h, pe);
  const float s = __fsub_rn(m.h, p);
  const float bb = __fsub_rn(s, m.h);
  const float e = __fsub_rn(__fsub_rn(m.h, __fsub_rn(s, bb)), __fadd_rn(p, bb));
  const float l = __fadd_rn(e, __fsub_rn(m.l, pe));
  const float h = __fadd_rn(s, l);
  return {h, __fsub_rn(l, __fsub_rn(h, s))};
}

template <int MMAX, int NW>
__global__ void __launch_bounds__(32 * NW) k_chol_lean(const double* __restrict__ S, double* __restrict__ X,
                                                      const double* __restrict__ diag0, int n, int base,
                                                      int* __restrict__ status) {
  constexpr int RA = MMAX / NW, NP = MMAX / 32;
  static_assert(MMAX % 32 == 0 && MMAX % NW == 0 && NW <= 32, "layout");
  pdl_entry();
  __shared__ float2 buf[2][MMAX];  // the vector of the step (double-buffered)
  __shared__ float2 piv[MMAX];     // the pivots d_j
  __shared__ float thr[MMAX];      // 2^-40 of the scaled original diagonal
  __shared__ int kx[MMAX];         // k_i: A = D S D, D = diag(2^k_i)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int m = min(MMAX, n - base);
  if (failed(status)) return;
  for (int t = threadIdx.x; t < MMAX; t += 32 * NW) {
    int k = 0;
    float th = 0.0f;
    if (t < m) {
      const int E = (int)((__double_as_longlong(S[(size_t)(base + t) * n + base + t]) >> 52) & 0x7FF);
      if (E != 0 && E != 0x7FF) k = -((E - 1023) >> 1);
      if (diag0) th = 0x1p-40f * df_of_double(diag0[base + t], 2 * k).h;
    }
    kx[t] = k;
    thr[t] = th;
    buf[0][t] = buf[1][t] = make_float2(0.0f, 0.0f);
  }
  __syncthreads();
  Dfl M[RA][NP];  // slot (i, q): i = w + NW a, q = lane + 32 p
#pragma unroll
  for (int a = 0; a < RA; ++a) {
    const int i = w + NW * a;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const int q = lane + 32 * p;
      M[a][p] = {0.0f, 0.0f};
      if (i < m && q <= i) {
        M[a][p] = df_of_double(S[(size_t)(base + q) * n + base + i], kx[i] + kx[q]);
        if (q == 0) buf[0][i] = make_float2(M[a][p].h, M[a][p].l);  // column 0, the first pivot included
        if (q == i && !diag0) thr[i] = 0x1p-40f * M[a][p].h;
      }
    }
  }
  for (int j = 0; j < m; ++j) {
    __syncthreads();
    const float2* b = buf[j & 1];
    float2* bn = buf[(j + 1) & 1];
    const float2 dv = b[j];
    if (!(dv.x > thr[j])) {  // the same pivot in every thread: a uniform exit
      if (threadIdx.x == 0) atomicExch(status, dv.x != dv.x ? -1 : base + j + 1);
      return;
    }
    if (threadIdx.x == 0) piv[j] = dv;
    const Dfl rd = df_rcp({dv.x, dv.y});
    Dfl u[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const int q = lane + 32 * p;
      const float2 x = b[q];
      u[p] = (q == j) ? df_add1(rd) : df_mul({x.x, x.y}, rd);
    }
#pragma unroll
    for (int a = 0; a < RA; ++a) {
      const int i = w + NW * a;
      if (i > j && i < m) {  // warp-uniform
        const float2 bi = b[i];
#pragma unroll
        for (int p = 0; p < NP; ++p)
          if (32 * p <= NW * a + NW - 1) M[a][p] = df_fms(M[a][p], {bi.x, bi.y}, u[p]);
      }
    }
    // the vector of step j + 1: row j + 1 (Z part and pivot) from its warp, column
    // j + 1 below the diagonal from lane (j + 1) mod 32 of every warp
    const int j1 = j + 1;
    if (j1 < m) {
      if (w == j1 % NW) {
        const int a1 = j1 / NW;
#pragma unroll
        for (int a = 0; a < RA; ++a)
          if (a == a1) {
#pragma unroll
            for (int p = 0; p < NP; ++p)
              if (lane + 32 * p <= j1) bn[lane + 32 * p] = make_float2(M[a][p].h, M[a][p].l);
          }
      }
      if (lane == (j1 & 31)) {
        const int p1 = j1 >> 5;
#pragma unroll
        for (int a = 0; a < RA; ++a) {
          const int i = w + NW * a;
          if (i > j1 && i < m) {
            Dfl v = M[a][0];
#pragma unroll
            for (int p = 1; p < NP; ++p)
              if (p == p1) v = M[a][p];
            bn[i] = make_float2(v.h, v.l);
          }
        }
      }
    }
  }
  __syncthreads();
  // X_qi = 2^k_q d_i^-1/2 Z_iq (q < i), X_ii = 2^k_i d_i^-1/2, zero below the diagonal
  double* xb = X + (size_t)base * n + base;
#pragma unroll
  for (int a = 0; a < RA; ++a) {
    const int i = w + NW * a;
    if (i < m) {
      const float2 pv = piv[i];
      const Dfl ri = df_rsqrt({pv.x, pv.y});
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const int q = lane + 32 * p;
        if (q == i) {
          xb[(size_t)i * n + i] = df_to_double(ri, kx[i]);
        } else if (q < i) {
          xb[(size_t)q * n + i] = df_to_double(df_mul(M[a][p], ri), kx[q]);
          xb[(size_t)i * n + q] = 0.0;
        }
      }
    }
  }
}

}  // namespace

// Queue U = chol(S) and X = U^{-1}; no synchronisation.  S is overwritten (the
// blocked FP64 chain) or left as it was (the one-CTA double-float kernel).
int chol_inverse(Ctx& c, double* S, double* X, int n) {
  // double-float: the whole job in one CTA up to 64 states (k_chol_lean), the
  // diagonal blocks of the blocked chain above (one CTA for all 128 states, option
  // 3, is slower than the chain)
  const bool df = c.chol_df >= 2 || (c.chol_df == 1 && c.precision == 1);
  if (c.chol_df == 3 && n <= 128) {
    ProfScope ps_(c, "k_chol_df");
    GBCP_LAUNCH_PDL(c, (k_chol_df<128, 16>), dim3(1), dim3(512), 0, (const double*)S, X, n, c.d_info);
    return 0;
  }
  if (df && n <= 64) {
    ProfScope ps_(c, "k_chol_df");
    if (n <= 32)
      GBCP_LAUNCH_PDL(c, (k_chol_lean<32, 8>), dim3(1), dim3(256), 0, (const double*)S, X, (const double*)nullptr, n,
                      0, c.d_info);
    else
      GBCP_LAUNCH_PDL(c, (k_chol_lean<64, 8>), dim3(1), dim3(256), 0, (const double*)S, X, (const double*)nullptr, n,
                      0, c.d_info);
    return 0;
  }
  const int nb = (n + B - 1) / B;
  if (!ensure(c, c.cdiag, sizeof(double) * (size_t)n)) return 6;
  if (!ensure(c, c.cwork, sizeof(double) * (size_t)n * n)) return 6;
  double* diag0 = static_cast<double*>(c.cdiag.p);
  double* Uw = static_cast<double*>(c.cwork.p);
  const dim3 blk(RG * B);
  {
    ProfScope ps_(c, "k_chol_misc");
    GBCP_LAUNCH_PDL(c, k_zero_lower, dim3(std::max(1, std::min(256, (n * n + 255) / 256))), dim3(256), 0, X,
                    (const double*)S, diag0, n);
  }
  for (int k = 0; k < nb; ++k) {
    if (df) {
      ProfScope ps_(c, "k_chol_diag");
      GBCP_LAUNCH_PDL(c, (k_chol_lean<B, 8>), dim3(1), dim3(8 * B), 0, (const double*)S, X, (const double*)diag0, n,
                      k * B, c.d_info);
    } else {
      ProfScope ps_(c, "k_chol_diag");
      GBCP_LAUNCH_PDL(c, k_chol_diag, dim3(1), dim3(8 * B), 0, (const double*)S, Uw, X, (const double*)diag0, n, k,
                      c.d_info);
    }
    const int m0 = nb - k - 1;
    if (m0 > 0) {
      {
        ProfScope ps_(c, "k_chol_panel");
        GBCP_LAUNCH_PDL(c, k_chol_panel, dim3(m0, B / RG), blk, 0, (const double*)S, (const double*)X, Uw, n, k,
                        (const int*)c.d_info);
      }
      {
        ProfScope ps_(c, "k_chol_update");
        GBCP_LAUNCH_PDL(c, k_chol_update, dim3(m0 * (m0 + 1) / 2, B / RG), blk, 0, S, (const double*)Uw, n, nb, k,
                        (const int*)c.d_info);
      }
    }
  }
  if (nb > 1) {
    ProfScope ps_(c, "k_trtri_v");
    GBCP_LAUNCH_PDL(c, k_trtri_v, dim3(nb * (nb - 1) / 2, B / RG), blk, 0, S, (const double*)Uw, (const double*)X, n,
                    nb, -1, (const int*)c.d_info);
  }
  for (int d = 1; d < nb; ++d) {
    ProfScope ps_(c, "k_trtri_diag");
    GBCP_LAUNCH_PDL(c, k_trtri_diag, dim3(nb - d, B / RG), blk, 0, (const double*)S, X, n, d, 0, (const int*)c.d_info);
  }
  return 0;
}

// The blocked chain with X = U^{-1} finished column block by column block, for the
// host-memory Gram-Schmidt, whose C U^{-1} and download then start one column block
// at a time while the factorisation goes on.  On the context stream, per block k:
// the diagonal factor; V_ik = X_ii U_ik (i < k) into S and X_ik for i = k-1 .. 0
// (the block diagonals of chol_inverse restricted to column k, in the same order);
// then column(k) is queued on the side stream (the context's stream set to it
// meanwhile) and the panel and update follow on the context stream.  Element by
// element the arithmetic of chol_inverse: S blocks (i, k), i < k, are no longer read
// by the factorisation once diagonal block k is done.  Returns with the context
// stream waiting for the side stream; 7 if the chain does not apply (one block, or
// above 8 x 8 blocks).
int chol_inverse_columns(Ctx& c, double* S, double* X, int n, const std::function<int(int)>& column) {
  const int nb = (n + B - 1) / B;
  if (nb < 2 || nb > 8) return 7;
  const bool df = c.chol_df >= 2 || (c.chol_df == 1 && c.precision == 1);
  if (!ensure(c, c.cdiag, sizeof(double) * (size_t)n)) return 6;
  if (!ensure(c, c.cwork, sizeof(double) * (size_t)n * n)) return 6;
  if (!c.side && cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking) != cudaSuccess) {
    c.err = "side stream";
    return 5;
  }
  while (c.col_ev.size() < (size_t)nb + 1) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      c.err = "events";
      return 5;
    }
    c.col_ev.push_back(e);
  }
  double* diag0 = static_cast<double*>(c.cdiag.p);
  double* Uw = static_cast<double*>(c.cwork.p);
  const dim3 blk(RG * B);
  cudaStream_t main = c.stream;
  int rc = 0;
  {
    ProfScope ps_(c, "k_chol_misc");
    GBCP_LAUNCH_PDL(c, k_zero_lower, dim3(std::max(1, std::min(256, (n * n + 255) / 256))), dim3(256), 0, X,
                    (const double*)S, diag0, n);
  }
  for (int k = 0; k < nb && !rc; ++k) {
    if (df) {
      ProfScope ps_(c, "k_chol_diag");
      GBCP_LAUNCH_PDL(c, (k_chol_lean<B, 8>), dim3(1), dim3(8 * B), 0, (const double*)S, X, (const double*)diag0, n,
                      k * B, c.d_info);
    } else {
      ProfScope ps_(c, "k_chol_diag");
      GBCP_LAUNCH_PDL(c, k_chol_diag, dim3(1), dim3(8 * B), 0, (const double*)S, Uw, X, (const double*)diag0, n, k,
                      c.d_info);
    }
    // column block k of X: V_ik = X_ii U_ik (i < k), then X_ik for i = k-1 .. 0
    if (k > 0) {
      {
        ProfScope ps_(c, "k_trtri_v");
        GBCP_LAUNCH_PDL(c, k_trtri_v, dim3(k, B / RG), blk, 0, S, (const double*)Uw, (const double*)X, n, nb, k,
                        (const int*)c.d_info);
      }
      for (int d = 1; d <= k; ++d) {
        ProfScope ps_(c, "k_trtri_diag");
        GBCP_LAUNCH_PDL(c, k_trtri_diag, dim3(1, B / RG), blk, 0, (const double*)S, X, n, d, k - d,
                        (const int*)c.d_info);
      }
    }
    GBCP_CUDA_TRY(c, cudaEventRecord(c.col_ev[k], main));
    GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.side, c.col_ev[k], 0));
    c.stream = c.side;
    rc = column(k);
    c.stream = main;
    if (rc) break;
    const int m0 = nb - k - 1;
    if (m0 > 0) {
      {
        ProfScope ps_(c, "k_chol_panel");
        GBCP_LAUNCH_PDL(c, k_chol_panel, dim3(m0, B / RG), blk, 0, (const double*)S, (const double*)X, Uw, n, k,
                        (const int*)c.d_info);
      }
      {
        ProfScope ps_(c, "k_chol_update");
        GBCP_LAUNCH_PDL(c, k_chol_update, dim3(m0 * (m0 + 1) / 2, B / RG), blk, 0, S, (const double*)Uw, n, nb, k,
                        (const int*)c.d_info);
      }
    }
  }
  c.stream = main;
  // the context stream waits for the side branches (also after an error)
  if (cudaEventRecord(c.col_ev[nb], c.side) == cudaSuccess) cudaStreamWaitEvent(main, c.col_ev[nb], 0);
  return rc;
}

}  // namespace gbcp
