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
// strict upper block triangle, blockIdx.y the row group
__global__ void __launch_bounds__(RG * B) k_trtri_v(double* __restrict__ S, const double* __restrict__ Uw,
                                                    const double* __restrict__ X, int n, int nb,
                                                    const int* __restrict__ status) {
  pdl_entry();
  __shared__ double u[B][B + 1];
  __shared__ double xi[RG][B + 1];
  int t = blockIdx.x, bi = 0;
  while (bi < nb - 1 && t >= nb - 1 - bi) {
    t -= nb - 1 - bi;
    ++bi;
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
// blockIdx.x = i, blockIdx.y the row group
__global__ void __launch_bounds__(RG * B) k_trtri_diag(const double* __restrict__ S, double* __restrict__ X, int n,
                                                       int d, const int* __restrict__ status) {
  pdl_entry();
  __shared__ double xk[B][B + 1];
  __shared__ double v[RG][B + 1];
  const int bi = blockIdx.x, bj = bi + d, r0 = blockIdx.y * RG;
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

}  // namespace

// Queue U = chol(S) and X = U^{-1}; no synchronisation.  S is overwritten.
int chol_inverse(Ctx& c, double* S, double* X, int n) {
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
    {
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
                    nb, (const int*)c.d_info);
  }
  for (int d = 1; d < nb; ++d) {
    ProfScope ps_(c, "k_trtri_diag");
    GBCP_LAUNCH_PDL(c, k_trtri_diag, dim3(nb - d, B / RG), blk, 0, (const double*)S, X, n, d, (const int*)c.d_info);
  }
  return 0;
}

}  // namespace gbcp
