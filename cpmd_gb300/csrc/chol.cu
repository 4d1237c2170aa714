// Blocked Cholesky factorisation S = U^T U and triangular inverse X = U^{-1}
// of the overlap matrix (the reference's uinv: dpotrf + dtrtri,
// rgs_utils.mod.F90:95-162), spread over many CTAs.
//
// 32 x 32 blocks, right-looking:
//   for each diagonal block k:
//     diag   one CTA of four warps factors A_kk = U_kk^T U_kk and inverts U_kk
//     panel  U_kj = U_kk^{-T} A_kj for every block j > k (one CTA per block)
//     update A_ij -= U_ki^T U_kj for k < i <= j (one CTA per block)
//   then X block-diagonal by block-diagonal: X_ii = U_ii^{-1} (from diag) and
//   X_ij = -U_ii^{-1} sum_{k=i+1..j} U_ik X_kj for j - i = 1, 2, ...
// Every kernel first reads the ortho status word and does nothing once a step
// has failed; diag sets it to (global pivot index + 1) at a pivot at or below
// 64 eps of that row's original diagonal (an exactly dependent set of states,
// where dpotrf's info > 0 would depend on rounding) and to -1 at a NaN.  S is row-major n x n (symmetric, upper part used and
// overwritten by U); X is row-major n x n, upper triangular, zero below.
#include <algorithm>

#include "ctx.h"

namespace gbcp {

namespace {

constexpr int B = 32;

__device__ __forceinline__ bool failed(const int* status) { return *(volatile const int*)status != 0; }

// load block (bi, bj) of a row-major n x n matrix into s[32][33]; out-of-range -> pad
__device__ __forceinline__ void load_block(const double* __restrict__ M, int n, int bi, int bj, double (*s)[B + 1],
                                           double pad_diag) {
  const int r = threadIdx.x / B, c = threadIdx.x % B;
  const int i = bi * B + r, j = bj * B + c;
  double v = 0.0;
  if (i < n && j < n) v = M[(size_t)i * n + j];
  else if (r == c) v = pad_diag;
  s[r][c] = v;
}

__device__ __forceinline__ void store_block(double* __restrict__ M, int n, int bi, int bj, const double (*s)[B + 1]) {
  const int r = threadIdx.x / B, c = threadIdx.x % B;
  const int i = bi * B + r, j = bj * B + c;
  if (i < n && j < n) M[(size_t)i * n + j] = s[r][c];
}

// Factor + invert the diagonal block k: U_kk -> S (upper), U_kk^{-1} -> X
// (diagonal block).  On GB300 the FP64 pipe (about 2 FMAs per clock per SM)
// bounds this small kernel, so its work is spread over the four warps of one CTA,
// one per SM sub-partition.
//   factor: lane c owns column c, warp w the rows r = w (mod 4) of it (8 values in
//           registers); the owner of pivot row p publishes the row in shared
//           memory, one barrier per step;
//   invert: column j of U^{-1} is independent of the others: warp w takes columns
//           j = w (mod 4); w[i] = -(sum_{m>i} U[i][m] w[m]) / U[i][i] with the dot
//           product split over the lanes and a shuffle reduction.
__global__ void __launch_bounds__(4 * B) k_chol_diag(double* __restrict__ S, double* __restrict__ X,
                                                     const double* __restrict__ diag0, int n, int k,
                                                     int* __restrict__ status) {
  __shared__ double u[B][B + 1];  // U (upper), row p published at step p
  __shared__ double dinv[B];
  __shared__ int bad_sh;
  if (failed(status)) return;
  const int c = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = k * B + c;
  constexpr int R = B / 4;
  double col[R];  // rows r = w + 4 q of column c
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int r = w + 4 * q, i = k * B + r;
    col[q] = (i < n && j < n) ? S[(size_t)i * n + j] : (r == c ? 1.0 : 0.0);
  }
  if (threadIdx.x == 0) bad_sh = 0;
  __syncthreads();
#pragma unroll
  for (int p = 0; p < B; ++p) {
    const int pw = p & 3, pq = p >> 2;
    if (w == pw) {  // owner of row p: pivot, row p of U
      const double d = __shfl_sync(0xffffffffu, col[pq], p);
      const double d0 = (k * B + p < n) ? diag0[k * B + p] : 1.0;
      if (!(d > 0x1p-46 * d0)) {
        if (c == 0) bad_sh = (d != d) ? -1 : k * B + p + 1;
      } else {
        const double inv = rsqrt(d);
        const double upc = (c == p) ? d * inv : (c > p ? col[pq] * inv : 0.0);
        col[pq] = upc;
        u[p][c] = upc;
        if (c == p) dinv[p] = inv;
      }
    }
    __syncthreads();
    if (bad_sh) break;
    const double upc = u[p][c];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int r = w + 4 * q;
      if (r > p && r <= c) col[q] = fma(-u[p][r], upc, col[q]);
    }
  }
  if (bad_sh) {
    if (threadIdx.x == 0) atomicExch(status, bad_sh);
    return;
  }
  // U rows below the diagonal are zero; store U
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int r = w + 4 * q, i = k * B + r;
    if (r > c) u[r][c] = 0.0;
    if (i < n && j < n) S[(size_t)i * n + j] = u[r][c];
  }
  __syncthreads();
  // invert by 2 x 2 blocks of 16: W11 = U11^-1 and W22 = U22^-1 (warps 0 and 1, lane = column,
  // uniform back-substitution with broadcast reads of U), then W12 = -W11 (U12 W22)
  constexpr int H = B / 2;
  __shared__ double wt[B][B + 1];
  __shared__ double tt[H][H + 1];
  if (w < 2 && c < H) {
    const int o = w * H;  // block offset
    double wc[H];
#pragma unroll
    for (int i = H - 1; i >= 0; --i) {
      double t = 0.0;
#pragma unroll
      for (int m = i + 1; m < H; ++m) t = fma(u[o + i][o + m], wc[m], t);
      const double di = dinv[o + i];
      wc[i] = (i == c) ? di : (i < c ? -t * di : 0.0);
    }
#pragma unroll
    for (int i = 0; i < H; ++i) wt[o + i][o + c] = wc[i];
  }
  __syncthreads();
  {  // T = U12 W22 (16 x 16), two outputs per thread
    const int e = threadIdx.x, r = e >> 3, c0 = (e & 7) * 2;
    double t0 = 0.0, t1 = 0.0;
#pragma unroll
    for (int m = 0; m < H; ++m) {
      t0 = fma(u[r][H + m], wt[H + m][H + c0], t0);
      t1 = fma(u[r][H + m], wt[H + m][H + c0 + 1], t1);
    }
    tt[r][c0] = t0;
    tt[r][c0 + 1] = t1;
  }
  __syncthreads();
  {  // W12 = -W11 T; lower-left block zero
    const int e = threadIdx.x, r = e >> 3, c0 = (e & 7) * 2;
    double t0 = 0.0, t1 = 0.0;
#pragma unroll
    for (int m = 0; m < H; ++m) {
      t0 = fma(wt[r][m], tt[m][c0], t0);
      t1 = fma(wt[r][m], tt[m][c0 + 1], t1);
    }
    wt[r][H + c0] = -t0;
    wt[r][H + c0 + 1] = -t1;
    wt[H + r][c0] = 0.0;
    wt[H + r][c0 + 1] = 0.0;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int r = w + 4 * q, i = k * B + r;
    if (i < n && j < n) X[(size_t)i * n + j] = wt[r][c];
  }
}

// U_kj = (U_kk^{-1})^T A_kj for block column j = k + 1 + blockIdx.x
__global__ void __launch_bounds__(1024) k_chol_panel(double* __restrict__ S, const double* __restrict__ X, int n,
                                                     int k, int* __restrict__ status) {
  __shared__ double ui[B][B + 1];
  __shared__ double a[B][B + 1];
  if (failed(status)) return;
  const int j = k + 1 + blockIdx.x;
  load_block(X, n, k, k, ui, 0.0);
  load_block(S, n, k, j, a, 0.0);
  __syncthreads();
  const int r = threadIdx.x / B, c = threadIdx.x % B;
  double s = 0.0;
#pragma unroll 8
  for (int m = 0; m <= r; ++m) s = fma(ui[m][r], a[m][c], s);
  __syncthreads();
  a[r][c] = s;
  __syncthreads();
  store_block(S, n, k, j, a);
}

// A_ij -= U_ki^T U_kj for k < i <= j; blockIdx.x enumerates the upper block triangle
__global__ void __launch_bounds__(1024) k_chol_update(double* __restrict__ S, int n, int nb, int k,
                                                      int* __restrict__ status) {
  __shared__ double ui[B][B + 1];
  __shared__ double uj[B][B + 1];
  if (failed(status)) return;
  const int m0 = nb - k - 1;  // trailing block count
  int t = blockIdx.x, ii = 0;
  while (ii < m0 && t >= m0 - ii) {
    t -= m0 - ii;
    ++ii;
  }
  const int bi = k + 1 + ii, bj = bi + t;
  load_block(S, n, k, bi, ui, 0.0);
  load_block(S, n, k, bj, uj, 0.0);
  __syncthreads();
  const int r = threadIdx.x / B, c = threadIdx.x % B;
  double s = 0.0;
#pragma unroll 8
  for (int m = 0; m < B; ++m) s = fma(ui[m][r], uj[m][c], s);
  const int i = bi * B + r, jj = bj * B + c;
  if (i < n && jj < n && (bi < bj || c >= r)) S[(size_t)i * n + jj] -= s;
}

// X_ij = -U_ii^{-1} sum_{k=i+1..j} U_ik X_kj for the block diagonal j - i = d
__global__ void __launch_bounds__(1024) k_trtri_diag(const double* __restrict__ S, double* __restrict__ X, int n,
                                                     int d, const int* __restrict__ status) {
  __shared__ double u[B][B + 1];
  __shared__ double x[B][B + 1];
  __shared__ double t[B][B + 1];
  if (failed(status)) return;
  const int bi = blockIdx.x, bj = bi + d;
  const int r = threadIdx.x / B, c = threadIdx.x % B;
  double acc = 0.0;
  for (int bk = bi + 1; bk <= bj; ++bk) {
    load_block(S, n, bi, bk, u, 0.0);
    load_block(X, n, bk, bj, x, 0.0);
    __syncthreads();
#pragma unroll 8
    for (int m = 0; m < B; ++m) acc = fma(u[r][m], x[m][c], acc);
    __syncthreads();
  }
  t[r][c] = acc;
  load_block(X, n, bi, bi, u, 0.0);  // U_ii^{-1}
  __syncthreads();
  double s = 0.0;
#pragma unroll 8
  for (int m = 0; m < B; ++m) s = fma(u[r][m], t[m][c], s);
  x[r][c] = -s;
  __syncthreads();
  store_block(X, n, bi, bj, x);
}

// zero the strict lower triangle of X and keep the original diagonal of S
__global__ void k_zero_lower(double* __restrict__ X, const double* __restrict__ S, double* __restrict__ diag0, int n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (j < i) X[e] = 0.0;
    if (j == i) diag0[i] = S[e];
  }
}

}  // namespace

// Queue U = chol(S) (in place, upper) and X = U^{-1}; no synchronisation.
int chol_inverse(Ctx& c, double* S, double* X, int n) {
  const int nb = (n + B - 1) / B;
  if (!ensure(c, c.cdiag, sizeof(double) * (size_t)n)) return 6;
  double* diag0 = static_cast<double*>(c.cdiag.p);
  {
    ProfScope ps_(c, "k_chol_misc");
    k_zero_lower<<<std::max(1, std::min(256, (n * n + 255) / 256)), 256, 0, c.stream>>>(X, S, diag0, n);
    GBCP_LAUNCH_CHECK(c);
  }
  for (int k = 0; k < nb; ++k) {
    {
      ProfScope ps_(c, "k_chol_diag");
      k_chol_diag<<<1, 4 * B, 0, c.stream>>>(S, X, diag0, n, k, c.d_info);
      GBCP_LAUNCH_CHECK(c);
    }
    const int m0 = nb - k - 1;
    if (m0 > 0) {
      {
        ProfScope ps_(c, "k_chol_panel");
        k_chol_panel<<<m0, B * B, 0, c.stream>>>(S, X, n, k, c.d_info);
        GBCP_LAUNCH_CHECK(c);
      }
      {
        ProfScope ps_(c, "k_chol_update");
        k_chol_update<<<m0 * (m0 + 1) / 2, B * B, 0, c.stream>>>(S, n, nb, k, c.d_info);
        GBCP_LAUNCH_CHECK(c);
      }
    }
  }
  for (int d = 1; d < nb; ++d) {
    ProfScope ps_(c, "k_trtri_diag");
    k_trtri_diag<<<nb - d, B * B, 0, c.stream>>>(S, X, n, d, c.d_info);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

}  // namespace gbcp
