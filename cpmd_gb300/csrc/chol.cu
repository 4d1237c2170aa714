// Blocked Cholesky factorisation S = U^T U and triangular inverse X = U^{-1}
// of the overlap matrix (the reference's uinv: dpotrf + dtrtri,
// rgs_utils.mod.F90:95-162), spread over many CTAs.
//
// 32 x 32 blocks, right-looking:
//   for each diagonal block k:
//     diag   one CTA factors A_kk = U_kk^T U_kk in shared memory and inverts U_kk
//     panel  U_kj = U_kk^{-T} A_kj for every block j > k (one CTA per block)
//     update A_ij -= U_ki^T U_kj for k < i <= j (one CTA per block)
//   then X block-diagonal by block-diagonal: X_ii = U_ii^{-1} (from diag) and
//   X_ij = -U_ii^{-1} sum_{k=i+1..j} U_ik X_kj for j - i = 1, 2, ...
// Every kernel first reads the ortho status word and does nothing once a step
// has failed; diag sets it to (global pivot index + 1) at a non-positive pivot
// and to -1 at a NaN.  S is row-major n x n (symmetric, upper part used and
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

// factor + invert the diagonal block k; U_kk -> S (upper), U_kk^{-1} -> X (diag block)
__global__ void __launch_bounds__(1024) k_chol_diag(double* __restrict__ S, double* __restrict__ X, int n, int k,
                                                    int* __restrict__ status) {
  __shared__ double a[B][B + 1];
  __shared__ double w[B][B + 1];
  __shared__ int bad;
  if (failed(status)) return;
  const int r = threadIdx.x / B, c = threadIdx.x % B;
  load_block(S, n, k, k, a, 1.0);
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int p = 0; p < B; ++p) {
    if (threadIdx.x == 0) {
      const double d = a[p][p];
      if (!(d > 0.0)) bad = (d != d) ? -1 : k * B + p + 1;
      else a[p][p] = sqrt(d);
    }
    __syncthreads();
    if (bad) break;
    if (r == p && c > p) a[p][c] /= a[p][p];
    __syncthreads();
    if (r > p && c >= r) a[r][c] -= a[p][r] * a[p][c];
    __syncthreads();
  }
  if (bad) {
    if (threadIdx.x == 0) atomicExch(status, bad);
    return;
  }
  // zero the strict lower part, then invert the upper triangular block by columns
  if (c < r) a[r][c] = 0.0;
  w[r][c] = 0.0;
  __syncthreads();
  if (threadIdx.x < B) {
    const int j = threadIdx.x;
    w[j][j] = 1.0 / a[j][j];
    for (int i = j - 1; i >= 0; --i) {
      double s = 0.0;
      for (int m = i + 1; m <= j; ++m) s = fma(a[i][m], w[m][j], s);
      w[i][j] = -s / a[i][i];
    }
  }
  __syncthreads();
  store_block(S, n, k, k, a);
  store_block(X, n, k, k, w);
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

__global__ void k_zero_lower(double* __restrict__ X, int n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (j < i) X[e] = 0.0;
  }
}

}  // namespace

// Queue U = chol(S) (in place, upper) and X = U^{-1}; no synchronisation.
int chol_inverse(Ctx& c, double* S, double* X, int n) {
  const int nb = (n + B - 1) / B;
  {
    ProfScope ps_(c, "k_chol");
    k_zero_lower<<<std::max(1, std::min(256, (n * n + 255) / 256)), 256, 0, c.stream>>>(X, n);
    GBCP_LAUNCH_CHECK(c);
    for (int k = 0; k < nb; ++k) {
      k_chol_diag<<<1, B * B, 0, c.stream>>>(S, X, n, k, c.d_info);
      GBCP_LAUNCH_CHECK(c);
      const int m0 = nb - k - 1;
      if (m0 > 0) {
        k_chol_panel<<<m0, B * B, 0, c.stream>>>(S, X, n, k, c.d_info);
        GBCP_LAUNCH_CHECK(c);
        k_chol_update<<<m0 * (m0 + 1) / 2, B * B, 0, c.stream>>>(S, n, nb, k, c.d_info);
        GBCP_LAUNCH_CHECK(c);
      }
    }
    for (int d = 1; d < nb; ++d) {
      k_trtri_diag<<<nb - d, B * B, 0, c.stream>>>(S, X, n, d, c.d_info);
      GBCP_LAUNCH_CHECK(c);
    }
  }
  return 0;
}

}  // namespace gbcp
