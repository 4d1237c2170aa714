// Orthonormality constraint of Car-Parrinello dynamics: the reference's
// rortog -> rortho (rortog_utils.mod.F90:315-498, the iteration of Parrinello
// and Car, Les Houches 1988), on one GPU.
//
// Given c0 (orthonormal) and the propagated cm, the Lagrange multipliers gam
// make cm + c0 gam orthonormal:
//   rho = I - sym <c0|cm>,  sig = I - <cm|cm>,  del = -(<c0|c0> - I)/2 (tnon),
//   gam = sig/2,  X = rho^T rho/2 + sig/2,
//   repeat  gam' = X - (rho - gam)^T (rho - gam)/2 [+ gam^T del gam]
//   until max|gam' - gam| <= epsog/2, at most maxit iterations,
//   gam = sym gam,  cm <- cm + c0 gam (rotate_utils.mod.F90:63-101).
// The three overlaps over the 2 ngw real-view rows are the large GEMMs (tensor
// cores, FP64-accurate split, in the mixed mode; FP64 SIMT otherwise), as is
// the update of cm.  The n x n iteration runs in FP64 with one host read of
// max|gam' - gam| per iteration, as the reference's loop has.  Small matrices
// are row-major, M[i*n + j] = M(i, j) of the reference.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ctx.h"

namespace gbcp {

namespace {

constexpr int TS = 64, BK = 16, NT = 256;  // cross-overlap tiles (16 x 16 threads, 4 x 4 outputs)
constexpr int ST = 16;                     // small GEMM: 16 x 16 outputs per CTA, one per thread

// part[split][i][j] = sum_{k in the split's chunk} X(k, i) Y(k, j), every tile of the grid
__global__ void __launch_bounds__(NT) k_xov_part(const double* __restrict__ X, int ldx, const double* __restrict__ Y,
                                                 int ldy, int K, int n, int kchunk, double* __restrict__ part) {
  __shared__ double As[BK][TS + 1];
  __shared__ double Bs[BK][TS + 1];
  const int i0 = blockIdx.x * TS, j0 = blockIdx.y * TS;
  const int k0 = blockIdx.z * kchunk, k1 = min(K, k0 + kchunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int kb = k0; kb < k1; kb += BK) {
    for (int q = 0; q < 4; ++q) {
      const int kk = threadIdx.x % 16, cc = threadIdx.x / 16 + 16 * q;
      const int k = kb + kk, ci = i0 + cc, cj = j0 + cc;
      As[kk][cc] = (k < k1 && ci < n) ? X[k + (size_t)ci * ldx] : 0.0;
      Bs[kk][cc] = (k < k1 && cj < n) ? Y[k + (size_t)cj * ldy] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][ty + 16 * u];
        b[u] = Bs[kk][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
  double* P = part + (size_t)blockIdx.z * n * n;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
      if (i < n && j < n) P[(size_t)i * n + j] = acc[u][v];
    }
}

// A[i][j] = 2 sum_split part - Re x_i(0) Re y_j(0)
__global__ void k_xov_fold(const double* __restrict__ part, int nsplit, int n, const double* __restrict__ X, int ldx,
                           const double* __restrict__ Y, int ldy, int geq0, double* __restrict__ A) {
  const size_t nn = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += part[(size_t)p * nn + e];
    s *= 2.0;
    if (geq0) s -= X[(size_t)i * ldx] * Y[(size_t)j * ldy];
    A[e] = s;
  }
}

// Cout(r, j) += sum_k A(r, k) M[k][j]: real views, rows = 2 ngw; skipped once the status word is set
__global__ void __launch_bounds__(NT) k_rotate_acc(const double* __restrict__ A, int lda, int rows, int n,
                                                   const double* __restrict__ M, double* __restrict__ Cout, int ldo,
                                                   const int* __restrict__ status) {
  __shared__ double As[BK][TS + 1];
  __shared__ double Ms[BK][TS + 1];
  if (*(volatile const int*)status != 0) return;
  const int r0 = blockIdx.x * TS, j0 = blockIdx.y * TS;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int kb = 0; kb < n; kb += BK) {
    for (int q = 0; q < 4; ++q) {
      const int rr = threadIdx.x % 64, kk = threadIdx.x / 64 + 4 * q;
      const int r = r0 + rr, k = kb + kk;
      As[kk][rr] = (r < rows && k < n) ? A[r + (size_t)k * lda] : 0.0;
      const int cc = threadIdx.x % 64, km = threadIdx.x / 64 + 4 * q;
      const int cj = j0 + cc, k2 = kb + km;
      Ms[km][cc] = (cj < n && k2 < n) ? M[(size_t)k2 * n + cj] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][tx + 16 * u];
        b[u] = Ms[kk][ty + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = r0 + tx + 16 * u, cj = j0 + ty + 16 * v;
      if (r < rows && cj < n) Cout[r + (size_t)cj * ldo] += acc[u][v];
    }
}

// C = beta C0 + alpha op(A1 - A2) op(B1 - B2), n x n row-major; op(M) = M^T when trans.
// A2 / B2 / C0 may be NULL (zero).  One output per thread, 16 x 16 per CTA: the
// FP64 pipe of each SM (a few FMAs per clock) bounds this, so the work is spread
// over (n/16)^2 CTAs.
__global__ void __launch_bounds__(ST * ST) k_small_gemm(const double* __restrict__ A1, const double* __restrict__ A2,
                                                        int transA, const double* __restrict__ B1,
                                                        const double* __restrict__ B2, int transB, int n, double alpha,
                                                        const double* __restrict__ C0, double beta,
                                                        double* __restrict__ C) {
  __shared__ double As[ST][ST + 1];  // As[k][i] = op(A)(i, k)
  __shared__ double Bs[ST][ST + 1];  // Bs[k][j] = op(B)(k, j)
  const int tx = threadIdx.x % ST, ty = threadIdx.x / ST;
  const int i = blockIdx.y * ST + ty, j = blockIdx.x * ST + tx;
  double acc = 0.0;
  for (int kb = 0; kb < n; kb += ST) {
    {  // thread (ty, tx): A element (row i0 + tx, k = kb + ty) and B element (k = kb + ty, col j)
      const int ia = blockIdx.y * ST + tx, k = kb + ty;
      double a = 0.0, b = 0.0;
      if (ia < n && k < n) {
        const size_t ea = transA ? (size_t)k * n + ia : (size_t)ia * n + k;
        a = A1[ea] - (A2 ? A2[ea] : 0.0);
      }
      if (j < n && k < n) {
        const size_t eb = transB ? (size_t)j * n + k : (size_t)k * n + j;
        b = B1[eb] - (B2 ? B2[eb] : 0.0);
      }
      As[ty][tx] = a;
      Bs[ty][tx] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ST; ++kk) acc = fma(As[kk][ty], Bs[kk][tx], acc);
    __syncthreads();
  }
  if (i < n && j < n) {
    const size_t e = (size_t)i * n + j;
    C[e] = alpha * acc + (C0 ? beta * C0[e] : 0.0);
  }
}

// rho = I - (A01 + A01^T)/2, sig = I - A11, gam = sig/2, del = -(A00 - I)/2 (when A00)
__global__ void k_rt_init(const double* __restrict__ A01, const double* __restrict__ A11,
                          const double* __restrict__ A00, int n, double* __restrict__ rho, double* __restrict__ sig,
                          double* __restrict__ gam, double* __restrict__ del) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    const double d = (i == j) ? 1.0 : 0.0;
    rho[e] = d - 0.5 * (A01[e] + A01[(size_t)j * n + i]);
    const double s = d - A11[e];
    sig[e] = s;
    gam[e] = 0.5 * s;
    if (A00) del[e] = -0.5 * (A00[e] - d);
  }
}

// max |a - b| as ordered bits (non-negative doubles order like their bit patterns)
__global__ void k_rt_maxdiff(const double* __restrict__ a, const double* __restrict__ b, size_t nn,
                             unsigned long long* __restrict__ bits) {
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    const double d = fabs(a[e] - b[e]);
    mx = (d > mx || d != d) ? d : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_down_sync(0xffffffffu, mx, o);
    mx = (v > mx || v != v) ? v : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(bits, (unsigned long long)__double_as_longlong(mx));
}

// g = (g + g^T)/2 into out
__global__ void k_rt_symma(const double* __restrict__ g, int n, double* __restrict__ out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    out[e] = 0.5 * (g[e] + g[(size_t)j * n + i]);
  }
}

int small_grid(int n) { return std::max(1, std::min(1024, (n * n + 255) / 256)); }

int small_gemm(Ctx& c, const double* A1, const double* A2, int transA, const double* B1, const double* B2, int transB,
               int n, double alpha, const double* C0, double beta, double* C) {
  ProfScope ps_(c, "k_small_gemm");
  const dim3 grid((n + ST - 1) / ST, (n + ST - 1) / ST);
  k_small_gemm<<<grid, ST * ST, 0, c.stream>>>(A1, A2, transA, B1, B2, transB, n, alpha, C0, beta, C);
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

}  // namespace

// A (row-major n x n) = <X_i|Y_j>, X and Y complex ngw x n with leading dimensions ldx, ldy
int xovlap(Ctx& c, const cx<double>* X, int ldx, const cx<double>* Y, int ldy, int n, double* A) {
  const double* Xr = reinterpret_cast<const double*>(X);
  const double* Yr = reinterpret_cast<const double*>(Y);
  const int K = 2 * c.ngw;
  if (use_tc_gemm(c)) return xovlap_tc(c, Xr, 2 * ldx, Yr, 2 * ldy, n, A, c.d_info);
  const int nt = (n + TS - 1) / TS;
  int nsplit = std::max(1, std::min(1024, (4 * 152 + nt * nt - 1) / (nt * nt)));
  int kchunk = (K + nsplit - 1) / nsplit;
  kchunk = ((kchunk + BK - 1) / BK) * BK;
  nsplit = (K + kchunk - 1) / kchunk;
  if (!ensure(c, c.sparts, sizeof(double) * (size_t)nsplit * n * n + 16)) return 6;
  double* part = static_cast<double*>(c.sparts.p);
  {
    ProfScope ps_(c, "k_xov_part");
    k_xov_part<<<dim3(nt, nt, nsplit), NT, 0, c.stream>>>(Xr, 2 * ldx, Yr, 2 * ldy, K, n, kchunk, part);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_xov_fold");
    k_xov_fold<<<small_grid(n), 256, 0, c.stream>>>(part, nsplit, n, Xr, 2 * ldx, Yr, 2 * ldy, c.geq0, A);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

int rortho(Ctx& c, const cx<double>* c0, int ldc0, cx<double>* cm, int ldcm, int n, int tnon, double epsog, int maxit,
           double* gam_out, int* iters) {
  if (iters) *iters = 0;
  if (n <= 0) return 0;
  const size_t nn = (size_t)n * n;
  // A01, A11, A00, rho, sig (then X), del, gam, gamn, tmp
  if (!ensure(c, c.rt_mats, sizeof(double) * (9 * nn + 2))) return 6;
  double* A01 = static_cast<double*>(c.rt_mats.p);
  double* A11 = A01 + nn;
  double* A00 = A11 + nn;
  double* rho = A00 + nn;
  double* sig = rho + nn;
  double* del = sig + nn;
  double* gam = del + nn;
  double* gamn = gam + nn;
  double* tmp = gamn + nn;
  unsigned long long* dbits = reinterpret_cast<unsigned long long*>(tmp + nn);
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, 16, c.stream));
  int rc;
  if ((rc = xovlap(c, c0, ldc0, cm, ldcm, n, A01))) return rc;
  if ((rc = xovlap(c, cm, ldcm, cm, ldcm, n, A11))) return rc;
  if (tnon && (rc = xovlap(c, c0, ldc0, c0, ldc0, n, A00))) return rc;
  {
    ProfScope ps_(c, "k_rt_init");
    k_rt_init<<<small_grid(n), 256, 0, c.stream>>>(A01, A11, tnon ? A00 : nullptr, n, rho, sig, gam, del);
    GBCP_LAUNCH_CHECK(c);
  }
  // fixed term X = rho^T rho / 2 + sig / 2 (in place of sig)
  if ((rc = small_gemm(c, rho, nullptr, 1, rho, nullptr, 0, n, 0.5, sig, 0.5, sig))) return rc;
  const double* X = sig;
  int it = 0;
  double dif = 0.0;
  while (true) {
    ++it;
    // gamn = X - (rho - gam)^T (rho - gam) / 2
    if ((rc = small_gemm(c, rho, gam, 1, rho, gam, 0, n, -0.5, X, 1.0, gamn))) return rc;
    if (tnon) {  // gamn += gam^T (del gam)
      if ((rc = small_gemm(c, del, nullptr, 0, gam, nullptr, 0, n, 1.0, nullptr, 0.0, tmp))) return rc;
      if ((rc = small_gemm(c, gam, nullptr, 1, tmp, nullptr, 0, n, 1.0, gamn, 1.0, gamn))) return rc;
    }
    GBCP_CUDA_TRY(c, cudaMemsetAsync(dbits, 0, sizeof(unsigned long long), c.stream));
    {
      ProfScope ps_(c, "k_rt_maxdiff");
      k_rt_maxdiff<<<small_grid(n), 256, 0, c.stream>>>(gamn, gam, nn, dbits);
      GBCP_LAUNCH_CHECK(c);
    }
    unsigned long long hb = 0;
    GBCP_CUDA_TRY(c, cudaMemcpyAsync(&hb, dbits, sizeof(hb), cudaMemcpyDeviceToHost, c.stream));
    GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    memcpy(&dif, &hb, sizeof(dif));
    std::swap(gam, gamn);
    if (!(dif > 0.5 * epsog && it <= maxit)) break;
  }
  if (iters) *iters = it;
  if (it > maxit || !std::isfinite(dif)) {
    c.err = "RORTHO: max|gam' - gam| = " + std::to_string(dif) + " after " + std::to_string(it) +
            " iterations (maximum " + std::to_string(maxit) + ")";
    return 8;
  }
  double* gsym = gamn;  // the buffer not holding gam
  {
    ProfScope ps_(c, "k_rt_symma");
    k_rt_symma<<<small_grid(n), 256, 0, c.stream>>>(gam, n, gsym);
    GBCP_LAUNCH_CHECK(c);
  }
  // cm <- cm + c0 gam (rotate with a = b = 1)
  const int rows = 2 * c.ngw;
  if (use_tc_gemm(c)) {
    if ((rc = rmul_tc(c, reinterpret_cast<const double*>(c0), 2 * ldc0, rows, n, gsym, 0,
                      reinterpret_cast<double*>(cm), 2 * ldcm, 0, c.d_info, 1)))
      return rc;
  } else {
    ProfScope ps_(c, "k_rotate_acc");
    k_rotate_acc<<<dim3((rows + TS - 1) / TS, (n + TS - 1) / TS), NT, 0, c.stream>>>(
        reinterpret_cast<const double*>(c0), 2 * ldc0, rows, n, gsym, reinterpret_cast<double*>(cm), 2 * ldcm,
        c.d_info);
    GBCP_LAUNCH_CHECK(c);
  }
  if (gam_out) GBCP_CUDA_TRY(c, cudaMemcpyAsync(gam_out, gsym, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c.stream));
  int st = 0;
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(&st, c.d_info, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (st == -2) {
    c.err = "rortho (tensor cores): an mbarrier wait timed out";
    return 4;
  }
  return 0;
}

}  // namespace gbcp
