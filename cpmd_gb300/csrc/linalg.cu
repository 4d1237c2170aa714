// Orthogonalisation of the Γ-point states (FP64 path).
//
// Reference: ortho -> rgs (rgs_utils.mod.F90:31-93): S = 2 C^T C - c0 c0^T
// over the real view of C (dsyrk 'U','T' alpha=2 + dger -1), dpotrf/dtrtri
// (uinv, l.95-162), C <- C U^{-1} (dtrmm R,U,N,N), zclean.
// lowdin (lowdin_utils.mod.F90:58-89): the same S via csmat/ovlap, then
// A = S^{-1/2} and C <- C A.
//
// GB300 form:
//  * S: split-K tiled FP64 GEMM over the real view (K = 2 ngw), upper block
//    triangle only, partial tiles folded by a second kernel that also applies
//    the G=0 correction, mirrors the lower triangle and computes max|S-I|.
//  * U and U^{-1}: blocked over many CTAs (chol.cu).
//  * S^{-1/2}: coupled Newton-Schulz iteration on GEMMs (Y -> S^{1/2},
//    Z -> S^{-1/2}); mathematically the same matrix as Z w^{-1/2} Z^T from the
//    reference's dspevy, reached without an eigensolver.
//  * C <- C M: tiled FP64 GEMM (triangular skip for U^{-1}) into scratch,
//    copied back with the zclean fused.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda.h>

#include "ctx.h"

namespace gbcp {

namespace {

constexpr int TS = 64;   // output tile
constexpr int BK = 16;   // K step
constexpr int NT = 256;  // threads (16 x 16, 4 x 4 outputs each)

// Partial S over one K-chunk for one upper tile pair (bi <= bj), TT x TT output
// tiles (TT = 64 or 32: 4 x 4 or 2 x 2 outputs per thread; the batch autotuner
// picks per size class).
// A(k, i) = Ar[k + i*lda]  (real view of C, lda = 2*ldc, K = 2*ngw)
template <int TT = TS>
__global__ void __launch_bounds__(NT) k_syrk_part(const double* __restrict__ Ar, int lda, int K, int n, int ntb,
                                                  int kchunk, double* __restrict__ part) {
  constexpr int U = TT / 16;
  __shared__ double As[BK][TT + 1];
  __shared__ double Bs[BK][TT + 1];
  // decode tile pair from blockIdx.x over the upper triangle of ntb x ntb tiles
  int t = blockIdx.x, bi = 0;
  while (t >= ntb - bi) {
    t -= ntb - bi;
    ++bi;
  }
  const int bj = bi + t;
  const int split = blockIdx.y;
  const int k0 = split * kchunk, k1 = min(K, k0 + kchunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[U][U] = {};
  const int i0 = bi * TT, j0 = bj * TT;
  for (int kb = k0; kb < k1; kb += BK) {
    // load 16 x TT for both operands: thread -> (k = tid % 16, col = tid / 16 + 16 q)
    for (int q = 0; q < U; ++q) {
      const int kk = threadIdx.x % 16, cc = threadIdx.x / 16 + 16 * q;
      const int k = kb + kk;
      const int ci = i0 + cc, cj = j0 + cc;
      As[kk][cc] = (k < k1 && ci < n) ? Ar[k + (size_t)ci * lda] : 0.0;
      Bs[kk][cc] = (k < k1 && cj < n) ? Ar[k + (size_t)cj * lda] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[U], b[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        a[u] = As[kk][ty + 16 * u];
        b[u] = Bs[kk][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int v = 0; v < U; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
  // part[split][i][j] (row-major n x n)
  double* P = part + (size_t)split * n * n;
#pragma unroll
  for (int u = 0; u < U; ++u)
#pragma unroll
    for (int v = 0; v < U; ++v) {
      const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
      if (i < n && j < n) P[(size_t)i * n + j] = acc[u][v];
    }
}

// S[i][j] = 2 sum_split part - Re c0_i Re c0_j for the upper triangle tiles,
// mirrored into the lower triangle.  Column-major == row-major (symmetric).
__global__ void k_syrk_fold(const double* __restrict__ part, int nsplit, int n, int ts, const double* __restrict__ Ar,
                            int lda, int geq0, double* __restrict__ S, unsigned long long* __restrict__ scond_bits) {
  const size_t nn = (size_t)n * n;
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    const int bi = i / ts, bj = j / ts;
    if (bi > bj) continue;  // lower block triangle handled by mirroring
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += part[(size_t)p * nn + e];
    s *= 2.0;
    if (geq0) s -= Ar[(size_t)i * lda] * Ar[(size_t)j * lda];
    S[(size_t)i * n + j] = s;
    S[(size_t)j * n + i] = s;
    const double d = fabs(i == j ? s - 1.0 : s);
    mx = fmax(mx, d);
  }
  if (scond_bits) {
    // non-negative doubles order like their bit patterns
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(scond_bits, (unsigned long long)__double_as_longlong(mx));
  }
}

// Cout = A * M.  A real view (rows = 2 ngw, lda), M (n x n) row-major (M[k][j]),
// TT x TT output tiles (64 or 32).
// upper != 0: M is upper triangular, column block j only needs k <= j.
template <int TT = TS>
__global__ void __launch_bounds__(NT) k_gemm_right(const double* __restrict__ A, int lda, int rows, int n,
                                                   const double* __restrict__ M, int upper, double* __restrict__ Cout,
                                                   int ldo, const int* __restrict__ status) {
  constexpr int U = TT / 16, R = NT / TT;  // outputs per thread per dimension, k rows per load pass
  __shared__ double As[BK][TT + 1];
  __shared__ double Ms[BK][TT + 1];
  if (*(volatile const int*)status != 0) return;
  const int r0 = blockIdx.x * TT, j0 = blockIdx.y * TT;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[U][U] = {};
  const int kend = upper ? min(n, j0 + TT) : n;
  for (int kb = 0; kb < kend; kb += BK) {
    for (int q = 0; q < BK / R; ++q) {
      // A tile: TT rows x 16 k, coalesced along rows
      const int rr = threadIdx.x % TT, kk = threadIdx.x / TT + R * q;
      const int r = r0 + rr, k = kb + kk;
      As[kk][rr] = (r < rows && k < n) ? A[r + (size_t)k * lda] : 0.0;
      // M tile: 16 k x TT cols
      const int cc = threadIdx.x % TT, km = threadIdx.x / TT + R * q;
      const int c = j0 + cc, k2 = kb + km;
      Ms[km][cc] = (c < n && k2 < n) ? M[(size_t)k2 * n + c] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[U], b[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        a[u] = As[kk][tx + 16 * u];
        b[u] = Ms[kk][ty + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int v = 0; v < U; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < U; ++u)
#pragma unroll
    for (int v = 0; v < U; ++v) {
      const int r = r0 + tx + 16 * u, c = j0 + ty + 16 * v;
      if (r < rows && c < n) Cout[r + (size_t)c * ldo] = acc[u][v];
    }
}

// copy the real view back (ngw complex rows per state) and zero Im c(G=0);
// nothing is written if the status word reports a failed step (c0 untouched)
__global__ void k_copy_back(const double* __restrict__ src, int lds, double* __restrict__ dst, int ldd, int rows,
                            int n, int geq0, const int* __restrict__ status) {
  if (*(volatile const int*)status != 0) return;
  const size_t tot = (size_t)rows * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % rows), c = (int)(e / rows);
    double v = src[r + (size_t)c * lds];
    if (geq0 && r == 1) v = 0.0;
    dst[r + (size_t)c * ldd] = v;
  }
}

// small dense n x n GEMM (row-major): C = alpha A B + beta C + gamma I
__global__ void __launch_bounds__(NT) k_gemm_nn(const double* __restrict__ A, const double* __restrict__ B,
                                                double* __restrict__ C, int n, double alpha, double beta,
                                                double gamma) {
  __shared__ double As[BK][TS + 1];
  __shared__ double Bs[BK][TS + 1];
  const int i0 = blockIdx.y * TS, j0 = blockIdx.x * TS;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int kb = 0; kb < n; kb += BK) {
    for (int q = 0; q < 4; ++q) {
      const int kk = threadIdx.x % 16, ii = threadIdx.x / 16 + 16 * q;
      As[kk][ii] = (i0 + ii < n && kb + kk < n) ? A[(size_t)(i0 + ii) * n + kb + kk] : 0.0;
      const int jj = threadIdx.x % 64, k2 = threadIdx.x / 64 + 4 * q;
      Bs[k2][jj] = (j0 + jj < n && kb + k2 < n) ? B[(size_t)(kb + k2) * n + j0 + jj] : 0.0;
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
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
      if (i < n && j < n) {
        double r = alpha * acc[u][v];
        if (beta != 0.0) r += beta * C[(size_t)i * n + j];
        if (i == j) r += gamma;
        C[(size_t)i * n + j] = r;
      }
    }
}

// Newton-Schulz set-up: alpha = max row sum |S| (>= lambda_max), Y = S/alpha, Z = I
// max |T - I| over an n x n matrix as ordered bits (many CTAs)
__global__ void k_dev_from_identity(const double* __restrict__ T, int n, unsigned long long* __restrict__ bits) {
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double d = fabs(T[e] - (((e / n) == (e % n)) ? 1.0 : 0.0));
    mx = (d > mx || d != d) ? d : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_down_sync(0xffffffffu, mx, o);
    mx = (v > mx || v != v) ? v : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(bits, (unsigned long long)__double_as_longlong(mx));
}

__global__ void k_scale(double* __restrict__ X, size_t n, const double* __restrict__ alpha, double power) {
  const double s = pow(*alpha, power);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) X[e] *= s;
}

// T = 3/2 I - (P + P^T)/4 (P = Z Y of the Newton-Schulz step, symmetric up to rounding,
// symmetrised here) and max |T - I| as ordered bits
__global__ void k_ns_t(const double* __restrict__ P, int n, double* __restrict__ T,
                       unsigned long long* __restrict__ dev_bits) {
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    const double d = (i == j) ? 1.0 : 0.0;
    const double t = 1.5 * d - 0.25 * (P[e] + P[(size_t)j * n + i]);
    T[e] = t;
    const double a = fabs(t - d);
    mx = (a > mx || a != a) ? a : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_down_sync(0xffffffffu, mx, o);
    mx = (v > mx || v != v) ? v : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(dev_bits, (unsigned long long)__double_as_longlong(mx));
}

// max over rows of sum_j |S_ij| as ordered bits (many CTAs, one warp per row)
__global__ void k_row_abs_max(const double* __restrict__ S, int n, unsigned long long* __restrict__ bits) {
  const int lane = threadIdx.x & 31;
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += gridDim.x * (blockDim.x >> 5)) {
    double sum = 0.0;
    for (int j = lane; j < n; j += 32) sum += fabs(S[(size_t)i * n + j]);
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) atomicMax(bits, (unsigned long long)__double_as_longlong(sum));
  }
}

// Y = S / alpha, Z = I, alpha from its ordered bits
__global__ void k_ns_start(const double* __restrict__ S, int n, const unsigned long long* __restrict__ abits,
                           double* __restrict__ Y, double* __restrict__ Z, double* __restrict__ alpha_out) {
  const double alpha = __longlong_as_double((long long)*abits);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    Y[e] = S[e] / alpha;
    Z[e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *alpha_out = alpha;
}

}  // namespace

// The ortho status word (c.d_info): int status at byte 0 (0 ok, k+1 not
// positive definite at pivot k, -1 non-finite, -2 timed-out tensor-core wait),
// max|S-I| as ordered bits at byte 8.  Every ortho kernel checks it, so a
// failed step leaves c0 untouched and the host synchronises once at the end.
static unsigned long long* scond_bits_of(Ctx& c) { return reinterpret_cast<unsigned long long*>(c.d_info + 2); }

static int status_error(Ctx& c, int st) {
  if (st > 0) {
    c.err = "UINV: leading minor " + std::to_string(st) + " not positive definite (dpotrf)";
    return 2;
  }
  if (st == -1) {
    c.err = "UINV: non-finite overlap";
    return 3;
  }
  if (st == -2) {
    c.err = "ortho (tensor cores): an mbarrier wait timed out";
    return 4;
  }
  return 0;
}

// read the status word (and scond) after one synchronisation
static int finish_status(Ctx& c, double* scond_host) {
  int h[4] = {0, 0, 0, 0};
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(h, c.d_info, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (scond_host) {
    unsigned long long b;
    memcpy(&b, h + 2, sizeof(b));
    double d;
    memcpy(&d, &b, sizeof(d));
    *scond_host = d;
  }
  return status_error(c, h[0]);
}

// S (n x n) queued on the stream; scond bits if requested.  No synchronisation.
int ovlap_gamma_ex(Ctx& c, const cx<double>* c0, int ldc, int nstate, double* S, bool want_scond) {
  unsigned long long* bits = want_scond ? scond_bits_of(c) : nullptr;
  if (use_tc_gemm(c)) return ovlap_tc(c, c0, ldc, nstate, S, bits, c.d_info);
  const int n = nstate;
  const int K = 2 * c.ngw;
  const int lda = 2 * ldc;
  const int ts = c.simt_tile == 32 ? 32 : TS;
  const int ntb = (n + ts - 1) / ts;
  const int npairs = ntb * (ntb + 1) / 2;
  // enough CTAs to fill the GPU: ~4 waves of 152 SMs
  int nsplit = std::max(1, std::min(1024, (4 * 152 + npairs - 1) / npairs));
  int kchunk = (K + nsplit - 1) / nsplit;
  kchunk = ((kchunk + BK - 1) / BK) * BK;
  nsplit = (K + kchunk - 1) / kchunk;
  if (!ensure(c, c.sparts, sizeof(double) * (size_t)nsplit * n * n + 16)) return 6;
  const double* Ar = reinterpret_cast<const double*>(c0);
  double* part = static_cast<double*>(c.sparts.p);
  {
    ProfScope ps_(c, "k_syrk_part");
    if (ts == 32)
      k_syrk_part<32><<<dim3(npairs, nsplit), NT, 0, c.stream>>>(Ar, lda, K, n, ntb, kchunk, part);
    else
      k_syrk_part<TS><<<dim3(npairs, nsplit), NT, 0, c.stream>>>(Ar, lda, K, n, ntb, kchunk, part);
    GBCP_LAUNCH_CHECK(c);
  }
  const int fb = std::max(1, std::min(1024, (n * n + 255) / 256));
  {
    ProfScope ps_(c, "k_syrk_fold");
    k_syrk_fold<<<fb, 256, 0, c.stream>>>(part, nsplit, n, ts, Ar, lda, c.geq0, S, bits);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

int ovlap_gamma(Ctx& c, const cx<double>* c0, int ldc, int nstate, double* S) {
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, 16, c.stream));
  const int rc = ovlap_gamma_ex(c, c0, ldc, nstate, S, false);
  if (rc) return rc;
  return finish_status(c, nullptr);
}

static int apply_right(Ctx& c, cx<double>* c0, int ldc, int nstate, const double* M, int upper) {
  const int rows = 2 * c.ngw;
  const int lda = 2 * ldc;
  if (use_tc_gemm(c)) {
    // in place: the split GEMM reads the digit planes of C, sliced before it starts, and
    // writes nothing once the status word reports a failed step
    return rmul_tc(c, reinterpret_cast<const double*>(c0), lda, rows, nstate, M, upper,
                   reinterpret_cast<double*>(c0), lda, c.geq0, c.d_info);
  }
  if (!ensure(c, c.cscr, sizeof(double) * (size_t)rows * nstate)) return 6;
  double* tmp = static_cast<double*>(c.cscr.p);
  {
    const int ts = c.simt_tile == 32 ? 32 : TS;
    dim3 grid((rows + ts - 1) / ts, (nstate + ts - 1) / ts);
    ProfScope ps_(c, "k_gemm_right");
    if (ts == 32)
      k_gemm_right<32><<<grid, NT, 0, c.stream>>>(reinterpret_cast<const double*>(c0), lda, rows, nstate, M, upper,
                                                  tmp, rows, c.d_info);
    else
      k_gemm_right<TS><<<grid, NT, 0, c.stream>>>(reinterpret_cast<const double*>(c0), lda, rows, nstate, M, upper,
                                                  tmp, rows, c.d_info);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_copy_back");
    k_copy_back<<<1024, 256, 0, c.stream>>>(tmp, rows, reinterpret_cast<double*>(c0), lda, rows, nstate, c.geq0,
                                            c.d_info);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

static int ortho_gs_steps(Ctx& c, cx<double>* c0, int ldc, int n, bool want_scond) {
  if (n > 4096) {
    c.err = "ortho: nstate above 4096 not supported";
    return 7;
  }
  if (!ensure(c, c.smat, sizeof(double) * (size_t)n * n) || !ensure(c, c.smat2, sizeof(double) * (size_t)n * n))
    return 6;
  double* S = static_cast<double*>(c.smat.p);
  double* X = static_cast<double*>(c.smat2.p);
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, 16, c.stream));
  // tensor-core engine: the digit planes of C for C U^-1 depend on C only, so they
  // are cut on the side stream while the Cholesky (a few SMs) runs -- queued after S,
  // whose own HBM-bound passes it would otherwise slow; not inside a stream capture
  // (the batch graph keeps the single-stream order)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GBCP_CUDA_TRY(c, cudaStreamIsCapturing(c.stream, &cap));
  const cudaEvent_t* sliced = nullptr;
  const int rows = 2 * c.ngw, lda = 2 * ldc;
  int rb[2] = {0, rows};
  double* Ar = reinterpret_cast<double*>(c0);
  int rc = ovlap_gamma_ex(c, c0, ldc, n, S, want_scond);
  if (rc) return rc;
  if (use_tc_gemm(c) && n <= 256 && cap == cudaStreamCaptureStatusNone) {
    rc = slice_rows_side(c, Ar, lda, rows, n, rb, 1, nullptr, &sliced);
    if (rc) return rc;
  }
  rc = chol_inverse(c, S, X, n);
  if (!rc && sliced) rc = rmul_tc_ranges(c, Ar, lda, rows, n, X, 1, Ar, lda, c.geq0, c.d_info, rb, 1, nullptr, sliced);
  if (rc || sliced) {
    // the side stream still reads C: the context stream waits for it before returning
    if (rc && sliced) cudaStreamWaitEvent(c.stream, sliced[0], 0);
    return rc;
  }
  return apply_right(c, c0, ldc, n, X, 1);
}

// Gram-Schmidt of host-memory c0 (ld ldh) with its copies overlapped: the states
// go up in R ranges of G rows on the copy stream, and range r's column exponents,
// digit planes and partial overlap start as soon as it has landed; after the
// Cholesky, C U^-1 runs range by range (in place in the staging buffer) and each
// finished range goes back on the download stream while the next is computed.
// A failed step skips the GEMM, so the download returns the unchanged states.
int ortho_gs_host(Ctx& c, double* h, int ldh, int n, double* scond_host, int resident,
                  const std::function<bool()>* confirm) {
  if (!use_tc_gemm(c) || n > 4096 || n <= 0) return 7;
  const int ngw = c.ngw;
  // G-row ranges: multiples of 64 complex rows (128 real rows: one C M row tile, four S sub-chunks)
  const int R = std::max(1, std::min(4, ngw / 4096));
  int gb[5];
  for (int r = 0; r <= R; ++r) gb[r] = (r == R) ? ngw : std::min(ngw, ((int)((long long)ngw * r / R) / 64) * 64);
  int kb[5];
  for (int r = 0; r <= R; ++r) kb[r] = 2 * gb[r];
  if (!ensure(c, c.st_c0, sizeof(cx<double>) * (size_t)ngw * n) ||
      !ensure(c, c.smat, sizeof(double) * (size_t)n * n) || !ensure(c, c.smat2, sizeof(double) * (size_t)n * n))
    return 6;
  if ((!c.copy && cudaStreamCreateWithFlags(&c.copy, cudaStreamNonBlocking) != cudaSuccess) ||
      (!c.copy_out && cudaStreamCreateWithFlags(&c.copy_out, cudaStreamNonBlocking) != cudaSuccess)) {
    c.err = "copy streams";
    return 5;
  }
  while (c.pipe_ev.size() < (size_t)(2 * R + 2)) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      c.err = "pipeline events";
      return 5;
    }
    c.pipe_ev.push_back(e);
  }
  cudaEvent_t* up = c.pipe_ev.data() + 1;
  cudaEvent_t* done = c.pipe_ev.data() + 1 + R;
  cx<double>* d = static_cast<cx<double>*>(c.st_c0.p);
  double* S = static_cast<double*>(c.smat.p);
  double* X = static_cast<double*>(c.smat2.p);
  // the staging buffer is free once earlier work on the context stream is done
  GBCP_CUDA_TRY(c, cudaEventRecord(c.pipe_ev[0], c.stream));
  GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.copy, c.pipe_ev[0], 0));
  for (int r = 0; r < R; ++r) {
    const int g0 = gb[r], g = gb[r + 1] - gb[r];
    if (g > 0 && !resident) {
      ProfScope ps_(c, "h2d_states", c.copy, 1);
      GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(d + g0, sizeof(cx<double>) * (size_t)ngw, h + 2 * (size_t)g0,
                                         sizeof(cx<double>) * (size_t)ldh, sizeof(cx<double>) * (size_t)g, n,
                                         cudaMemcpyHostToDevice, c.copy));
    }
    GBCP_CUDA_TRY(c, cudaEventRecord(up[r], c.copy));
  }
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, 16, c.stream));
  double* Ar = reinterpret_cast<double*>(d);
  // C U^-1's digit planes of range r are cut on the side stream once range r has
  // landed, beside the overlap ranges and the Cholesky.  States already on the
  // device (the wavefunction cache): S in one pass as in the device-memory call,
  // the planes cut beside the Cholesky only
  const cudaEvent_t* sliced = nullptr;
  unsigned long long* sbits = scond_host ? scond_bits_of(c) : nullptr;
  int rc = 0;
  const bool cols_ok = c.ortho_cols && n > 64 && n <= 256 && c.chol_df != 3;
  if (resident && cols_ok) {
    // by column blocks the first C U^-1 follows the first diagonal block: the row
    // planes are cut beside the overlap instead of after it
    rc = slice_rows_side(c, Ar, 2 * ngw, 2 * ngw, n, kb, R, nullptr, &sliced);
    if (!rc) rc = ovlap_tc(c, d, ngw, n, S, sbits, c.d_info);
  } else if (resident) {
    rc = ovlap_tc(c, d, ngw, n, S, sbits, c.d_info);
    if (!rc && n <= 256) rc = slice_rows_side(c, Ar, 2 * ngw, 2 * ngw, n, kb, R, nullptr, &sliced);
  } else {
    rc = n <= 256 ? slice_rows_side(c, Ar, 2 * ngw, 2 * ngw, n, kb, R, up, &sliced) : 0;
    if (!rc) rc = ovlap_tc_ranges(c, Ar, 2 * ngw, n, kb, R, up, S, sbits, c.d_info);
  }
  // C U^-1 and the download by column blocks of 32 states as the chain finishes each
  // block of U^-1 (65 to 256 states; the planes of C cut on the side stream), else
  // by G-row ranges after the whole chain
  const int nb = (n + 31) / 32;
  const bool cols = cols_ok && sliced != nullptr;
  if (cols) {
    // the key is confirmed before anything writes the states or the host array
    if (!rc && resident && confirm && !(*confirm)()) {
      cudaStreamSynchronize(c.stream);
      if (c.side) cudaStreamSynchronize(c.side);
      return 8;
    }
    while (!rc && c.col_ev.size() < (size_t)(2 * nb + 1)) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        c.err = "events";
        rc = 5;
      } else {
        c.col_ev.push_back(e);
      }
    }
    // column block k, queued on the side stream: C U^-1 into st_c2, then its download.
    // The early blocks reach the host before the factorisation is known to succeed,
    // so C stays in st_c0 for restoring the host array after a failure
    if (!rc && !ensure(c, c.st_c2, sizeof(cx<double>) * (size_t)ngw * n)) rc = 6;
    cx<double>* o = static_cast<cx<double>*>(c.st_c2.p);
    auto column = [&](int k) -> int {
      const int r = rmul_tc_column_block(c, 2 * ngw, n, X, reinterpret_cast<double*>(o), 2 * ngw, c.geq0, c.d_info, k);
      if (r) return r;
      const cudaEvent_t e = c.col_ev[nb + 1 + k];
      GBCP_CUDA_TRY(c, cudaEventRecord(e, c.stream));
      GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.copy_out, e, 0));
      const int j0 = 32 * k, nj = std::min(n, j0 + 32) - j0;
      ProfScope ps_(c, "d2h_states", c.copy_out, 2);
      GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(h + 2 * (size_t)j0 * ldh, sizeof(cx<double>) * (size_t)ldh,
                                         o + (size_t)j0 * ngw, sizeof(cx<double>) * (size_t)ngw,
                                         sizeof(cx<double>) * (size_t)ngw, nj, cudaMemcpyDeviceToHost, c.copy_out));
      return 0;
    };
    if (!rc) rc = chol_inverse_columns(c, S, X, n, column);
  } else {
    if (!rc) rc = chol_inverse(c, S, X, n);
    if (!rc && resident && confirm && !(*confirm)()) {
      // the host array changed under the same key parts: the speculative overlap and
      // factor (which only read st_c0) are dropped before anything writes the states
      cudaStreamSynchronize(c.stream);
      if (c.side) cudaStreamSynchronize(c.side);
      return 8;
    }
    if (!rc) rc = rmul_tc_ranges(c, Ar, 2 * ngw, 2 * ngw, n, X, 1, Ar, 2 * ngw, c.geq0, c.d_info, kb, R, done, sliced);
  }
  if (rc) {
    cudaStreamSynchronize(c.copy);
    if (c.side) cudaStreamSynchronize(c.side);
    cudaStreamSynchronize(c.copy_out);
    if (cols && cudaStreamSynchronize(c.stream) == cudaSuccess)  // best effort: the states back to the host
      cudaMemcpy2D(h, sizeof(cx<double>) * (size_t)ldh, d, sizeof(cx<double>) * (size_t)ngw,
                   sizeof(cx<double>) * (size_t)ngw, n, cudaMemcpyDeviceToHost);
    return rc;
  }
  for (int r = 0; r < R && !cols; ++r) {
    const int g0 = gb[r], g = gb[r + 1] - gb[r];
    GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.copy_out, done[r], 0));
    ProfScope ps_(c, "d2h_states", c.copy_out, 2);
    if (g > 0)
      GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(h + 2 * (size_t)g0, sizeof(cx<double>) * (size_t)ldh, d + g0,
                                         sizeof(cx<double>) * (size_t)ngw, sizeof(cx<double>) * (size_t)g, n,
                                         cudaMemcpyDeviceToHost, c.copy_out));
  }
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.copy_out));
  const int st = finish_status(c, scond_host);
  if (st && cols) {
    // a failed step by column blocks: the host array gets its states back from st_c0
    GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(h, sizeof(cx<double>) * (size_t)ldh, d, sizeof(cx<double>) * (size_t)ngw,
                                       sizeof(cx<double>) * (size_t)ngw, n, cudaMemcpyDeviceToHost, c.stream));
    GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  }
  return st;
}

int ortho_gs(Ctx& c, cx<double>* c0, int ldc, int nstate, double* scond_host) {
  if (nstate <= 0) return 0;
  const int rc = ortho_gs_steps(c, c0, ldc, nstate, scond_host != nullptr);
  if (rc) return rc;
  return finish_status(c, scond_host);
}

int ortho_gs_queue(Ctx& c, cx<double>* c0, int ldc, int nstate) {
  if (nstate <= 0) return 0;
  return ortho_gs_steps(c, c0, ldc, nstate, false);
}

int ortho_lowdin(Ctx& c, cx<double>* c0, int ldc, int nstate, double* scond_host) {
  const int n = nstate;
  if (n <= 0) return 0;
  if (n > 4096) {
    c.err = "ortho: nstate above 4096 not supported";
    return 7;
  }
  const size_t nn = (size_t)n * n;
  if (!ensure(c, c.smat, sizeof(double) * nn) || !ensure(c, c.smat2, sizeof(double) * nn * 3) ||
      !ensure(c, c.smat3, sizeof(double) * (nn + 8)))
    return 6;
  double* S = static_cast<double*>(c.smat.p);
  double* Y = static_cast<double*>(c.smat2.p);
  double* Z = Y + nn;
  double* T = Z + nn;
  double* W = static_cast<double*>(c.smat3.p);
  double* scal = W + nn;  // [0] alpha, [1] residual
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, 16, c.stream));
  int rc = ovlap_gamma_ex(c, c0, ldc, n, S, scond_host != nullptr);
  if (rc) return rc;
  if ((rc = finish_status(c, scond_host))) return rc;
  const int nbe = std::max(1, std::min(1024, (int)((nn + 255) / 256)));
  unsigned long long* bits = reinterpret_cast<unsigned long long*>(scal + 2);  // [0] alpha, [1] max|T - I|
  {
    ProfScope ps_(c, "k_ns_init");
    GBCP_CUDA_TRY(c, cudaMemsetAsync(bits, 0, 2 * sizeof(unsigned long long), c.stream));
    k_row_abs_max<<<std::max(1, std::min(1024, (n + 7) / 8)), 256, 0, c.stream>>>(S, n, bits);
    GBCP_LAUNCH_CHECK(c);
    k_ns_start<<<nbe, 256, 0, c.stream>>>(S, n, bits, Y, Z, scal);
    GBCP_LAUNCH_CHECK(c);
  }
  dim3 grid((n + TS - 1) / TS, (n + TS - 1) / TS);
  double prev = 1e300, res = 1e300;
  bool ok = false;
  const bool tc = use_tc_gemm(c);
  for (int it = 0; it < 100; ++it) {
    if (tc) {
      // the products on the tensor cores, FP64-accurate (split GEMM): column-major
      // A times row-major M; all of Y, Z, T are symmetric polynomials in S and commute,
      // so the transposed views give the same matrices
      GBCP_CUDA_TRY(c, cudaMemsetAsync(bits + 1, 0, sizeof(unsigned long long), c.stream));
      c.rmul_name = "k_ozaki_ns";  // the n x n x n products of the iteration, timed apart from C A
      rc = rmul_tc(c, Z, n, n, n, Y, 0, W, n, 0, c.d_info);  // W = Z Y
      c.rmul_name = nullptr;
      if (rc) return rc;
      {
        ProfScope ps_(c, "k_ns_t");
        k_ns_t<<<nbe, 256, 0, c.stream>>>(W, n, T, bits + 1);
        GBCP_LAUNCH_CHECK(c);
      }
      c.rmul_name = "k_ozaki_ns";
      rc = rmul_tc(c, Y, n, n, n, T, 0, W, n, 0, c.d_info);  // W = Y T
      if (!rc) {
        std::swap(Y, W);
        rc = rmul_tc(c, T, n, n, n, Z, 0, W, n, 0, c.d_info);  // W = T Z
        std::swap(Z, W);
      }
      c.rmul_name = nullptr;
      if (rc) return rc;
      unsigned long long hb = 0;
      GBCP_CUDA_TRY(c, cudaMemcpyAsync(&hb, bits + 1, sizeof(hb), cudaMemcpyDeviceToHost, c.stream));
      GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
      memcpy(&res, &hb, sizeof(res));
      if (!std::isfinite(res)) break;
      if (res < 1e-15 * std::max(1, n / 16) || (res < 1e-10 && res >= prev)) {
        ok = true;
        break;
      }
      prev = res;
      continue;
    }
    // T = (3 I - Z Y) / 2 ; Y <- Y T ; Z <- T Z
    {
      ProfScope ps_(c, "k_gemm_nn");
      k_gemm_nn<<<grid, NT, 0, c.stream>>>(Z, Y, T, n, -0.5, 0.0, 1.5);
      GBCP_LAUNCH_CHECK(c);
    }
    {
      ProfScope ps_(c, "k_gemm_nn");
      k_gemm_nn<<<grid, NT, 0, c.stream>>>(Y, T, W, n, 1.0, 0.0, 0.0);
      GBCP_LAUNCH_CHECK(c);
    }
    std::swap(Y, W);
    {
      ProfScope ps_(c, "k_gemm_nn");
      k_gemm_nn<<<grid, NT, 0, c.stream>>>(T, Z, W, n, 1.0, 0.0, 0.0);
      GBCP_LAUNCH_CHECK(c);
    }
    std::swap(Z, W);
    {
      ProfScope ps_(c, "k_dev_from_identity");
      GBCP_CUDA_TRY(c, cudaMemsetAsync(bits + 1, 0, sizeof(unsigned long long), c.stream));
      k_dev_from_identity<<<nbe, 256, 0, c.stream>>>(T, n, bits + 1);
      GBCP_LAUNCH_CHECK(c);
    }
    {
      unsigned long long hb = 0;
      GBCP_CUDA_TRY(c, cudaMemcpyAsync(&hb, bits + 1, sizeof(hb), cudaMemcpyDeviceToHost, c.stream));
      GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
      memcpy(&res, &hb, sizeof(res));
    }
    if (!std::isfinite(res)) break;
    // quadratic convergence ends at rounding level: stop when T = I to ~n eps
    // or when the deviation no longer drops
    if (res < 1e-15 * std::max(1, n / 16) || (res < 1e-10 && res >= prev)) {
      ok = true;
      break;
    }
    prev = res;
  }
  if (!ok) {
    c.err = "lowdin: Newton-Schulz iteration for S^-1/2 did not converge (S ill-conditioned or not SPD)";
    return std::isfinite(res) ? 8 : 3;
  }
  // A = Z / sqrt(alpha)
  {
    ProfScope ps_(c, "k_scale");
    k_scale<<<256, 256, 0, c.stream>>>(Z, nn, scal, -0.5);
    GBCP_LAUNCH_CHECK(c);
  }
  if ((rc = apply_right(c, c0, ldc, n, Z, 0))) return rc;
  return finish_status(c, nullptr);
}

}  // namespace gbcp

// ---------------------------------------------------------------------------
// Allocation-free overlap matrix: gbcp_ovlap_noalloc.
//
// Some callers of this library cannot call cudaMalloc: an application whose
// device memory is owned by its own pool allocator (every byte handed out by
// that pool), or a time-stepping loop that must not stall every stream on the
// device with the implicit synchronisation an allocation brings.  For them
// this entry point computes the same Γ-point overlap matrix as gbcp_ovlap but
// allocates nothing: the caller passes device pointers for the wavefunctions
// and the result, and the split-K partial sums live in the fixed device array
// below.  That array (8 MiB, room for nsplit * nstate^2 <= 2^20 doubles, so
// nstate <= 1024) is part of the library image: every GPU that loads the
// library holds it until the process exits.  All calls share it and it keeps
// the last call's contents; the kernels overwrite every partial they later
// read, so nothing needs clearing.  Calls whose work overlaps on the GPU
// (different streams, or several host threads) race on the array.
namespace gbcp {

static __device__ __align__(256) double g_noalloc_scratch[size_t(1) << 20];

namespace {
constexpr size_t kNoAllocDoubles = size_t(1) << 20;
constexpr int kNoAllocSlots = 64;

// The array's device address belongs to the module as loaded into one CUDA
// context: a cudaDeviceReset, or a caller's own driver-API context on the same
// device, loads the module again at another address.  So the address is looked
// up once per context and remembered under the context's process-unique id
// (cuCtxGetId, reached through the runtime's driver entry points so that no
// driver library is linked), never under the device ordinal.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);
struct NoAllocSlot {
  unsigned long long ctx_id = 0;
  double* ptr = nullptr;
};
NoAllocSlot g_noalloc_slots[kNoAllocSlots];
int g_noalloc_next = 0;
std::mutex g_noalloc_mu;
PfnCtxGetCurrent g_ctx_current = nullptr;
PfnCtxGetId g_ctx_id = nullptr;
bool g_entry_looked_up = false;

// id of the current context; false when it cannot be told (then the address
// is looked up on every call, which is always correct)
bool current_ctx_id(unsigned long long* id) {
  if (!g_entry_looked_up) {
    g_entry_looked_up = true;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      g_ctx_current = reinterpret_cast<PfnCtxGetCurrent>(f1);
      g_ctx_id = reinterpret_cast<PfnCtxGetId>(f2);
    }
  }
  if (!g_ctx_current || !g_ctx_id) return false;
  CUcontext cx = nullptr;
  if (g_ctx_current(&cx) != CUDA_SUCCESS || cx == nullptr) return false;
  return g_ctx_id(cx, id) == CUDA_SUCCESS && *id != 0;
}

// Device address of the scratch array in the current context.  The host-side
// name g_noalloc_scratch is only a stand-in for the symbol, not a device
// address, so it is resolved with cudaGetSymbolAddress (which allocates
// nothing; on a context's first use it loads the module, which is why the
// first call in a context should come before any stream capture).
int noalloc_scratch(double** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned long long id = 0;
  const bool known = current_ctx_id(&id);
  if (known) {
    for (const NoAllocSlot& s : g_noalloc_slots)
      if (s.ctx_id == id) {
        *out = s.ptr;
        return 0;
      }
  }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return 5;
  *out = static_cast<double*>(p);
  // the lookup may have made the primary context current just now
  if (known || current_ctx_id(&id)) {
    g_noalloc_slots[g_noalloc_next] = {id, *out};
    g_noalloc_next = (g_noalloc_next + 1) % kNoAllocSlots;
  }
  return 0;
}
}  // namespace

}  // namespace gbcp

extern "C" int gbcp_ovlap_noalloc(const double* c0, int ldc, int ngw, int nstate, int geq0, double* smat,
                                  void* stream) {
  using namespace gbcp;
  if (!c0 || !smat || ngw < 1 || ldc < ngw || nstate < 1) return 1;
  const int n = nstate;
  const size_t nn = (size_t)n * n;
  if (nn > kNoAllocDoubles) return 1;  // nstate above 1024
  // an error the caller left pending is theirs: report it without launching,
  // so that the launch checks below see only this call's own errors
  if (cudaPeekAtLastError() != cudaSuccess) return 5;
  double* scratch = nullptr;
  if (noalloc_scratch(&scratch)) return 5;
  const int K = 2 * ngw, lda = 2 * ldc;
  const int ntb = (n + TS - 1) / TS;
  const int npairs = ntb * (ntb + 1) / 2;
  int nsplit = std::max(1, std::min(1024, (4 * 152 + npairs - 1) / npairs));
  nsplit = std::max(1, std::min(nsplit, (int)(kNoAllocDoubles / nn)));
  int kchunk = (K + nsplit - 1) / nsplit;
  kchunk = ((kchunk + BK - 1) / BK) * BK;
  nsplit = (K + kchunk - 1) / kchunk;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_syrk_part<TS><<<dim3(npairs, nsplit), NT, 0, st>>>(c0, lda, K, n, ntb, kchunk, scratch);
  count_launch();
  if (cudaGetLastError() != cudaSuccess) return 5;
  const int fb = std::max(1, std::min(1024, (int)((nn + 255) / 256)));
  k_syrk_fold<<<fb, 256, 0, st>>>(scratch, nsplit, n, TS, c0, lda, geq0 ? 1 : 0, smat, nullptr);
  count_launch();
  if (cudaGetLastError() != cudaSuccess) return 5;
  return 0;
}
