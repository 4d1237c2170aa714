// Γ-point overlap matrix S = 2 Re(C^H C) - Re c(0) Re c(0)^T on the tcgen05
// tensor cores, to FP64 accuracy, by error-free splitting (after Ozaki, Ogita,
// Oishi and Rump, "Error-free transformations of matrix multiplication by using
// fast routines of matrix multiplication and its applications", Numer.
// Algorithms 59, 2012; arranged here for bf16 MMAs with FP32 accumulators).
//
// Reference: rgs_utils.mod.F90:63-68 / ovlap_utils.mod.F90:150-165 (dsyrk over
// the real view of C, K = 2 ngw, then dger for G = 0).
//
// Splitting.  Every state column j has an exponent E_j with |a_kj| < 2^E_j.
// Each element becomes the 56-bit fixed-point magnitude v = trunc(|a| 2^(56-E_j))
// cut into 8 signed 7-bit digits m_s (s = 0 most significant), so
// a = 2^E_j sum_s m_s 2^(-7(s+1)) up to 2^(E_j-56).  A digit is an integer in
// [-127, 127]: exact in bf16, and a digit product is exact in FP32.
//
// Products.  For a 128 x 64 output tile the CTA runs, per K-chunk of 128 real
// rows, the 36 digit-pair products with s + t = d <= 7 (level d), accumulating
// every pair of one level in one FP32 TMEM accumulator (8 accumulators x 64
// columns = all 512 TMEM columns).  A level sum is an integer below
// 8 * 128 * 127^2 < 2^24, so FP32 holds it exactly.  After each chunk the
// accumulators are read back and folded into two int64 registers per output
// (H = levels 0-3, Lo = levels 4-7, shifted by 7 bits per level); int64 keeps
// the sum over all chunks exact.  Split-K partials are added with 64-bit
// integer atomics, and only the final conversion is FP64:
//   sum_k a_ki a_kj = 2^(E_i+E_j) (H 2^-35 + Lo 2^-63).
// Levels above 7 (digit pairs beyond 56 bits) are dropped: < 2^-49 relative to
// 2^(E_i+E_j) per product term.
//
// The digits are produced in the kernel from FP64 data with integer
// instructions and stored straight into shared memory in the tensor core's
// K-major core-matrix layout: no slice matrices in HBM, no FP64 arithmetic in
// the inner loop.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ctx.h"
#include "tc_common.cuh"

namespace gbcp {

namespace {

constexpr int OZ_M = 128;      // output rows per CTA (states i)
constexpr int OZ_N = 64;       // output columns per CTA (states j)
constexpr int OZ_KS = 32;      // real K rows per sub-chunk (two MMAs of K = 16)
constexpr int OZ_SUBS = 4;     // sub-chunks per exact accumulation chunk (K = 128)
constexpr int OZ_SL = 8;       // digit slices
constexpr int OZ_LEV = 8;      // levels kept (s + t <= 7)
constexpr int OZ_THREADS = 256;
constexpr int A_SLICE_BYTES = OZ_M * OZ_KS * 2;  // 8 KB
constexpr int B_SLICE_BYTES = OZ_N * OZ_KS * 2;  // 4 KB
constexpr int A_BUF_BYTES = OZ_SL * A_SLICE_BYTES;
constexpr int B_BUF_BYTES = OZ_SL * B_SLICE_BYTES;
constexpr int OZ_SMEM = 2 * A_BUF_BYTES + 2 * B_BUF_BYTES;  // 192 KB, double-buffered

// byte offset of (row, k-group) core-matrix row in a K-major no-swizzle tile of 32 K
__device__ __forceinline__ int core_off(int row, int kg) { return (((row >> 3) << 2) + kg) * 128 + (row & 7) * 16; }

// signed 7-bit digit -> bf16 bits (exact: |d| <= 127)
__device__ __forceinline__ uint32_t digit_bf16(int d) { return __float_as_uint((float)d) >> 16; }

// Fixed-point magnitude trunc(|a| 2^(56-E)) (< 2^56) and the sign of a, integer ops only.
__device__ __forceinline__ unsigned long long fixed56(double a, int E, bool& neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0) return 0ull;  // zero or subnormal
  const unsigned long long M = (b & ((1ull << 52) - 1)) | (1ull << 52);
  int sh = ex - 1019 - E;  // = (ex - 1023) + 4 - E
  if (sh > 3) sh = 3;      // cannot happen when |a| < 2^E; keeps v < 2^56
  if (sh >= 0) return M << sh;
  return (sh <= -64) ? 0ull : (M >> (-sh));
}

// Produce the 8 digit slices of rows [r0, r0+rows) x K [kb, kb+32) into smem.
__device__ __forceinline__ void produce(const double* __restrict__ Ar, int lda, int K, int n, int kb, int s0,
                                        int rows, const int* __restrict__ E, uint8_t* __restrict__ dst,
                                        int slice_bytes) {
  // task = (row, kg): 4 k-groups of 8 per row; consecutive threads read consecutive k-groups
  for (int task = threadIdx.x; task < rows * 4; task += OZ_THREADS) {
    const int row = task >> 2, kg = task & 3;
    const int state = s0 + row;
    const bool valid = state < n;
    const int e = valid ? E[state] : 0;
    uint32_t w[OZ_SL][4];
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2) {
      const int k = kb + kg * 8 + 2 * q2;
      double2 v2 = make_double2(0.0, 0.0);
      if (valid && k < K) v2 = *reinterpret_cast<const double2*>(Ar + k + (size_t)state * lda);
      bool n0, n1;
      const unsigned long long f0 = fixed56(v2.x, e, n0), f1 = fixed56(v2.y, e, n1);
#pragma unroll
      for (int s = 0; s < OZ_SL; ++s) {
        const int sh = 7 * (OZ_SL - 1 - s);
        const int d0 = (int)((f0 >> sh) & 127ull), d1 = (int)((f1 >> sh) & 127ull);
        w[s][q2] = digit_bf16(n0 ? -d0 : d0) | (digit_bf16(n1 ? -d1 : d1) << 16);
      }
    }
    const int off = core_off(row, kg);
#pragma unroll
    for (int s = 0; s < OZ_SL; ++s) {
      *reinterpret_cast<uint4*>(dst + s * slice_bytes + off) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
  }
}

// Per-state exponent: E_j = unbiased exponent of max_k |a_kj| + 1 (so |a| < 2^E).
__global__ void k_col_exp(const double* __restrict__ Ar, int lda, int K, int n, int* __restrict__ E) {
  const int j = blockIdx.x;
  unsigned long long mx = 0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(Ar[k + (size_t)j * lda]) & ~(1ull << 63);
    mx = b > mx ? b : mx;
  }
  __shared__ unsigned long long red[256];
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = red[threadIdx.x] > red[threadIdx.x + s] ? red[threadIdx.x] : red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int ex = (int)((red[0] >> 52) & 0x7FF);
    E[j] = (ex == 0) ? -1021 : ex - 1023 + 1;
  }
}

__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_ozaki_syrk(const double* __restrict__ Ar, int lda, int K, int n, const int* __restrict__ E, int njb,
                 int subs_per_split, unsigned long long* __restrict__ Hacc, unsigned long long* __restrict__ Lacc,
                 int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t* sA = sm;
  uint8_t* sB = sm + 2 * A_BUF_BYTES;
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;

  // tile (ib, jb) among those touching the upper triangle: jb >= 2 ib
  int t = blockIdx.x, ib = 0;
  while (ib < 4096 && t >= max(0, njb - 2 * ib)) {
    t -= max(0, njb - 2 * ib);
    ++ib;
  }
  if (ib >= 4096) return;
  const int i0 = ib * OZ_M, j0 = (2 * ib + t) * OZ_N;
  const int total_subs = (K + OZ_KS - 1) / OZ_KS;
  const int sub0 = blockIdx.y * subs_per_split;
  const int nsub = min(total_subs, sub0 + subs_per_split) - sub0;
  if (nsub <= 0) return;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    tc::tmem_alloc(&tmem_sh, 512);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::fence_mbar_init();
    abort_sh = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_sh;

  long long H[32], Lo[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    H[c] = 0;
    Lo[c] = 0;
  }
  constexpr uint32_t idesc = tc::idesc_bf16_f32(OZ_M, OZ_N);
  uint32_t ph[2] = {0u, 0u};
  int pend[2] = {0, 0};
  bool done_ok = true;

  for (int it = 0; it < nsub; ++it) {
    const int buf = it & 1;
    if (pend[buf]) {
      if (!tc::mbar_wait(&mbar[buf], ph[buf])) {
        abort_sh = 1;
        atomicExch(err, 4);
      }
      ph[buf] ^= 1u;
      pend[buf] = 0;
    }
    __syncthreads();
    if (abort_sh) {
      done_ok = false;
      break;
    }
    const int kb = (sub0 + it) * OZ_KS;
    uint8_t* a_dst = sA + buf * A_BUF_BYTES;
    uint8_t* b_dst = sB + buf * B_BUF_BYTES;
    produce(Ar, lda, K, n, kb, i0, OZ_M, E, a_dst, A_SLICE_BYTES);
    produce(Ar, lda, K, n, kb, j0, OZ_N, E, b_dst, B_SLICE_BYTES);
    tc::fence_proxy_async();
    __syncthreads();
    const int ci = it % OZ_SUBS;
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      const uint32_t a_base = tc::smem_u32(a_dst), b_base = tc::smem_u32(b_dst);
#pragma unroll 1
      for (int d = 0; d < OZ_LEV; ++d) {
        const uint32_t dt = tmem + (uint32_t)(OZ_N * d);
#pragma unroll 1
        for (int s = 0; s <= d; ++s) {
          const int u = d - s;
#pragma unroll
          for (int kk = 0; kk < 2; ++kk) {
            const uint64_t ad = tc::sdesc_kmajor(a_base + s * A_SLICE_BYTES + kk * 256, 128, 512);
            const uint64_t bd = tc::sdesc_kmajor(b_base + u * B_SLICE_BYTES + kk * 256, 128, 512);
            tc::mma_f16(dt, ad, bd, idesc, (ci == 0 && s == 0 && kk == 0) ? 0u : 1u);
          }
        }
      }
      tc::mma_commit(&mbar[buf]);
    }
    pend[buf] = 1;
    if (ci == OZ_SUBS - 1 || it == nsub - 1) {
      bool ok = tc::mbar_wait(&mbar[buf], ph[buf]);
      ph[buf] ^= 1u;
      pend[buf] = 0;
      if (pend[buf ^ 1]) {
        ok = tc::mbar_wait(&mbar[buf ^ 1], ph[buf ^ 1]) && ok;
        ph[buf ^ 1] ^= 1u;
        pend[buf ^ 1] = 0;
      }
      if (!ok) {
        abort_sh = 1;
        atomicExch(err, 4);
      }
      __syncthreads();
      if (abort_sh) {
        done_ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint32_t lane_base = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * (warp >> 2));
#pragma unroll 1
      for (int d = 0; d < OZ_LEV; ++d) {
        uint32_t r[32];
        tc::tmem_ld32(lane_base + (uint32_t)(OZ_N * d), r);
        tc::tmem_ld_wait();
        const int sh = 7 * (3 - (d & 3));
        if (d < 4) {
#pragma unroll
          for (int c = 0; c < 32; ++c) H[c] += (long long)__float2int_rn(__uint_as_float(r[c])) * (1ll << sh);
        } else {
#pragma unroll
          for (int c = 0; c < 32; ++c) Lo[c] += (long long)__float2int_rn(__uint_as_float(r[c])) * (1ll << sh);
        }
      }
      tc::fence_before_sync();
      __syncthreads();
    }
  }

  if (done_ok) {
    const int row = i0 + 32 * (warp & 3) + lane;
    if (row < n) {
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int col = j0 + 32 * (warp >> 2) + c;
        if (col < n) {
          atomicAdd(Hacc + (size_t)row * n + col, (unsigned long long)H[c]);
          atomicAdd(Lacc + (size_t)row * n + col, (unsigned long long)Lo[c]);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc::tmem_dealloc(tmem, 512);
  }
}

// S[i][j] (i <= j, mirrored) = 2 * 2^(E_i+E_j) (H 2^-35 + Lo 2^-63) - Re c0_i Re c0_j
__global__ void k_ozaki_syrk_finalize(const long long* __restrict__ H, const long long* __restrict__ Lo,
                                      const int* __restrict__ E, int n, const double* __restrict__ Ar, int lda,
                                      int geq0, double* __restrict__ S, unsigned long long* __restrict__ scond_bits) {
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (i > j) continue;
    const int ee = E[i] + E[j];
    double v = ldexp((double)H[e], ee - 35) + ldexp((double)Lo[e], ee - 63);
    v *= 2.0;
    if (geq0) v -= Ar[(size_t)i * lda] * Ar[(size_t)j * lda];
    S[(size_t)i * n + j] = v;
    S[(size_t)j * n + i] = v;
    mx = fmax(mx, fabs(i == j ? v - 1.0 : v));
  }
  if (scond_bits) {
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(scond_bits, (unsigned long long)__double_as_longlong(mx));
  }
}

}  // namespace

// Overlap matrix on the tensor cores; scond (max|S-I|) if scond_host.
int ovlap_tc(Ctx& c, const cx<double>* c0, int ldc, int nstate, double* S, double* scond_host) {
  const int n = nstate;
  const int K = 2 * c.ngw;
  const int lda = 2 * ldc;
  const double* Ar = reinterpret_cast<const double*>(c0);
  const int nib = (n + OZ_M - 1) / OZ_M;
  const int njb = (n + OZ_N - 1) / OZ_N;
  int ntiles = 0;
  for (int ib = 0; ib < nib; ++ib) ntiles += std::max(0, njb - 2 * ib);
  const int total_subs = (K + OZ_KS - 1) / OZ_KS;
  int nsplit = std::max(1, std::min((total_subs + OZ_SUBS - 1) / OZ_SUBS, 148 / std::max(1, ntiles)));
  int subs_per = (total_subs + nsplit - 1) / nsplit;
  subs_per = ((subs_per + OZ_SUBS - 1) / OZ_SUBS) * OZ_SUBS;
  nsplit = (total_subs + subs_per - 1) / subs_per;
  const size_t nn = (size_t)n * n;
  // workspace: H, Lo (int64 n*n each), E (n ints), err, scond bits
  const size_t bytes = 2 * nn * 8 + (size_t)n * 4 + 64;
  if (!ensure(c, c.sparts, bytes)) return 6;
  unsigned long long* Hacc = static_cast<unsigned long long*>(c.sparts.p);
  unsigned long long* Lacc = Hacc + nn;
  int* E = reinterpret_cast<int*>(Lacc + nn);
  int* err = E + n;
  unsigned long long* bits = reinterpret_cast<unsigned long long*>(err + 2 + (n & 1));
  GBCP_CUDA_TRY(c, cudaMemsetAsync(Hacc, 0, bytes, c.stream));
  {
    ProfScope ps_(c, "k_col_exp");
    k_col_exp<<<n, 256, 0, c.stream>>>(Ar, lda, K, n, E);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    static bool attr_set = false;
    if (!attr_set) {
      cudaFuncSetAttribute(k_ozaki_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM);
      attr_set = true;
    }
    ProfScope ps_(c, "k_ozaki_syrk");
    k_ozaki_syrk<<<dim3(ntiles, nsplit), OZ_THREADS, OZ_SMEM, c.stream>>>(Ar, lda, K, n, E, njb, subs_per, Hacc, Lacc,
                                                                          err);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_ozaki_syrk_finalize");
    const int fb = std::max(1, std::min(1024, (int)((nn + 255) / 256)));
    k_ozaki_syrk_finalize<<<fb, 256, 0, c.stream>>>(reinterpret_cast<const long long*>(Hacc),
                                                    reinterpret_cast<const long long*>(Lacc), E, n, Ar, lda, c.geq0, S,
                                                    scond_host ? bits : nullptr);
    GBCP_LAUNCH_CHECK(c);
  }
  int herr = 0;
  unsigned long long hb = 0;
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  if (scond_host) GBCP_CUDA_TRY(c, cudaMemcpyAsync(&hb, bits, sizeof(hb), cudaMemcpyDeviceToHost, c.stream));
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (herr) {
    c.err = "ovlap (tensor cores): an mbarrier wait timed out";
    return 4;
  }
  if (scond_host) {
    double d;
    memcpy(&d, &hb, sizeof(d));
    *scond_host = d;
  }
  return 0;
}

}  // namespace gbcp
