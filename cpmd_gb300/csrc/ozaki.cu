// FP64-accurate GEMMs of the ortho step on the tcgen05 tensor cores, by
// error-free splitting (after Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012; arranged
// here for bf16 MMAs with FP32 accumulators and int64 folding).
//
//  * ovlap_tc: S = 2 Re(C^H C) - Re c(0) Re c(0)^T over the real view of C
//    (K = 2 ngw) -- rgs_utils.mod.F90:63-68, ovlap_utils.mod.F90:150-165.
//  * rmul_tc:  C <- C M for an n x n matrix M (U^{-1} of Gram-Schmidt, upper
//    triangular, rgs_utils.mod.F90:71-73; or S^{-1/2} of Loewdin,
//    lowdin_utils.mod.F90:81-83).
//
// Splitting.  Every row of the left operand and every column of the right
// operand has an exponent E with |x| < 2^E (row/column maxima).  An element
// becomes the 56-bit fixed-point magnitude v = trunc(|x| 2^(56-E)), cut into 8
// signed 7-bit digits m_s (s = 0 most significant): x = 2^E sum_s m_s 2^(-7(s+1))
// up to 2^(E-56).  A digit is an integer in [-127, 127] -- exact in bf16 -- and
// a digit product is exact in FP32.
//
// Products.  For a 128 x 64 output tile the CTA runs, per K-chunk of 128, the
// 36 digit-pair products with s + t = d <= 7 ("level" d), accumulating all pairs
// of a level in one FP32 TMEM accumulator (8 levels x 64 columns = the 512 TMEM
// columns).  A level sum is an integer below 8 * 128 * 127^2 < 2^24, so FP32
// holds it exactly.  After each chunk the accumulators are read back and folded
// into two int64 registers per output (H = levels 0-3, Lo = levels 4-7, 7 bits
// apart); int64 keeps the sum over every chunk exact and only the final
// conversion is FP64:  sum_k x_ik y_kj = 2^(E_i+E_j) (H 2^-35 + Lo 2^-63).
// Levels above 7 are dropped (< 2^-49 of 2^(E_i+E_j) per product term).
//
// The digits are produced in the kernels from FP64 data with integer
// instructions and stored straight into shared memory in the tensor core's
// K-major core-matrix layout: no slice matrices in HBM, no FP64 arithmetic in
// the inner loop.  Every mbarrier wait is bounded; on expiry the kernel sets
// the ortho status word to -2 (reported as GBCP_ERR_TIMEOUT), frees its TMEM
// and returns.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ctx.h"
#include "tc_common.cuh"

namespace gbcp {

namespace {

constexpr int OZ_M = 128;      // output rows per tile
constexpr int OZ_N = 64;       // output columns per tile
constexpr int OZ_KS = 32;      // K per sub-chunk (two MMAs of K = 16)
constexpr int OZ_SUBS = 4;     // sub-chunks per exact accumulation chunk (K = 128)
constexpr int OZ_SL = 8;       // digit slices
constexpr int OZ_LEV = 8;      // levels kept (s + t <= 7)
constexpr int OZ_THREADS = 256;
constexpr int A_SLICE_BYTES = OZ_M * OZ_KS * 2;  // 8 KB
constexpr int B_SLICE_BYTES = OZ_N * OZ_KS * 2;  // 4 KB
constexpr int A_BUF_BYTES = OZ_SL * A_SLICE_BYTES;
constexpr int B_BUF_BYTES = OZ_SL * B_SLICE_BYTES;
constexpr int OZ_SMEM = 2 * A_BUF_BYTES + 2 * B_BUF_BYTES;  // 192 KB, double-buffered
constexpr uint32_t kIdesc = tc::idesc_bf16_f32(OZ_M, OZ_N);

// byte offset of the (row, k-group) core-matrix row in a K-major no-swizzle tile of 32 K
__device__ __forceinline__ int core_off(int row, int kg) { return (((row >> 3) << 2) + kg) * 128 + (row & 7) * 16; }

// signed 7-bit digit -> bf16 bits (exact: |d| <= 127)
__device__ __forceinline__ uint32_t digit_bf16(int d) { return __float_as_uint((float)d) >> 16; }

// exponent E with |x| < 2^E from the bit pattern of max |x|
__device__ __forceinline__ int exp_of_max(unsigned long long bits) {
  const int ex = (int)((bits >> 52) & 0x7FF);
  return (ex == 0) ? -1021 : ex - 1022;
}

// Fixed-point magnitude trunc(|x| 2^(56-E)) (< 2^56) and the sign, integer ops only.
__device__ __forceinline__ unsigned long long fixed56(double x, int E, bool& neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0) return 0ull;  // zero or subnormal
  const unsigned long long M = (b & ((1ull << 52) - 1)) | (1ull << 52);
  int sh = ex - 1019 - E;  // = (ex - 1023) + 4 - E
  if (sh > 3) sh = 3;      // cannot happen when |x| < 2^E; keeps v < 2^56
  if (sh >= 0) return M << sh;
  return (sh <= -64) ? 0ull : (M >> (-sh));
}

// Digits of 8 consecutive K elements of one operand row -> 8 slices x 16 bytes in smem.
__device__ __forceinline__ void store_digits(const double (&x)[8], int E, uint8_t* dst, int slice_bytes, int off) {
  uint32_t w[OZ_SL][4];
#pragma unroll
  for (int q2 = 0; q2 < 4; ++q2) {
    bool n0, n1;
    const unsigned long long f0 = fixed56(x[2 * q2], E, n0), f1 = fixed56(x[2 * q2 + 1], E, n1);
#pragma unroll
    for (int s = 0; s < OZ_SL; ++s) {
      const int sh = 7 * (OZ_SL - 1 - s);
      const int d0 = (int)((f0 >> sh) & 127ull), d1 = (int)((f1 >> sh) & 127ull);
      w[s][q2] = digit_bf16(n0 ? -d0 : d0) | (digit_bf16(n1 ? -d1 : d1) << 16);
    }
  }
#pragma unroll
  for (int s = 0; s < OZ_SL; ++s)
    *reinterpret_cast<uint4*>(dst + s * slice_bytes + off) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// Issue the 72 MMAs of one sub-chunk (36 digit pairs x 2 K-steps) into the 8
// level accumulators; `first` restarts the accumulators (chunk start).
__device__ __forceinline__ void issue_levels(uint32_t tmem, uint32_t a_base, uint32_t b_base, bool first) {
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
        tc::mma_f16(dt, ad, bd, kIdesc, (first && s == 0 && kk == 0) ? 0u : 1u);
      }
    }
  }
}

// Fold the 8 level accumulators of this thread's TMEM lane, 32 columns, into H / Lo.
__device__ __forceinline__ void fold_levels(uint32_t lane_base, long long (&H)[32], long long (&Lo)[32]) {
#pragma unroll 1
  for (int d = 0; d < OZ_LEV; ++d) {
    uint32_t r[32];
    tc::tmem_ld32(lane_base + (uint32_t)(OZ_N * d), r);
    tc::tmem_ld_wait();
    const long long m = 1ll << (7 * (3 - (d & 3)));
    if (d < 4) {
#pragma unroll
      for (int c = 0; c < 32; ++c) H[c] += (long long)__float2int_rn(__uint_as_float(r[c])) * m;
    } else {
#pragma unroll
      for (int c = 0; c < 32; ++c) Lo[c] += (long long)__float2int_rn(__uint_as_float(r[c])) * m;
    }
  }
}

// (H 2^28 + Lo) 2^(ee-63) as a correctly rounded double, with integer
// instructions only (the FP64 pipe, 1/58 of FP32 on GB300, would otherwise
// bound the epilogue).  Results below the normal range flush to zero.
__device__ __forceinline__ double fold_to_double(long long H, long long Lo, int ee) {
  __int128 v = ((__int128)H << 28) + (__int128)Lo;
  const bool neg = v < 0;
  unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  if (m == 0) return 0.0;
  const unsigned long long hi = (unsigned long long)(m >> 64), lo = (unsigned long long)m;
  int top = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);  // index of the leading bit
  unsigned long long mant;
  const int sh = top - 52;
  if (sh > 0) {
    mant = (unsigned long long)(m >> sh);
    const unsigned __int128 rem = m & (((unsigned __int128)1 << sh) - 1);
    const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) {
      if (++mant == (1ull << 53)) {
        mant >>= 1;
        ++top;
      }
    }
  } else {
    mant = lo << (-sh);
  }
  const int be = top + ee - 63 + 1023;
  if (be <= 0) return neg ? -0.0 : 0.0;
  if (be >= 2047) return __longlong_as_double((long long)((neg ? (1ull << 63) : 0ull) | 0x7FF0000000000000ull));
  const unsigned long long bits =
      (neg ? (1ull << 63) : 0ull) | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

// ---------------------------------------------------------------- exponent pre-passes
// column maxima |a_kj| over k (state columns of the real view): bits into cmax[j]
__global__ void k_col_max(const double* __restrict__ Ar, int lda, int K, int n, int kper,
                          unsigned long long* __restrict__ cmax) {
  const int j = blockIdx.x;
  const int k0 = blockIdx.y * kper, k1 = min(K, k0 + kper);
  unsigned long long mx = 0;
  for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(Ar[k + (size_t)j * lda]) & ~(1ull << 63);
    mx = b > mx ? b : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_down_sync(0xffffffffu, mx, o);
    mx = v > mx ? v : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(cmax + j, mx);
}

// row maxima of the real view over the n states: bits into rmax[r]
__global__ void k_row_max(const double* __restrict__ Ar, int lda, int rows, int n,
                          unsigned long long* __restrict__ rmax) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  unsigned long long mx = 0;
  for (int k = 0; k < n; ++k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(Ar[r + (size_t)k * lda]) & ~(1ull << 63);
    mx = b > mx ? b : mx;
  }
  rmax[r] = mx;
}

// column maxima of a small row-major n x n matrix M over its rows
__global__ void k_mat_col_max(const double* __restrict__ M, int n, unsigned long long* __restrict__ cmax) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  unsigned long long mx = 0;
  for (int k = 0; k < n; ++k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(M[(size_t)k * n + j]) & ~(1ull << 63);
    mx = b > mx ? b : mx;
  }
  cmax[j] = mx;
}

// ---------------------------------------------------------------- S = C^T C (real view)
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_ozaki_syrk(const double* __restrict__ Ar, int lda, int K, int n, const unsigned long long* __restrict__ cmax,
                 int njb, int subs_per_split, unsigned long long* __restrict__ Hacc,
                 unsigned long long* __restrict__ Lacc, int* __restrict__ status) {
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
  const uint32_t lane_base = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * (warp >> 2));

  long long H[32], Lo[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    H[c] = 0;
    Lo[c] = 0;
  }
  uint32_t ph[2] = {0u, 0u};
  int pend[2] = {0, 0};
  bool done_ok = true;

  for (int it = 0; it < nsub; ++it) {
    const int buf = it & 1;
    if (pend[buf]) {
      if (!tc::mbar_wait(&mbar[buf], ph[buf])) {
        abort_sh = 1;
        atomicExch(status, -2);
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
    // A: 128 state rows, B: 64 state rows; task = (row, k-group of 8), k contiguous in memory
    for (int task = threadIdx.x; task < (OZ_M + OZ_N) * 4; task += OZ_THREADS) {
      const bool isA = task < OZ_M * 4;
      const int tt = isA ? task : task - OZ_M * 4;
      const int row = tt >> 2, kg = tt & 3;
      const int state = (isA ? i0 : j0) + row;
      const bool valid = state < n;
      const int e = valid ? exp_of_max(cmax[state]) : 0;
      double x[8];
#pragma unroll
      for (int q2 = 0; q2 < 4; ++q2) {
        const int k = kb + kg * 8 + 2 * q2;
        double2 v2 = make_double2(0.0, 0.0);
        if (valid && k < K) v2 = *reinterpret_cast<const double2*>(Ar + k + (size_t)state * lda);
        x[2 * q2] = v2.x;
        x[2 * q2 + 1] = v2.y;
      }
      store_digits(x, e, isA ? a_dst : b_dst, isA ? A_SLICE_BYTES : B_SLICE_BYTES, core_off(row, kg));
    }
    tc::fence_proxy_async();
    __syncthreads();
    const int ci = it % OZ_SUBS;
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      issue_levels(tmem, tc::smem_u32(a_dst), tc::smem_u32(b_dst), ci == 0);
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
        atomicExch(status, -2);
      }
      __syncthreads();
      if (abort_sh) {
        done_ok = false;
        break;
      }
      tc::fence_after_sync();
      fold_levels(lane_base, H, Lo);
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
                                      const unsigned long long* __restrict__ cmax, int n,
                                      const double* __restrict__ Ar, int lda, int geq0, double* __restrict__ S,
                                      unsigned long long* __restrict__ scond_bits) {
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (i > j) continue;
    double v = 2.0 * fold_to_double(H[e], Lo[e], exp_of_max(cmax[i]) + exp_of_max(cmax[j]));
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

// ---------------------------------------------------------------- Cout = A M (persistent over tiles)
// A: real view (rows x n, column-major, lda); M: n x n row-major; Cout column-major (ldo).
// upper: M is upper triangular, column tile j only needs k < j0 + 64.
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_ozaki_rmul(const double* __restrict__ A, int lda, int rows, int n, const double* __restrict__ M, int upper,
                 const unsigned long long* __restrict__ rmax, const unsigned long long* __restrict__ mcmax,
                 double* __restrict__ Cout, int ldo, int* __restrict__ status) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t* sA = sm;
  uint8_t* sB = sm + 2 * A_BUF_BYTES;
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;

  const int nrt = (rows + OZ_M - 1) / OZ_M, nct = (n + OZ_N - 1) / OZ_N;
  const int ntiles = nrt * nct;
  if ((int)blockIdx.x >= ntiles) return;
  if (*(volatile const int*)status != 0) return;  // an earlier step of this ortho failed
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
  const uint32_t lane_base = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * (warp >> 2));
  uint32_t ph[2] = {0u, 0u};
  int pend[2] = {0, 0};
  int it = 0;

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    // column tile outer so that consecutive CTAs share the M slices of a column tile
    const int ct = tile / nrt, rt = tile % nrt;
    const int r0 = rt * OZ_M, j0 = ct * OZ_N;
    const int kmax = upper ? min(n, j0 + OZ_N) : n;
    const int nsub = (kmax + OZ_KS - 1) / OZ_KS;
    long long H[32], Lo[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      H[c] = 0;
      Lo[c] = 0;
    }
    for (int s = 0; s < nsub; ++s, ++it) {
      const int buf = it & 1;
      if (pend[buf]) {
        if (!tc::mbar_wait(&mbar[buf], ph[buf])) {
          abort_sh = 1;
          atomicExch(status, -2);
        }
        ph[buf] ^= 1u;
        pend[buf] = 0;
      }
      __syncthreads();
      if (abort_sh) break;
      const int kb = s * OZ_KS;
      uint8_t* a_dst = sA + buf * A_BUF_BYTES;
      uint8_t* b_dst = sB + buf * B_BUF_BYTES;
      // A rows r (consecutive threads -> consecutive r: coalesced), 8 k each
      for (int task = threadIdx.x; task < OZ_M * 4; task += OZ_THREADS) {
        const int row = task & (OZ_M - 1), kg = task >> 7;
        const int r = r0 + row;
        const bool valid = r < rows;
        const int e = valid ? exp_of_max(rmax[r]) : 0;
        double x[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int k = kb + kg * 8 + q;
          x[q] = (valid && k < n) ? A[r + (size_t)k * lda] : 0.0;
        }
        store_digits(x, e, a_dst, A_SLICE_BYTES, core_off(row, kg));
      }
      // B rows j = columns of M: B[j][k] = M[k][j]
      for (int task = threadIdx.x; task < OZ_N * 4; task += OZ_THREADS) {
        const int row = task & (OZ_N - 1), kg = task >> 6;
        const int j = j0 + row;
        const bool valid = j < n;
        const int e = valid ? exp_of_max(mcmax[j]) : 0;
        double x[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int k = kb + kg * 8 + q;
          x[q] = (valid && k < n) ? M[(size_t)k * n + j] : 0.0;
        }
        store_digits(x, e, b_dst, B_SLICE_BYTES, core_off(row, kg));
      }
      tc::fence_proxy_async();
      __syncthreads();
      const int ci = s % OZ_SUBS;
      if (threadIdx.x == 0) {
        tc::fence_after_sync();
        issue_levels(tmem, tc::smem_u32(a_dst), tc::smem_u32(b_dst), ci == 0);
        tc::mma_commit(&mbar[buf]);
      }
      pend[buf] = 1;
      if (ci == OZ_SUBS - 1 || s == nsub - 1) {
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
          atomicExch(status, -2);
        }
        __syncthreads();
        if (abort_sh) break;
        tc::fence_after_sync();
        fold_levels(lane_base, H, Lo);
        tc::fence_before_sync();
        __syncthreads();
      }
    }
    if (abort_sh) break;
    // write the tile: consecutive lanes -> consecutive rows of one column (coalesced)
    const int r = r0 + 32 * (warp & 3) + lane;
    if (r < rows) {
      const int er = exp_of_max(rmax[r]);
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int j = j0 + 32 * (warp >> 2) + c;
        if (j < n) {
          Cout[r + (size_t)j * ldo] = fold_to_double(H[c], Lo[c], er + exp_of_max(mcmax[j]));
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

}  // namespace

// Overlap matrix on the tensor cores, queued without a host synchronisation.
// scond_bits (device, may be NULL) receives max|S-I| as ordered bits; a timed-out
// wait sets *status = -2.
int ovlap_tc(Ctx& c, const cx<double>* c0, int ldc, int nstate, double* S, unsigned long long* scond_bits,
             int* status) {
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
  // workspace: H, Lo (int64 n*n each), column maxima (n)
  const size_t bytes = 2 * nn * 8 + (size_t)n * 8;
  if (!ensure(c, c.sparts, bytes)) return 6;
  unsigned long long* Hacc = static_cast<unsigned long long*>(c.sparts.p);
  unsigned long long* Lacc = Hacc + nn;
  unsigned long long* cmax = Lacc + nn;
  GBCP_CUDA_TRY(c, cudaMemsetAsync(Hacc, 0, bytes, c.stream));
  {
    ProfScope ps_(c, "k_col_max");
    const int ks = std::max(1, std::min(64, (K + 4095) / 4096));
    const int kper = (K + ks - 1) / ks;
    k_col_max<<<dim3(n, ks), 256, 0, c.stream>>>(Ar, lda, K, n, kper, cmax);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    allow_smem(k_ozaki_syrk, OZ_SMEM);
    ProfScope ps_(c, "k_ozaki_syrk");
    k_ozaki_syrk<<<dim3(ntiles, nsplit), OZ_THREADS, OZ_SMEM, c.stream>>>(Ar, lda, K, n, cmax, njb, subs_per, Hacc,
                                                                          Lacc, status);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_ozaki_syrk_finalize");
    const int fb = std::max(1, std::min(1024, (int)((nn + 255) / 256)));
    k_ozaki_syrk_finalize<<<fb, 256, 0, c.stream>>>(reinterpret_cast<const long long*>(Hacc),
                                                    reinterpret_cast<const long long*>(Lacc), cmax, n, Ar, lda, c.geq0,
                                                    S, scond_bits);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

// Cout (rows x n, ldo) = A (rows x n, lda) * M (n x n row-major) on the tensor
// cores, queued without a host synchronisation; skipped when *status != 0 on
// entry, *status = -2 on a timed-out wait.
int rmul_tc(Ctx& c, const double* A, int lda, int rows, int n, const double* M, int upper, double* Cout, int ldo,
            int* status) {
  const size_t bytes = ((size_t)rows + n) * 8;
  if (!ensure(c, c.nl_a, bytes)) return 6;
  unsigned long long* rmax = static_cast<unsigned long long*>(c.nl_a.p);
  unsigned long long* mcmax = rmax + rows;
  {
    ProfScope ps_(c, "k_row_max");
    k_row_max<<<(rows + 255) / 256, 256, 0, c.stream>>>(A, lda, rows, n, rmax);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_mat_col_max");
    k_mat_col_max<<<(n + 255) / 256, 256, 0, c.stream>>>(M, n, mcmax);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    allow_smem(k_ozaki_rmul, OZ_SMEM);
    const int ntiles = ((rows + OZ_M - 1) / OZ_M) * ((n + OZ_N - 1) / OZ_N);
    const int grid = std::max(1, std::min(ntiles, 148));
    ProfScope ps_(c, "k_ozaki_rmul");
    k_ozaki_rmul<<<grid, OZ_THREADS, OZ_SMEM, c.stream>>>(A, lda, rows, n, M, upper, rmax, mcmax, Cout, ldo, status);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

}  // namespace gbcp
