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
// Products.  For a 128 x 32 output tile the CTA runs, per K-chunk of 128, the
// 36 digit-pair products with s + t = d <= 7 ("level" d), accumulating all pairs
// of a level in one FP32 TMEM accumulator (8 levels x 32 columns = one
// accumulator set; two sets fill the 512 TMEM columns).  A level sum is an
// integer below 8 * 128 * 127^2 < 2^24, so FP32 holds it exactly.  After each
// chunk the accumulators are read back and folded into two int64 registers per
// output (H = levels 0-3, Lo = levels 4-7, 7 bits apart); int64 keeps the sum
// over every chunk exact and only the final conversion is rounded:
// sum_k x_ik y_kj = 2^(E_i+E_j) (H 2^-35 + Lo 2^-63).  Levels above 7 are
// dropped (< 2^-49 of 2^(E_i+E_j) per product term).
//
// Data flow.  The digits are produced ONCE per operand by integer-only slicing
// kernels into eight bf16 digit planes in HBM (row-major, K contiguous, planes
// stacked along rows), and the GEMM kernel streams them with TMA (64-byte
// swizzle, K = 32 per sub-chunk, two shared-memory stages).  The CTA is split by
// role: one thread issues the TMA loads, one thread the 16 MMAs per sub-chunk,
// and sixteen warps fold a finished accumulator set into int64 and write the
// outputs while the MMAs of the next chunk fill the other set, so that the
// integer fold and the FP64 rounding run beside the tensor core instead of
// between its chunks.  Every mbarrier wait is bounded; on expiry the kernel sets
// the ortho status word to -2 (reported as GBCP_ERR_TIMEOUT), waits for its own
// loads and MMAs, frees its TMEM and returns.
#include <algorithm>
#include <cmath>
#include <cstring>

#include <cuda.h>

#include "ctx.h"
#include "fold_round.h"
#include "tc_common.cuh"
#include "tc_gemm.h"

namespace gbcp {

namespace {

constexpr int OZ_M = 128;      // output rows per tile
constexpr int OZ_N = 32;       // output columns per tile
constexpr int OZ_NB = OZ_M / OZ_N;  // column tiles per row-tile width (upper block triangle)
constexpr int OZ_KS = 32;      // K per sub-chunk (two MMAs of K = 16)
constexpr int OZ_SUBS = 4;     // sub-chunks per exact accumulation chunk (K = 128)
constexpr int OZ_SL = 8;       // digit slices
constexpr int OZ_LEV = 8;      // levels kept (s + t <= 7)
constexpr int OZ_CONS = 16;    // fold / epilogue warps (four per TMEM lane quadrant)
constexpr int OZ_CW = OZ_N / (OZ_CONS / 4);  // output columns per fold warp
constexpr int OZ_TMA_WARP = OZ_CONS, OZ_MMA_WARP = OZ_CONS + 1;
constexpr int OZ_THREADS = 32 * (OZ_CONS + 2);
constexpr int OZ_TBUF = OZ_LEV * OZ_N;  // TMEM columns of one accumulator set (two sets: 512)
constexpr int A_SLICE_BYTES = OZ_M * OZ_KS * 2;  // 8 KB
constexpr int B_SLICE_BYTES = OZ_N * OZ_KS * 2;  // 2 KB
constexpr int A_BUF_BYTES = OZ_SL * A_SLICE_BYTES;
constexpr int B_BUF_BYTES = OZ_SL * B_SLICE_BYTES;
constexpr int STAGE_BYTES = A_BUF_BYTES + B_BUF_BYTES;       // 80 KB
constexpr int OZ_SMEM = 2 * STAGE_BYTES + 1024;              // two stages, + alignment slack
static_assert(2 * OZ_TBUF == 512, "two accumulator sets fill the TMEM columns");
static_assert(OZ_N * OZ_LEV <= 256 && OZ_SL == OZ_LEV, "one MMA covers the levels s..7 of A plane s");
static_assert(OZ_CW % 8 == 0, "fold warps read TMEM 8 columns at a time");

// signed 7-bit digit -> bf16 bits (exact: |d| <= 127)
__device__ __forceinline__ uint32_t digit_bf16(int d) { return __float_as_uint((float)d) >> 16; }

// exponent E with |x| < 2^E from the bit pattern of max |x| (fold_round.h)
__device__ __forceinline__ int exp_of_max(unsigned long long bits) { return fold::exp_of_max(bits); }
// a column maximum that is NaN or infinite: its column held a non-finite value, and every
// overlap entry of that column is reported as NaN (the digit split of it is meaningless)
__device__ __forceinline__ bool max_nonfinite(unsigned long long bits) { return ((bits >> 52) & 0x7FF) == 0x7FF; }

// Fixed-point magnitude trunc(|x| 2^(56-E)) (< 2^56) and the sign (fold_round.h)
__device__ __forceinline__ unsigned long long fixed56(double x, int E, bool& neg) { return fold::fixed56(x, E, neg); }

// Digits of 8 consecutive K elements of one operand row -> 8 planes, 16 bytes each.
__device__ __forceinline__ void digits8(const double (&x)[8], int E, uint4 (&out)[OZ_SL]) {
  uint32_t w[OZ_SL][4];
#pragma unroll
  for (int q2 = 0; q2 < 4; ++q2) {
    bool n0, n1;
    const unsigned long long f0 = fixed56(x[2 * q2], E, n0), f1 = fixed56(x[2 * q2 + 1], E, n1);
#pragma unroll
    for (int s = 0; s < OZ_SL; ++s) {
      w[s][q2] = digit_bf16(fold::digit(f0, n0, s)) | (digit_bf16(fold::digit(f1, n1, s)) << 16);
    }
  }
#pragma unroll
  for (int s = 0; s < OZ_SL; ++s) out[s] = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// Issue the MMAs of one sub-chunk (all 36 digit pairs, 2 K-steps) into the 8
// level accumulators at tmem (level d at column OZ_N d); `first` restarts them
// (chunk start).  The B planes t = 0..7 of a stage lie back to back, each a
// K-major 64-byte-swizzle tile of OZ_N rows, so planes t = 0..7-s read as one
// B operand of OZ_N (8 - s) rows; with D at level s, its column block t lands in
// level s + t.  One MMA per A plane and K-step (8 x 2 instead of 36 x 2) reads
// each A plane from shared memory once per K-step, not once per pair.
__device__ __forceinline__ void issue_levels(uint32_t tmem, uint32_t a_base, uint32_t b_base, bool first) {
  const uint64_t a0 = tc::sdesc_kmajor_sw64(a_base), b0 = tc::sdesc_kmajor_sw64(b_base);
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
    for (int s = 0; s < OZ_SL; ++s) {
      const uint64_t ad = a0 + (uint64_t)((s * A_SLICE_BYTES + kk * 32) >> 4);
      const uint64_t bd = b0 + (uint64_t)((kk * 32) >> 4);
      tc::mma_f16(tmem + (uint32_t)(OZ_N * s), ad, bd, tc::idesc_bf16_f32(OZ_M, OZ_N * (OZ_LEV - s)),
                  (first && kk == 0 && s == 0) ? 0u : 1u);
    }
  }
}

// Fold one chunk's 8 level accumulators (this thread's TMEM lane, OZ_CW columns at
// taddr) into H (levels 0-3) and Lo (levels 4-7).  Levels are read in pairs and
// combined in 32-bit first: v_2k 2^7 + v_2k+1 stays below 2^31 because a level-d
// sum is bounded by 128 (d + 1) 127^2 (level 7: 16 516 096; pair 6-7:
// 1 866 318 848).  Once the last pair is in registers the warp releases the
// accumulator set (`tempty`), so the MMAs of a later chunk may overwrite it while
// the integer work finishes.
__device__ __forceinline__ void fold_chunk(uint32_t taddr, long long (&H)[OZ_CW], long long (&Lo)[OZ_CW],
                                           uint64_t* tempty, int lane) {
  uint32_t ra[OZ_CW], rb[OZ_CW];
  int pr[OZ_CW];
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    tc::tmem_ld8(taddr + (uint32_t)(OZ_N * (2 * g)), ra);
    tc::tmem_ld8(taddr + (uint32_t)(OZ_N * (2 * g + 1)), rb);
    tc::tmem_ld_wait();
    if (g == 3) {
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tempty);
    }
    if ((g & 1) == 0) {
#pragma unroll
      for (int c = 0; c < OZ_CW; ++c)
        pr[c] = __float2int_rn(__uint_as_float(ra[c])) * 128 + __float2int_rn(__uint_as_float(rb[c]));
    } else {
#pragma unroll
      for (int c = 0; c < OZ_CW; ++c) {
        const int lo = __float2int_rn(__uint_as_float(ra[c])) * 128 + __float2int_rn(__uint_as_float(rb[c]));
        const long long v = (long long)pr[c] * 16384 + (long long)lo;
        if (g == 1) H[c] += v;
        else Lo[c] += v;
      }
    }
  }
}

// Conversions of the int64 level sums: fold_round.h (the S finalizers round
// exactly; the C M epilogue uses the 62-bit window, whose dropped part, below
// 2^-54 of the scale 2^(E_i+E_j) for one chunk, lies under the truncation of the
// split itself: levels s + t > 7, 2^-49 of the scale per product term).
__device__ __forceinline__ double fold_to_double(long long H, long long Lo, int ee) {
  return fold::to_double_exact(H, Lo, ee);
}
__device__ __forceinline__ double fold_to_double_fast(long long H, long long Lo, int ee, int s) {
  return fold::to_double_window(H, Lo, ee, s);
}

// ---------------------------------------------------------------- exponent pre-passes
// column maxima |a_kj| over k (state columns of the real view): bits into cmax[j].
// Eight independent loads per thread and pass keep enough reads in flight for
// the HBM bandwidth (one dependent load per pass left the kernel latency-bound).
__global__ void k_col_max(const double* __restrict__ Ar, int lda, int K, int n, int kper,
                          unsigned long long* __restrict__ cmax) {
  pdl_entry();
  const int j = blockIdx.x;
  const int k0 = blockIdx.y * kper, k1 = min(K, k0 + kper);
  const unsigned long long* a = reinterpret_cast<const unsigned long long*>(Ar) + (size_t)j * lda;
  unsigned long long mx = 0;
  for (int kb = k0 + threadIdx.x; kb < k1; kb += 8 * blockDim.x) {
    unsigned long long b[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = kb + u * blockDim.x;
      b[u] = k < k1 ? (__ldg(a + k) & ~(1ull << 63)) : 0ull;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) mx = b[u] > mx ? b[u] : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_down_sync(0xffffffffu, mx, o);
    mx = v > mx ? v : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(cmax + j, mx);
}

// column maxima of a small row-major n x n matrix M over its rows, columns j0 ..:
// block = 32 columns x 8 row groups, reduced in shared memory
__global__ void __launch_bounds__(256) k_mat_col_max(const double* __restrict__ M, int n,
                                                     unsigned long long* __restrict__ cmax, int j0) {
  pdl_entry();
  __shared__ unsigned long long red[8][33];
  const int j = j0 + blockIdx.x * 32 + threadIdx.x, g = threadIdx.y;
  unsigned long long mx = 0;
  if (j < n) {
    for (int k = g; k < n; k += 8) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(__ldg(M + (size_t)k * n + j)) & ~(1ull << 63);
      mx = b > mx ? b : mx;
    }
  }
  red[g][threadIdx.x] = mx;
  __syncthreads();
  if (g == 0 && j < n) {
#pragma unroll
    for (int q = 1; q < 8; ++q) mx = red[q][threadIdx.x] > mx ? red[q][threadIdx.x] : mx;
    cmax[j] = mx;
  }
}

// ---------------------------------------------------------------- digit planes
// S operand: plane s, row j (state), columns k < K of the real view; exponent per state.
// k0: first row of the slab (a multiple of 8); rows k0 .. k0+K-1 of Ar go to plane columns k0 ..
__global__ void k_oz_slice_cols(const double* __restrict__ Ar, int lda, int K, int n,
                                const unsigned long long* __restrict__ emax, size_t ks, uint4* __restrict__ out,
                                int k0) {
  pdl_entry();
  const int j = blockIdx.y;
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) * 8;
  if (k >= K) return;
  const int e = exp_of_max(emax[j]);
  const double* a = Ar + (size_t)j * lda + k0 + k;
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = (k + q < K) ? a[q] : 0.0;
  uint4 d[OZ_SL];
  digits8(x, e, d);
  const size_t plane = (size_t)n * ks / 8, off = ((size_t)j * ks + k0 + k) / 8;
#pragma unroll
  for (int s = 0; s < OZ_SL; ++s) out[s * plane + off] = d[s];
}

// row maxima of the real view over the n states: bits into rmax[r]
__global__ void k_row_max(const double* __restrict__ Ar, int lda, int rows, int n,
                          unsigned long long* __restrict__ rmax) {
  pdl_entry();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  unsigned long long mx = 0;
  for (int k = 0; k < n; ++k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(Ar[r + (size_t)k * lda]) & ~(1ull << 63);
    mx = b > mx ? b : mx;
  }
  rmax[r] = mx;
}

// C M operand A: plane s, row r (real-view row of C), columns k < n (states); exponent per
// row.  Thread = (row, 16 states): consecutive threads read consecutive rows (coalesced)
// and each plane store is one full 32-byte sector.
__global__ void k_oz_slice_rows(const double* __restrict__ Ar, int lda, int rows, int n,
                                const unsigned long long* __restrict__ emax, size_t ks, uint4* __restrict__ out) {
  pdl_entry();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y * 16;
  if (r >= rows) return;
  const int e = exp_of_max(emax[r]);
  double x0[8], x1[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    x0[q] = (k + q < n) ? Ar[r + (size_t)(k + q) * lda] : 0.0;
    x1[q] = (k + 8 + q < n) ? Ar[r + (size_t)(k + 8 + q) * lda] : 0.0;
  }
  uint4 d0[OZ_SL], d1[OZ_SL];
  digits8(x0, e, d0);
  digits8(x1, e, d1);
  const size_t plane = (size_t)rows * ks / 8, off = ((size_t)r * ks + k) / 8;
#pragma unroll
  for (int s = 0; s < OZ_SL; ++s) {
    out[s * plane + off] = d0[s];
    if (k + 8 < n) out[s * plane + off + 1] = d1[s];
  }
}

// The same slicing with the row exponents found in the same pass (n <= 256): block
// (32 rows, ceil(n/16) column groups), thread (row, 16 states); the row maximum is
// reduced over the column groups in shared memory and also stored to rmax.
// rows r0 .. r1-1 (r1 <= rows; rows sets the plane stride)
__global__ void __launch_bounds__(512) k_oz_slice_rows_max(const double* __restrict__ Ar, int lda, int rows, int n,
                                                           unsigned long long* __restrict__ rmax, size_t ks,
                                                           uint4* __restrict__ out, int r0, int r1) {
  pdl_entry();
  __shared__ unsigned long long red[16][33];
  const int r = r0 + blockIdx.x * 32 + threadIdx.x, k = threadIdx.y * 16;
  double x0[8], x1[8];
  unsigned long long mx = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    x0[q] = (r < r1 && k + q < n) ? Ar[r + (size_t)(k + q) * lda] : 0.0;
    x1[q] = (r < r1 && k + 8 + q < n) ? Ar[r + (size_t)(k + 8 + q) * lda] : 0.0;
    const unsigned long long b0 = (unsigned long long)__double_as_longlong(x0[q]) & ~(1ull << 63);
    const unsigned long long b1 = (unsigned long long)__double_as_longlong(x1[q]) & ~(1ull << 63);
    mx = b0 > mx ? b0 : mx;
    mx = b1 > mx ? b1 : mx;
  }
  red[threadIdx.y][threadIdx.x] = mx;
  __syncthreads();
  if (threadIdx.y == 0) {
    for (int j = 1; j < (int)blockDim.y; ++j) {
      const unsigned long long o = red[j][threadIdx.x];
      mx = o > mx ? o : mx;
    }
    red[0][threadIdx.x] = mx;
    if (r < r1) rmax[r] = mx;
  }
  __syncthreads();
  if (r >= r1) return;
  const int e = exp_of_max(red[0][threadIdx.x]);
  uint4 d0[OZ_SL], d1[OZ_SL];
  digits8(x0, e, d0);
  digits8(x1, e, d1);
  const size_t plane = (size_t)rows * ks / 8, off = ((size_t)r * ks + k) / 8;
#pragma unroll
  for (int s = 0; s < OZ_SL; ++s) {
    out[s * plane + off] = d0[s];
    if (k + 8 < n) out[s * plane + off + 1] = d1[s];
  }
}

// C M operand B: plane s, row j (column of M), columns k < n: M[k][j]; exponent per column of M.
__global__ void k_oz_slice_mat(const double* __restrict__ M, int n, const unsigned long long* __restrict__ emax,
                               size_t ks, uint4* __restrict__ out, int j0, int j1) {
  pdl_entry();
  const int j = j0 + blockIdx.x * blockDim.x + threadIdx.x;  // columns j0 .. j1 - 1
  const int k = blockIdx.y * 8;
  if (j >= j1) return;
  const int e = exp_of_max(emax[j]);
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = (k + q < n) ? M[(size_t)(k + q) * n + j] : 0.0;
  uint4 d[OZ_SL];
  digits8(x, e, d);
  const size_t plane = (size_t)n * ks / 8, off = ((size_t)j * ks + k) / 8;
#pragma unroll
  for (int s = 0; s < OZ_SL; ++s) out[s * plane + off] = d[s];
}

// ---------------------------------------------------------------- the split GEMM
struct OzParams {
  int M, N;           // rows per digit plane of A and of B
  int K;              // contraction length
  int mode;           // 0: S, tiles of the upper block triangle x K splits; 1: C M, persistent over tiles
  int full;           // mode 0: every tile of the nib x njb grid (two different operands)
  int njb;            // mode 0: column tiles
  int subs_per;       // mode 0: sub-chunks per K split (a multiple of OZ_SUBS)
  int upper;          // mode 1: M upper triangular (column tile j needs k < j0 + OZ_N)
  const unsigned long long* eA;  // mode 1: exponent bits per row of A
  const unsigned long long* eB;  // mode 1: exponent bits per column
  unsigned long long* Hacc;      // mode 0: int64 accumulators (n x n)
  unsigned long long* Lacc;
  double* Cout;                  // mode 1
  int ldo;
  int zero_row1;                 // mode 1: write 0 to row 1 (Im c(G=0) of the real view)
  int accumulate;                // mode 1: Cout += A M instead of Cout = A M
  int sub_base;                  // mode 0: K offset of this launch, in sub-chunks
  int rt0, nrt;                  // mode 1: row tiles rt0 .. rt0+nrt-1 (nrt = 0: every row tile)
  int ct0, nct;                  // mode 1: column tiles ct0 .. ct0+nct-1 (nct = 0: every column tile)
  int* status;
  // test of the timeout path: stall != 0 makes the TMA thread issue no loads, so the
  // MMA thread's first wait on a stage (no copy in flight towards it) runs out after
  // wait_limit cycles (0 = the default limit of about a second)
  int stall;
  long long wait_limit;
};

struct OzUnit {
  int m0, n0, sub0, nsub;
  bool valid;
};

__device__ __forceinline__ OzUnit oz_unit(const OzParams& p, int u) {
  OzUnit w{0, 0, 0, 0, false};
  const int total_subs = (p.K + OZ_KS - 1) / OZ_KS;
  if (p.mode == 0) {
    if (u != (int)blockIdx.x) return w;  // one unit per CTA
    if (p.full) {
      w.m0 = (blockIdx.x / p.njb) * OZ_M;
      w.n0 = (blockIdx.x % p.njb) * OZ_N;
    } else {
      int t = blockIdx.x, ib = 0;
      while (ib < 4096 && t >= max(0, p.njb - OZ_NB * ib)) {
        t -= max(0, p.njb - OZ_NB * ib);
        ++ib;
      }
      if (ib >= 4096) return w;
      w.m0 = ib * OZ_M;
      w.n0 = (OZ_NB * ib + t) * OZ_N;
    }
    w.sub0 = blockIdx.y * p.subs_per;
    w.nsub = min(total_subs, w.sub0 + p.subs_per) - w.sub0;
    w.valid = w.nsub > 0;
    return w;
  }
  const int nrt = p.nrt > 0 ? p.nrt : (p.M + OZ_M - 1) / OZ_M, nct = p.nct > 0 ? p.nct : (p.N + OZ_N - 1) / OZ_N;
  // Round k of the persistent loop covers units [k G, k G + G) (G = grid size);
  // odd rounds run the CTAs in reverse order, so that with an upper triangular M
  // (column tile ct costs ct + 1 sub-chunks) each CTA alternates cheap and
  // dear column tiles instead of keeping one for every round.
  const int G = (int)gridDim.x, k = u / G, v = (k & 1) ? k * G + (G - 1 - u % G) : u;
  if (v >= nrt * nct) return w;
  const int rt = p.rt0 + v / nct, ct = p.ct0 + v % nct;  // row tile outer: the CTAs of one row tile share its planes in L2
  w.m0 = rt * OZ_M;
  w.n0 = ct * OZ_N;
  const int kmax = p.upper ? min(p.K, w.n0 + OZ_N) : p.K;
  w.sub0 = 0;
  w.nsub = (kmax + OZ_KS - 1) / OZ_KS;
  w.valid = true;
  return w;
}

__device__ __forceinline__ int oz_next_unit(const OzParams& p, int u) { return p.mode == 0 ? -1 : u + (int)gridDim.x; }

// the TMA thread: the 16 loads (8 A planes, 8 B planes) of one sub-chunk into stage buf
__device__ __forceinline__ void oz_load(const CUtensorMap* tmA, const CUtensorMap* tmB, const OzParams& p,
                                        const OzUnit& w, int s, uint8_t* buf, uint64_t* bar) {
  const int k = (p.sub_base + w.sub0 + s) * OZ_KS;
  tc::mbar_expect_tx(bar, STAGE_BYTES);
#pragma unroll 1
  for (int pl = 0; pl < OZ_SL; ++pl) {
    tc::tma_load_2d(buf + pl * A_SLICE_BYTES, tmA, bar, k, pl * p.M + w.m0);
    tc::tma_load_2d(buf + A_BUF_BYTES + pl * B_SLICE_BYTES, tmB, bar, k, pl * p.N + w.n0);
  }
}

// Warp roles: warp OZ_TMA_WARP (one thread) streams the digit planes into two
// shared-memory stages; warp OZ_MMA_WARP (one thread) issues each chunk's MMAs
// into one of two TMEM accumulator sets; the OZ_CONS fold warps read a finished
// set, fold it into int64 and, at the end of a unit, write the unit's outputs,
// while the MMAs of the next chunk run in the other set.
//   full[s]  : stage s loaded (TMA transaction bytes)     empty[s]  : stage s read by its MMAs (commit)
//   tfull[b] : accumulator set b complete (commit)        tempty[b] : set b read by every fold warp
// Every barrier completes once per use; use j of a two-slot resource is slot
// j & 1, phase j >> 1, so a consumer waits for parity (j >> 1) & 1 and the
// producer of use j waits for the release of use j - 2, parity ((j >> 1) & 1) ^ 1
// (a fresh barrier reports that parity as complete).
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_oz_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const OzParams p) {
  pdl_entry();
  extern __shared__ uint8_t oz_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(oz_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full[2], empty[2], tfull[2], tempty[2], drain;
  __shared__ uint32_t tmem_sh;
  __shared__ volatile int abort_sh;
  __shared__ int skip_sh, issued_sh, consumed_sh;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    // an earlier step of this ortho failed: every thread leaves before any setup
    skip_sh = (p.mode == 1 && *(volatile const int*)p.status != 0) ? 1 : 0;
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], OZ_CONS);
    }
    tc::mbar_init(&drain, 1);
    tc::fence_mbar_init();
    abort_sh = 0;
    issued_sh = 0;
    consumed_sh = 0;
  }
  __syncthreads();
  if (skip_sh) return;
  if (warp == 0) {
    tc::tmem_alloc(&tmem_sh, 512);
    tc::tmem_relinquish();
  }
  if (warp == OZ_TMA_WARP && lane == 0) {
    tc::tma_prefetch_desc(&tmA);
    tc::tma_prefetch_desc(&tmB);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_sh;
  const long long lim = p.wait_limit > 0 ? p.wait_limit : 2000000000LL;

  if (warp == OZ_TMA_WARP) {
    if (lane == 0) {
      int it = 0;  // sub-chunks loaded by this CTA
      for (int u = blockIdx.x; u >= 0 && !abort_sh && !p.stall; u = oz_next_unit(p, u)) {
        const OzUnit w = oz_unit(p, u);
        if (!w.valid) break;
        for (int s = 0; s < w.nsub && !abort_sh; ++s, ++it) {
          const int slot = it & 1;
          if (!tc::mbar_wait(&empty[slot], (uint32_t)(((it >> 1) & 1) ^ 1), lim)) {
            abort_sh = 1;
            atomicExch(p.status, -2);
            break;
          }
          oz_load(&tmA, &tmB, p, w, s, sm + slot * STAGE_BYTES, &full[slot]);
        }
      }
      issued_sh = it;
    }
  } else if (warp == OZ_MMA_WARP) {
    if (lane == 0) {
      int it = 0, ch = 0;  // sub-chunks consumed, chunks issued
      bool stop = false;
      for (int u = blockIdx.x; u >= 0 && !stop; u = oz_next_unit(p, u)) {
        const OzUnit w = oz_unit(p, u);
        if (!w.valid) break;
        for (int c0 = 0; c0 < w.nsub && !stop; c0 += OZ_SUBS, ++ch) {
          const int b = ch & 1;
          if (abort_sh || !tc::mbar_wait(&tempty[b], (uint32_t)(((ch >> 1) & 1) ^ 1), lim)) {
            stop = true;
            break;
          }
          tc::fence_after_sync();
          const int c1 = min(w.nsub, c0 + OZ_SUBS);
          for (int s = c0; s < c1; ++s, ++it) {
            const int slot = it & 1;
            if (abort_sh || !tc::mbar_wait(&full[slot], (uint32_t)((it >> 1) & 1), lim)) {
              stop = true;
              break;
            }
            tc::fence_after_sync();
            uint8_t* cur = sm + slot * STAGE_BYTES;
            issue_levels(tmem + (uint32_t)(b * OZ_TBUF), tc::smem_u32(cur), tc::smem_u32(cur + A_BUF_BYTES), s == c0);
            tc::mma_commit(&empty[slot]);
          }
          if (stop) break;
          tc::mma_commit(&tfull[b]);
        }
      }
      if (stop && !abort_sh) {
        abort_sh = 1;
        atomicExch(p.status, -2);
      }
      consumed_sh = it;
      // every MMA this thread issued has finished once this commit arrives
      tc::mma_commit(&drain);
      if (!tc::mbar_wait(&drain, 0, lim)) atomicExch(p.status, -2);
    }
  } else {
    const int q = warp & 3, h = warp >> 2;  // TMEM lane quadrant, column group
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(OZ_CW * h);
    int ch = 0;
    bool stop = false;
    for (int u = blockIdx.x; u >= 0 && !stop; u = oz_next_unit(p, u)) {
      const OzUnit w = oz_unit(p, u);
      if (!w.valid) break;
      const int row = w.m0 + 32 * q + lane;
      // mode 1: the scale exponents of this thread's outputs, read before the
      // fold so that their latency hides behind it (loaded between the output
      // stores they would be serialised with them: the compiler cannot tell
      // that the exponent arrays and the output do not overlap)
      int eo[OZ_CW];
#pragma unroll
      for (int c = 0; c < OZ_CW; ++c) {
        const int j = w.n0 + OZ_CW * h + c;
        eo[c] = (p.mode == 1 && j < p.N) ? exp_of_max(__ldg(p.eB + j)) : 0;
      }
      const int er = (p.mode == 1 && row < p.M) ? exp_of_max(__ldg(p.eA + row)) : 0;
      long long H[OZ_CW], Lo[OZ_CW];
#pragma unroll
      for (int c = 0; c < OZ_CW; ++c) {
        H[c] = 0;
        Lo[c] = 0;
      }
      for (int c0 = 0; c0 < w.nsub; c0 += OZ_SUBS, ++ch) {
        const int b = ch & 1;
        const bool ok = !abort_sh && tc::mbar_wait(&tfull[b], (uint32_t)((ch >> 1) & 1), lim);
        if (!__all_sync(0xffffffffu, ok ? 1 : 0)) {
          stop = true;
          break;
        }
        tc::fence_after_sync();
        fold_chunk(tl + (uint32_t)(b * OZ_TBUF), H, Lo, &tempty[b], lane);
      }
      if (stop) break;
      if (p.mode == 0) {
        if (row < p.M) {
#pragma unroll
          for (int c = 0; c < OZ_CW; ++c) {
            const int col = w.n0 + OZ_CW * h + c;
            if (col < p.N) {
              atomicAdd(p.Hacc + (size_t)row * p.N + col, (unsigned long long)H[c]);
              atomicAdd(p.Lacc + (size_t)row * p.N + col, (unsigned long long)Lo[c]);
            }
          }
        }
      } else if (row < p.M) {
        double* o = p.Cout + row + (size_t)(w.n0 + OZ_CW * h) * p.ldo;
        const int ncol = min(OZ_CW, p.N - (w.n0 + OZ_CW * h));
        const int sdrop = fold::window_drop_bits((w.nsub + OZ_SUBS - 1) / OZ_SUBS);
#pragma unroll
        for (int g = 0; g < OZ_CW; g += 8) {
          double prev[8];
          if (p.accumulate) {  // the group's reads before its stores
#pragma unroll
            for (int c = 0; c < 8; ++c) prev[c] = g + c < ncol ? o[(size_t)(g + c) * p.ldo] : 0.0;
          }
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            if (g + c < ncol) {
              double v = (p.zero_row1 && row == 1) ? 0.0 : fold_to_double_fast(H[g + c], Lo[g + c], er + eo[g + c], sdrop);
              if (p.accumulate) v += prev[c];
              o[(size_t)(g + c) * p.ldo] = v;
            }
          }
        }
      }
    }
    if (stop && lane == 0 && !abort_sh) {
      abort_sh = 1;
      atomicExch(p.status, -2);
    }
  }
  __syncthreads();
  if (warp == OZ_TMA_WARP && lane == 0) {
    // loads issued but never consumed (after an abort) still land in shared
    // memory: wait for them before the CTA exits (at most one per stage)
    for (int j = consumed_sh; j < issued_sh; ++j) tc::mbar_wait(&full[j & 1], (uint32_t)((j >> 1) & 1), lim);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

// S[i][j] (i <= j, mirrored) = 2 * 2^(E_i+E_j) (H 2^-35 + Lo 2^-63) - Re c0_i Re c0_j
__global__ void k_ozaki_syrk_finalize(const long long* __restrict__ H, const long long* __restrict__ Lo,
                                      const unsigned long long* __restrict__ cmax, int n,
                                      const double* __restrict__ Ar, int lda, int geq0, double* __restrict__ S,
                                      unsigned long long* __restrict__ scond_bits) {
  pdl_entry();
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (i > j) continue;
    double v = 2.0 * fold_to_double(H[e], Lo[e], exp_of_max(cmax[i]) + exp_of_max(cmax[j]));
    if (geq0) v -= Ar[(size_t)i * lda] * Ar[(size_t)j * lda];
    if (max_nonfinite(cmax[i]) || max_nonfinite(cmax[j])) v = __longlong_as_double(0x7FF8000000000000LL);
    S[(size_t)i * n + j] = v;
    S[(size_t)j * n + i] = v;
    mx = fmax(mx, fabs(i == j ? v - 1.0 : v));
  }
  if (scond_bits) {
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(scond_bits, (unsigned long long)__double_as_longlong(mx));
  }
}

// A[i][j] = 2 <x_i|y_j> - Re x_i(0) Re y_j(0) from the int64 level sums of the full grid
__global__ void k_ozaki_xov_finalize(const long long* __restrict__ H, const long long* __restrict__ Lo,
                                     const unsigned long long* __restrict__ xmax,
                                     const unsigned long long* __restrict__ ymax, int n, const double* __restrict__ X,
                                     int ldx, const double* __restrict__ Y, int ldy, int geq0, double* __restrict__ A) {
  pdl_entry();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    double v = 2.0 * fold_to_double(H[e], Lo[e], exp_of_max(xmax[i]) + exp_of_max(ymax[j]));
    if (geq0) v -= X[(size_t)i * ldx] * Y[(size_t)j * ldy];
    if (max_nonfinite(xmax[i]) || max_nonfinite(ymax[j])) v = __longlong_as_double(0x7FF8000000000000LL);
    A[e] = v;
  }
}

// S[i][j] (i <= j, mirrored) = the sum over R K ranges, in range order, of
// 2 * 2^(E_i^r + E_j^r) (H_r 2^-35 + Lo_r 2^-63), minus Re c0_i Re c0_j
__global__ void k_ozaki_syrk_finalize_ranges(const long long* __restrict__ H, const long long* __restrict__ Lo,
                                             const unsigned long long* __restrict__ cmax, int R, int n,
                                             const double* __restrict__ Ar, int lda, int geq0,
                                             double* __restrict__ S, unsigned long long* __restrict__ scond_bits) {
  pdl_entry();
  const size_t nn = (size_t)n * n;
  double mx = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (i > j) continue;
    double v = 0.0;
    for (int r = 0; r < R; ++r) {
      v += 2.0 * fold_to_double(H[r * nn + e], Lo[r * nn + e],
                                exp_of_max(cmax[(size_t)r * n + i]) + exp_of_max(cmax[(size_t)r * n + j]));
      if (max_nonfinite(cmax[(size_t)r * n + i]) || max_nonfinite(cmax[(size_t)r * n + j]))
        v = __longlong_as_double(0x7FF8000000000000LL);
    }
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
  for (int ib = 0; ib < nib; ++ib) ntiles += std::max(0, njb - OZ_NB * ib);
  const int total_subs = (K + OZ_KS - 1) / OZ_KS;
  // K splits per output tile: enough CTAs to fill the SMs, or the tuned count (c.oz_ksplit)
  const int want = c.oz_ksplit > 0 ? c.oz_ksplit : (c.nsm > 0 ? c.nsm : 148) / std::max(1, ntiles);
  int nsplit = std::max(1, std::min((total_subs + OZ_SUBS - 1) / OZ_SUBS, want));
  int subs_per = (total_subs + nsplit - 1) / nsplit;
  subs_per = ((subs_per + OZ_SUBS - 1) / OZ_SUBS) * OZ_SUBS;
  nsplit = (total_subs + subs_per - 1) / subs_per;
  const size_t nn = (size_t)n * n;
  const size_t ks = ((size_t)K + 7) & ~size_t(7);
  // workspace: H, Lo (int64 n*n each), column maxima (n); digit planes 8 x n x ks bf16
  const size_t bytes = 2 * nn * 8 + (size_t)n * 8;
  if (!ensure(c, c.sparts, bytes) || !ensure(c, c.oz_a, sizeof(uint16_t) * OZ_SL * (size_t)n * ks)) return 6;
  unsigned long long* Hacc = static_cast<unsigned long long*>(c.sparts.p);
  unsigned long long* Lacc = Hacc + nn;
  unsigned long long* cmax = Lacc + nn;
  GBCP_CUDA_TRY(c, cudaMemsetAsync(Hacc, 0, bytes, c.stream));
  {
    ProfScope ps_(c, "k_col_max");
    const int kspl = std::max(1, std::min(64, (K + 4095) / 4096));
    const int kper = (K + kspl - 1) / kspl;
    GBCP_LAUNCH_PDL(c, k_col_max, dim3(n, kspl), dim3(256), 0, Ar, lda, K, n, kper, cmax);
  }
  {
    ProfScope ps_(c, "k_oz_slice");
    GBCP_LAUNCH_PDL(c, k_oz_slice_cols, dim3((K / 8 + 255) / 256 + 1, n), dim3(256), 0, Ar, lda, K, n, cmax, ks,
        static_cast<uint4*>(c.oz_a.p), 0);
  }
  CUtensorMap ma, mb;
  if (!tmap_bf16_2d(&ma, c.oz_a.p, K, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_M, 64) ||
      !tmap_bf16_2d(&mb, c.oz_a.p, K, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_N, 64)) {
    c.err = "ovlap: tensor map encoding failed";
    return 5;
  }
  OzParams p{};
  p.M = n;
  p.N = n;
  p.K = K;
  p.mode = 0;
  p.njb = njb;
  p.subs_per = subs_per;
  p.Hacc = Hacc;
  p.Lacc = Lacc;
  p.status = status;
  if (c.test_stall) {  // one call only: the test of the timeout path
    p.stall = 1;
    p.wait_limit = 2000000;  // about a millisecond
    c.test_stall = 0;
  }
  {
    allow_smem(k_oz_tc, OZ_SMEM);
    ProfScope ps_(c, "k_ozaki_syrk");
    GBCP_LAUNCH_PDL(c, k_oz_tc, dim3(ntiles, nsplit), dim3(OZ_THREADS), OZ_SMEM, ma, mb, p);
  }
  {
    ProfScope ps_(c, "k_ozaki_syrk_finalize");
    const int fb = std::max(1, std::min(1024, (int)((nn + 255) / 256)));
    GBCP_LAUNCH_PDL(c, k_ozaki_syrk_finalize, dim3(fb), dim3(256), 0, reinterpret_cast<const long long*>(Hacc),
        reinterpret_cast<const long long*>(Lacc), cmax, n, Ar, lda, c.geq0, S, scond_bits);
  }
  return 0;
}

// Cross overlap <X_i|Y_j> of two different sets of n states on the tensor cores:
// both operands sliced into digit planes with their own column exponents, every
// tile of the n x n grid (mode 0, full), then the Γ-metric finalize.
int xovlap_tc(Ctx& c, const double* X, int ldx, const double* Y, int ldy, int n, double* A, int* status) {
  const int K = 2 * c.ngw;
  const int nib = (n + OZ_M - 1) / OZ_M, njb = (n + OZ_N - 1) / OZ_N;
  const int ntiles = nib * njb;
  const int total_subs = (K + OZ_KS - 1) / OZ_KS;
  int nsplit = std::max(1, std::min((total_subs + OZ_SUBS - 1) / OZ_SUBS, (c.nsm > 0 ? c.nsm : 148) / std::max(1, ntiles)));
  int subs_per = (total_subs + nsplit - 1) / nsplit;
  subs_per = ((subs_per + OZ_SUBS - 1) / OZ_SUBS) * OZ_SUBS;
  nsplit = (total_subs + subs_per - 1) / subs_per;
  const size_t nn = (size_t)n * n;
  const size_t ks = ((size_t)K + 7) & ~size_t(7);
  const size_t bytes = 2 * nn * 8 + 2 * (size_t)n * 8;
  if (!ensure(c, c.sparts, bytes) || !ensure(c, c.oz_a, sizeof(uint16_t) * OZ_SL * (size_t)n * ks) ||
      !ensure(c, c.oz_b, sizeof(uint16_t) * OZ_SL * (size_t)n * ks))
    return 6;
  unsigned long long* Hacc = static_cast<unsigned long long*>(c.sparts.p);
  unsigned long long* Lacc = Hacc + nn;
  unsigned long long* xmax = Lacc + nn;
  unsigned long long* ymax = xmax + n;
  GBCP_CUDA_TRY(c, cudaMemsetAsync(Hacc, 0, bytes, c.stream));
  {
    ProfScope ps_(c, "k_col_max");
    const int kspl = std::max(1, std::min(64, (K + 4095) / 4096));
    const int kper = (K + kspl - 1) / kspl;
    GBCP_LAUNCH_PDL(c, k_col_max, dim3(n, kspl), dim3(256), 0, X, ldx, K, n, kper, xmax);
    GBCP_LAUNCH_PDL(c, k_col_max, dim3(n, kspl), dim3(256), 0, Y, ldy, K, n, kper, ymax);
  }
  {
    ProfScope ps_(c, "k_oz_slice");
    GBCP_LAUNCH_PDL(c, k_oz_slice_cols, dim3((K / 8 + 255) / 256 + 1, n), dim3(256), 0, X, ldx, K, n, xmax, ks,
        static_cast<uint4*>(c.oz_a.p), 0);
    GBCP_LAUNCH_PDL(c, k_oz_slice_cols, dim3((K / 8 + 255) / 256 + 1, n), dim3(256), 0, Y, ldy, K, n, ymax, ks,
        static_cast<uint4*>(c.oz_b.p), 0);
  }
  CUtensorMap ma, mb;
  if (!tmap_bf16_2d(&ma, c.oz_a.p, K, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_M, 64) ||
      !tmap_bf16_2d(&mb, c.oz_b.p, K, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_N, 64)) {
    c.err = "cross overlap: tensor map encoding failed";
    return 5;
  }
  OzParams p{};
  p.M = n;
  p.N = n;
  p.K = K;
  p.mode = 0;
  p.full = 1;
  p.njb = njb;
  p.subs_per = subs_per;
  p.Hacc = Hacc;
  p.Lacc = Lacc;
  p.status = status;
  {
    allow_smem(k_oz_tc, OZ_SMEM);
    ProfScope ps_(c, "k_ozaki_xov");
    GBCP_LAUNCH_PDL(c, k_oz_tc, dim3(ntiles, nsplit), dim3(OZ_THREADS), OZ_SMEM, ma, mb, p);
  }
  {
    ProfScope ps_(c, "k_ozaki_syrk_finalize");
    const int fb = std::max(1, std::min(1024, (int)((nn + 255) / 256)));
    GBCP_LAUNCH_PDL(c, k_ozaki_xov_finalize, dim3(fb), dim3(256), 0, reinterpret_cast<const long long*>(Hacc),
        reinterpret_cast<const long long*>(Lacc), xmax, ymax, n, X, ldx, Y, ldy, c.geq0, A);
  }
  return 0;
}

// Cout (rows x n, ldo) = A (rows x n, lda) * M (n x n row-major) on the tensor
// cores, queued without a host synchronisation; skipped when *status != 0 on
// entry, *status = -2 on a timed-out wait.
int rmul_tc(Ctx& c, const double* A, int lda, int rows, int n, const double* M, int upper, double* Cout, int ldo,
            int zero_row1, int* status, int accumulate) {
  const size_t ks = ((size_t)n + 7) & ~size_t(7);
  const size_t bytes = ((size_t)rows + n) * 8;
  if (!ensure(c, c.nl_a, bytes) || !ensure(c, c.oz_a, sizeof(uint16_t) * OZ_SL * (size_t)rows * ks) ||
      !ensure(c, c.oz_b, sizeof(uint16_t) * OZ_SL * (size_t)n * ks))
    return 6;
  unsigned long long* rmax = static_cast<unsigned long long*>(c.nl_a.p);
  unsigned long long* mcmax = rmax + rows;
  {
    ProfScope ps_(c, "k_mat_col_max");
    GBCP_LAUNCH_PDL(c, k_mat_col_max, dim3((n + 31) / 32), dim3(32, 8), 0, M, n, mcmax, 0);
  }
  if (n <= 256) {
    ProfScope ps_(c, "k_oz_slice");
    GBCP_LAUNCH_PDL(c, k_oz_slice_rows_max, dim3((rows + 31) / 32), dim3(32, (n + 15) / 16), 0, A, lda, rows, n, rmax,
        ks, static_cast<uint4*>(c.oz_a.p), 0, rows);
  } else {
    {
      ProfScope ps_(c, "k_row_max");
      GBCP_LAUNCH_PDL(c, k_row_max, dim3((rows + 255) / 256), dim3(256), 0, A, lda, rows, n, rmax);
    }
    ProfScope ps_(c, "k_oz_slice");
    GBCP_LAUNCH_PDL(c, k_oz_slice_rows, dim3((rows + 127) / 128, (n + 15) / 16), dim3(128), 0, A, lda, rows, n, rmax,
        ks, static_cast<uint4*>(c.oz_a.p));
  }
  {
    ProfScope ps_(c, "k_oz_slice");
    GBCP_LAUNCH_PDL(c, k_oz_slice_mat, dim3((n + 127) / 128, (n + 7) / 8), dim3(128), 0, M, n, mcmax, ks,
        static_cast<uint4*>(c.oz_b.p), 0, n);
  }
  CUtensorMap ma, mb;
  if (!tmap_bf16_2d(&ma, c.oz_a.p, n, (long long)OZ_SL * rows, (int)ks, OZ_KS, OZ_M, 64) ||
      !tmap_bf16_2d(&mb, c.oz_b.p, n, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_N, 64)) {
    c.err = "C.M: tensor map encoding failed";
    return 5;
  }
  OzParams p{};
  p.M = rows;
  p.N = n;
  p.K = n;
  p.mode = 1;
  p.upper = upper;
  p.eA = rmax;
  p.eB = mcmax;
  p.Cout = Cout;
  p.ldo = ldo;
  p.zero_row1 = zero_row1;
  p.accumulate = accumulate;
  p.status = status;
  {
    allow_smem(k_oz_tc, OZ_SMEM);
    const int ntiles = ((rows + OZ_M - 1) / OZ_M) * ((n + OZ_N - 1) / OZ_N);
    const int nsm = c.nsm > 0 ? c.nsm : 148;
    // persistent CTAs: one per SM, or the tuned count (c.oz_rgrid)
    const int grid = std::max(1, std::min(ntiles, c.oz_rgrid > 0 ? c.oz_rgrid : nsm));
    ProfScope ps_(c, c.rmul_name ? c.rmul_name : "k_ozaki_rmul");
    GBCP_LAUNCH_PDL(c, k_oz_tc, dim3(grid), dim3(OZ_THREADS), OZ_SMEM, ma, mb, p);
  }
  return 0;
}

// S over the K ranges [kb[r], kb[r+1]) of the real view (boundaries multiples of
// OZ_KS): range r gets its own column exponents, digit planes and int64 partial
// sums once ready[r] (may be null) has completed on the stream, so that a host
// upload of range r+1 overlaps range r's work; the ranges are added in order in
// the finalize.  Queued without a host synchronisation.
int ovlap_tc_ranges(Ctx& c, const double* Ar, int lda, int n, const int* kb, int R, const cudaEvent_t* ready,
                    double* S, unsigned long long* scond_bits, int* status) {
  const int K = kb[R];
  const int nib = (n + OZ_M - 1) / OZ_M;
  const int njb = (n + OZ_N - 1) / OZ_N;
  int ntiles = 0;
  for (int ib = 0; ib < nib; ++ib) ntiles += std::max(0, njb - OZ_NB * ib);
  const size_t nn = (size_t)n * n;
  const size_t ks = ((size_t)K + 7) & ~size_t(7);
  const size_t bytes = (size_t)R * (2 * nn * 8 + (size_t)n * 8);
  if (!ensure(c, c.sparts, bytes) || !ensure(c, c.oz_a, sizeof(uint16_t) * OZ_SL * (size_t)n * ks)) return 6;
  unsigned long long* Hacc = static_cast<unsigned long long*>(c.sparts.p);
  unsigned long long* Lacc = Hacc + (size_t)R * nn;
  unsigned long long* cmax = Lacc + (size_t)R * nn;
  GBCP_CUDA_TRY(c, cudaMemsetAsync(Hacc, 0, bytes, c.stream));
  CUtensorMap ma, mb;
  if (!tmap_bf16_2d(&ma, c.oz_a.p, K, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_M, 64) ||
      !tmap_bf16_2d(&mb, c.oz_a.p, K, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_N, 64)) {
    c.err = "ovlap: tensor map encoding failed";
    return 5;
  }
  allow_smem(k_oz_tc, OZ_SMEM);
  for (int r = 0; r < R; ++r) {
    const int k0 = kb[r], Kr = kb[r + 1] - kb[r];
    if (Kr <= 0) continue;
    if (ready && ready[r]) GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, ready[r], 0));
    {
      ProfScope ps_(c, "k_col_max");
      const int kspl = std::max(1, std::min(64, (Kr + 4095) / 4096));
      const int kper = (Kr + kspl - 1) / kspl;
      GBCP_LAUNCH_PDL(c, k_col_max, dim3(n, kspl), dim3(256), 0, Ar + k0, lda, Kr, n, kper, cmax + (size_t)r * n);
    }
    {
      ProfScope ps_(c, "k_oz_slice");
      GBCP_LAUNCH_PDL(c, k_oz_slice_cols, dim3((Kr / 8 + 255) / 256 + 1, n), dim3(256), 0, Ar, lda, Kr, n,
          cmax + (size_t)r * n, ks, static_cast<uint4*>(c.oz_a.p), k0);
    }
    const int total_subs = (Kr + OZ_KS - 1) / OZ_KS;
    int nsplit = std::max(1, std::min((total_subs + OZ_SUBS - 1) / OZ_SUBS, (c.nsm > 0 ? c.nsm : 148) / std::max(1, ntiles)));
    int subs_per = (total_subs + nsplit - 1) / nsplit;
    subs_per = ((subs_per + OZ_SUBS - 1) / OZ_SUBS) * OZ_SUBS;
    nsplit = (total_subs + subs_per - 1) / subs_per;
    OzParams p{};
    p.M = n;
    p.N = n;
    p.K = Kr;
    p.mode = 0;
    p.njb = njb;
    p.subs_per = subs_per;
    p.sub_base = k0 / OZ_KS;
    p.Hacc = Hacc + (size_t)r * nn;
    p.Lacc = Lacc + (size_t)r * nn;
    p.status = status;
    if (c.test_stall && r == 0) {  // the test of the timeout path, first range of one call
      p.stall = 1;
      p.wait_limit = 2000000;
    }
    ProfScope ps_(c, "k_ozaki_syrk");
    GBCP_LAUNCH_PDL(c, k_oz_tc, dim3(ntiles, nsplit), dim3(OZ_THREADS), OZ_SMEM, ma, mb, p);
  }
  c.test_stall = 0;
  {
    ProfScope ps_(c, "k_ozaki_syrk_finalize");
    const int fb = std::max(1, std::min(1024, (int)((nn + 255) / 256)));
    GBCP_LAUNCH_PDL(c, k_ozaki_syrk_finalize_ranges, dim3(fb), dim3(256), 0, reinterpret_cast<const long long*>(Hacc),
        reinterpret_cast<const long long*>(Lacc), cmax, R, n, Ar, lda, c.geq0, S, scond_bits);
  }
  return 0;
}

// C M by row ranges [rb[r], rb[r+1]) (boundaries multiples of OZ_M): done[r] (may
// be null) is recorded once range r's rows of Cout are written, so that a host
// download of range r overlaps the later ranges.  Otherwise as rmul_tc.
int slice_rows_side(Ctx& c, const double* A, int lda, int rows, int n, const int* rb, int R,
                    const cudaEvent_t* ready, const cudaEvent_t** sliced) {
  if (n > 256 || n <= 0 || R <= 0) return 7;
  const size_t ks = ((size_t)n + 7) & ~size_t(7);
  if (!ensure(c, c.oz_c, sizeof(uint16_t) * OZ_SL * (size_t)rows * ks) ||
      !ensure(c, c.oz_rmax, sizeof(unsigned long long) * (size_t)rows))
    return 6;
  if (!c.side && cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking) != cudaSuccess) {
    c.err = "side stream";
    return 5;
  }
  while (c.side_ev.size() < (size_t)(R + 1)) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      c.err = "side stream events";
      return 5;
    }
    c.side_ev.push_back(e);
  }
  if (!ready) {  // A as queued so far on the context stream
    GBCP_CUDA_TRY(c, cudaEventRecord(c.side_ev[R], c.stream));
    GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.side, c.side_ev[R], 0));
  }
  unsigned long long* rmax = static_cast<unsigned long long*>(c.oz_rmax.p);
  for (int r = 0; r < R; ++r) {
    const int r0 = rb[r], r1 = rb[r + 1];
    if (ready && ready[r]) GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.side, ready[r], 0));
    if (r1 > r0) {
      ProfScope ps_(c, "k_oz_slice", c.side, 0);
      k_oz_slice_rows_max<<<(r1 - r0 + 31) / 32, dim3(32, (n + 15) / 16), 0, c.side>>>(
          A, lda, rows, n, rmax, ks, static_cast<uint4*>(c.oz_c.p), r0, r1);
      GBCP_LAUNCH_CHECK(c);
    }
    GBCP_CUDA_TRY(c, cudaEventRecord(c.side_ev[r], c.side));
  }
  *sliced = c.side_ev.data();
  return 0;
}

int rmul_tc_ranges(Ctx& c, const double* A, int lda, int rows, int n, const double* M, int upper, double* Cout,
                   int ldo, int zero_row1, int* status, const int* rb, int R, const cudaEvent_t* done,
                   const cudaEvent_t* sliced) {
  const size_t ks = ((size_t)n + 7) & ~size_t(7);
  const size_t bytes = ((size_t)rows + n) * 8;
  if (!ensure(c, c.nl_a, bytes) || (!sliced && !ensure(c, c.oz_a, sizeof(uint16_t) * OZ_SL * (size_t)rows * ks)) ||
      !ensure(c, c.oz_b, sizeof(uint16_t) * OZ_SL * (size_t)n * ks))
    return 6;
  if (sliced && (n > 256 || !c.oz_c.p || !c.oz_rmax.p)) return 7;
  unsigned long long* rmax =
      sliced ? static_cast<unsigned long long*>(c.oz_rmax.p) : static_cast<unsigned long long*>(c.nl_a.p);
  unsigned long long* mcmax = static_cast<unsigned long long*>(c.nl_a.p) + rows;
  void* planes = sliced ? c.oz_c.p : c.oz_a.p;
  {
    ProfScope ps_(c, "k_mat_col_max");
    GBCP_LAUNCH_PDL(c, k_mat_col_max, dim3((n + 31) / 32), dim3(32, 8), 0, M, n, mcmax, 0);
  }
  {
    ProfScope ps_(c, "k_oz_slice");
    if (n > 256) {  // no fused row-maximum slicer: all rows up front
      GBCP_LAUNCH_PDL(c, k_row_max, dim3((rows + 255) / 256), dim3(256), 0, A, lda, rows, n, rmax);
      GBCP_LAUNCH_PDL(c, k_oz_slice_rows, dim3((rows + 127) / 128, (n + 15) / 16), dim3(128), 0, A, lda, rows, n,
          rmax, ks, static_cast<uint4*>(c.oz_a.p));
    }
    GBCP_LAUNCH_PDL(c, k_oz_slice_mat, dim3((n + 127) / 128, (n + 7) / 8), dim3(128), 0, M, n, mcmax, ks,
        static_cast<uint4*>(c.oz_b.p), 0, n);
  }
  CUtensorMap ma, mb;
  if (!tmap_bf16_2d(&ma, planes, n, (long long)OZ_SL * rows, (int)ks, OZ_KS, OZ_M, 64) ||
      !tmap_bf16_2d(&mb, c.oz_b.p, n, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_N, 64)) {
    c.err = "C.M: tensor map encoding failed";
    return 5;
  }
  allow_smem(k_oz_tc, OZ_SMEM);
  const int nsm = c.nsm > 0 ? c.nsm : 148;
  const int nct = (n + OZ_N - 1) / OZ_N;
  for (int r = 0; r < R; ++r) {
    const int r0 = rb[r], r1 = rb[r + 1];
    if (r1 > r0) {
      if (sliced) {  // planes of this range written on the side stream
        GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, sliced[r], 0));
      } else if (n <= 256) {
        ProfScope ps_(c, "k_oz_slice");
        GBCP_LAUNCH_PDL(c, k_oz_slice_rows_max, dim3((r1 - r0 + 31) / 32), dim3(32, (n + 15) / 16), 0, A, lda, rows,
            n, rmax, ks, static_cast<uint4*>(c.oz_a.p), r0, r1);
      }
      OzParams p{};
      p.M = rows;
      p.N = n;
      p.K = n;
      p.mode = 1;
      p.upper = upper;
      p.eA = rmax;
      p.eB = mcmax;
      p.Cout = Cout;
      p.ldo = ldo;
      p.zero_row1 = zero_row1;
      p.status = status;
      p.rt0 = r0 / OZ_M;
      p.nrt = (r1 - r0 + OZ_M - 1) / OZ_M;
      const int grid = std::max(1, std::min(p.nrt * nct, nsm));
      ProfScope ps_(c, "k_ozaki_rmul");
      GBCP_LAUNCH_PDL(c, k_oz_tc, dim3(grid), dim3(OZ_THREADS), OZ_SMEM, ma, mb, p);
    }
    if (done && done[r]) GBCP_CUDA_TRY(c, cudaEventRecord(done[r], c.stream));
  }
  return 0;
}

// C U^-1 of column block k (columns 32 k .. 32 k + 31, K = 32 (k + 1) of the upper
// triangular M) into Cout, from the row planes and row maxima slice_rows_side cut
// into oz_c / oz_rmax (queued earlier on the stream this runs on): the block's column
// maxima and digit planes of M, then the persistent split GEMM over every row tile
// of that one column tile.  Per output element the arithmetic of rmul_tc_ranges.
int rmul_tc_column_block(Ctx& c, int rows, int n, const double* M, double* Cout, int ldo, int zero_row1,
                         int* status, int k) {
  static_assert(OZ_N == 32, "one column tile per Cholesky block");
  const size_t ks = ((size_t)n + 7) & ~size_t(7);
  if (n > 256 || !c.oz_c.p || !c.oz_rmax.p) return 7;
  if (!ensure(c, c.nl_a, ((size_t)rows + n) * 8) || !ensure(c, c.oz_b, sizeof(uint16_t) * OZ_SL * (size_t)n * ks))
    return 6;
  unsigned long long* rmax = static_cast<unsigned long long*>(c.oz_rmax.p);
  unsigned long long* mcmax = static_cast<unsigned long long*>(c.nl_a.p) + rows;
  const int j0 = k * OZ_N, j1 = std::min(n, j0 + OZ_N);
  {
    ProfScope ps_(c, "k_mat_col_max");
    GBCP_LAUNCH_PDL(c, k_mat_col_max, dim3(1), dim3(32, 8), 0, M, n, mcmax, j0);
  }
  {
    ProfScope ps_(c, "k_oz_slice");
    GBCP_LAUNCH_PDL(c, k_oz_slice_mat, dim3(1, (n + 7) / 8), dim3(32), 0, M, n, mcmax, ks,
        static_cast<uint4*>(c.oz_b.p), j0, j1);
  }
  CUtensorMap ma, mb;
  if (!tmap_bf16_2d(&ma, c.oz_c.p, n, (long long)OZ_SL * rows, (int)ks, OZ_KS, OZ_M, 64) ||
      !tmap_bf16_2d(&mb, c.oz_b.p, n, (long long)OZ_SL * n, (int)ks, OZ_KS, OZ_N, 64)) {
    c.err = "C.M: tensor map encoding failed";
    return 5;
  }
  allow_smem(k_oz_tc, OZ_SMEM);
  OzParams p{};
  p.M = rows;
  p.N = n;
  p.K = n;
  p.mode = 1;
  p.upper = 1;
  p.eA = rmax;
  p.eB = mcmax;
  p.Cout = Cout;
  p.ldo = ldo;
  p.zero_row1 = zero_row1;
  p.status = status;
  p.rt0 = 0;
  p.nrt = (rows + OZ_M - 1) / OZ_M;
  p.ct0 = k;
  p.nct = 1;
  const int nsm = c.nsm > 0 ? c.nsm : 148;
  ProfScope ps_(c, "k_ozaki_rmul");
  GBCP_LAUNCH_PDL(c, k_oz_tc, dim3(std::max(1, std::min(p.nrt, nsm))), dim3(OZ_THREADS), OZ_SMEM, ma, mb, p);
  return 0;
}

}  // namespace gbcp
