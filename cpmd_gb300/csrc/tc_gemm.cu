// Split-bf16 GEMM on the tcgen05 tensor cores, fed by TMA: the engine of the
// mixed-precision projector contractions (rnlsm1 / fnonloc).
//
//   D[m][n] = sum_{(s,t) in pairs} sum_k A_s[m][k] B_t[n][k]
//
// A_s / B_t are bf16 "slices" of FP32 operands (x = x0 + x1 + x2, each x_j the
// bf16 rounding of the remainder, so x0 + x1 + x2 holds the 24-bit FP32
// significand).  With the six pairs s + t <= 2 the product carries the accuracy
// of an FP32 GEMM; all pairs accumulate into one FP32 accumulator in TMEM.
//
// Layout.  Slices are stored row-major, K contiguous, one matrix per slice
// stacked along rows (slice s = rows [s*M, (s+1)*M)), row stride a multiple of
// 16 bytes.  A 2D tensor map with 128-byte swizzle serves tiles of 64 K x 128
// rows (A) and 64 K x 256 rows (B) straight into the K-major SWIZZLE_128B
// layout of the MMA; out-of-range K and rows read as zero.
//
// Kernel.  Persistent, one CTA per SM, warp-specialised:
//   warp 0  TMA producer: 4-stage ring of (A 16 KB + B 32 KB) tiles, full/empty mbarriers;
//   warp 1  MMA issuer: per stage 4 x tcgen05.mma (M 128, N 256, K 16), commit frees the stage;
//   warp 2  allocates 512 TMEM columns = two 128 x 256 FP32 accumulators, so the
//           epilogue of one tile overlaps the MMAs of the next;
//   warps 4-7 epilogue: tcgen05.ld 32 lanes x 32 columns, then either FP32 split-K
//           partials (mode 0) or an FP64 read-modify-write C += D (mode 1).
// Work unit = (K split, M tile, N tile); consecutive units share the A tile.
// Every wait is bounded (about a second): on expiry the CTA raises the status
// word (-2), drains its own TMA loads and MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "ctx.h"
#include "tc_common.cuh"
#include "tc_gemm.h"

namespace gbcp {

namespace {

constexpr int TG_M = 128, TG_N = 256, TG_K = 64, TG_ST = 4;
constexpr int TG_A_BYTES = TG_M * TG_K * 2;  // 16 KB
constexpr int TG_B_BYTES = TG_N * TG_K * 2;  // 32 KB
constexpr int TG_STAGE = TG_A_BYTES + TG_B_BYTES;
constexpr int TG_SMEM = TG_ST * TG_STAGE + 1024;  // + slack for 1024-byte alignment
constexpr int TG_THREADS = 256;
constexpr uint32_t kIdescTG = tc::idesc_bf16_f32(TG_M, TG_N);

struct TGParams {
  int M, N;                  // rows per slice of A and of B
  int mt, nt, ksplit, kcps, nkc;  // M tiles, N tiles, K splits, K chunks per split, K chunks
  int npairs;
  int ps[kTGMaxPairs], pt[kTGMaxPairs];
  int mode;                  // 0: FP32 partials; 1: FP64 C += D
  float* part;               // mode 0: part[(split * N + n) * M + m]
  double* C;                 // mode 1: C[m + ldc * n]
  long long ldc;
  int* status;
};

__device__ __forceinline__ bool aborted(const volatile int* f) { return *f != 0; }

__global__ void __launch_bounds__(TG_THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const TGParams p) {
  extern __shared__ uint8_t tg_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tg_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full[TG_ST], empty[TG_ST], tfull[2], tempty[2], mdone;
  __shared__ uint32_t tmem_sh;
  __shared__ volatile int abort_sh;
  __shared__ int issued_sh, consumed_sh;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < TG_ST; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], 4);
    }
    tc::mbar_init(&mdone, 1);
    tc::fence_mbar_init();
    abort_sh = 0;
    issued_sh = 0;
    consumed_sh = 0;
  }
  if (warp == 2) {
    tc::tmem_alloc(&tmem_sh, 512);
    tc::tmem_relinquish();
  }
  if (warp == 0 && lane == 0) {
    tc::tma_prefetch_desc(&tmA);
    tc::tma_prefetch_desc(&tmB);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_sh;
  const int units = p.mt * p.nt * p.ksplit;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int stage = 0, issued = 0;
    uint32_t ph = 0;
    for (int u = blockIdx.x; u < units && !aborted(&abort_sh); u += gridDim.x) {
      const int split = u / (p.mt * p.nt), r = u % (p.mt * p.nt);
      const int m0 = (r / p.nt) * TG_M, n0 = (r % p.nt) * TG_N;
      const int kc0 = split * p.kcps, kc1 = min(p.nkc, kc0 + p.kcps);
      for (int kc = kc0; kc < kc1 && !aborted(&abort_sh); ++kc) {
        for (int q = 0; q < p.npairs; ++q) {
          if (!tc::mbar_wait(&empty[stage], ph ^ 1u)) {
            abort_sh = 1;
            atomicExch(p.status, -2);
            break;
          }
          uint8_t* sa = sm + stage * TG_STAGE;
          tc::mbar_expect_tx(&full[stage], TG_STAGE);
          tc::tma_load_2d(sa, &tmA, &full[stage], kc * TG_K, p.ps[q] * p.M + m0);
          tc::tma_load_2d(sa + TG_A_BYTES, &tmB, &full[stage], kc * TG_K, p.pt[q] * p.N + n0);
          ++issued;
          if (++stage == TG_ST) {
            stage = 0;
            ph ^= 1u;
          }
        }
      }
    }
    issued_sh = issued;
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    int stage = 0, acc = 0, consumed = 0;
    uint32_t ph = 0, aph = 0;
    for (int u = blockIdx.x; u < units && !aborted(&abort_sh); u += gridDim.x) {
      const int split = u / (p.mt * p.nt);
      const int kc0 = split * p.kcps, kc1 = min(p.nkc, kc0 + p.kcps);
      if (!tc::mbar_wait(&tempty[acc], aph ^ 1u)) {
        abort_sh = 1;
        atomicExch(p.status, -2);
        break;
      }
      tc::fence_after_sync();
      const uint32_t d = tmem + (uint32_t)(acc * TG_N);
      bool first = true, ok = true;
      for (int kc = kc0; kc < kc1 && ok; ++kc) {
        for (int q = 0; q < p.npairs; ++q) {
          if (!tc::mbar_wait(&full[stage], ph)) {
            abort_sh = 1;
            atomicExch(p.status, -2);
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t sa = tc::smem_u32(sm + stage * TG_STAGE);
          const uint32_t sb = sa + TG_A_BYTES;
#pragma unroll
          for (int kk = 0; kk < TG_K / 16; ++kk)
            tc::mma_f16(d, tc::sdesc_kmajor_sw128(sa + 32 * kk), tc::sdesc_kmajor_sw128(sb + 32 * kk), kIdescTG,
                        (first && kk == 0) ? 0u : 1u);
          first = false;
          tc::mma_commit(&empty[stage]);
          ++consumed;
          if (++stage == TG_ST) {
            stage = 0;
            ph ^= 1u;
          }
        }
      }
      if (!ok) break;
      tc::mma_commit(&tfull[acc]);
      acc ^= 1;
      if (acc == 0) aph ^= 1u;
    }
    consumed_sh = consumed;
    // all MMAs of this thread complete before TMEM is released
    tc::mma_commit(&mdone);
    if (!tc::mbar_wait(&mdone, 0)) atomicExch(p.status, -2);
  } else if (warp >= 4) {
    // ---------------- epilogue
    const int q4 = warp & 3;
    int acc = 0;
    uint32_t aph = 0;
    for (int u = blockIdx.x; u < units && !aborted(&abort_sh); u += gridDim.x) {
      const int split = u / (p.mt * p.nt), r = u % (p.mt * p.nt);
      const int m0 = (r / p.nt) * TG_M, n0 = (r % p.nt) * TG_N;
      // warp-uniform outcome: the TMEM loads below are .sync.aligned
      if (!__all_sync(0xffffffffu, tc::mbar_wait(&tfull[acc], aph) ? 1 : 0)) {
        abort_sh = 1;
        atomicExch(p.status, -2);
        break;
      }
      tc::fence_after_sync();
      const int row = m0 + 32 * q4 + lane;
      const uint32_t taddr = tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(acc * TG_N);
#pragma unroll 1
      for (int cc = 0; cc < TG_N / 32; ++cc) {
        uint32_t v[32];
        tc::tmem_ld32(taddr + 32 * cc, v);
        tc::tmem_ld_wait();
        if (row < p.M) {
          const int col0 = n0 + 32 * cc;
          if (p.mode == 0) {
            float* o = p.part + ((size_t)split * p.N) * p.M + row;
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (col0 + j < p.N) o[(size_t)(col0 + j) * p.M] = __uint_as_float(v[j]);
          } else {
            // all 32 loads in flight before the first store; the FP32 -> FP64
            // conversion runs on the integer pipe (the FP64 pipe is 1/58 of FP32)
            double* __restrict__ o = p.C + row;
            const int nc = min(32, p.N - col0);
            double old[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) old[j] = (j < nc) ? o[(size_t)(col0 + j) * p.ldc] : 0.0;
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (j < nc) o[(size_t)(col0 + j) * p.ldc] = old[j] + f2d_int(__uint_as_float(v[j]));
          }
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&tempty[acc]);
      acc ^= 1;
      if (acc == 0) aph ^= 1u;
    }
  }

  __syncthreads();
  if (abort_sh && threadIdx.x == 0) {
    // loads issued but never consumed still land in shared memory: wait for them
    for (int j = consumed_sh; j < issued_sh; ++j) tc::mbar_wait(&full[j % TG_ST], (uint32_t)((j / TG_ST) & 1));
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 2) {
    __syncwarp();
    tc::tmem_dealloc(tmem, 512);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}


}  // namespace

bool tmap_bf16_2d(CUtensorMap* m, const void* base, int K, long long rows, int kstride, int box_k, int box_rows,
                  int swizzle_bytes) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kstride * 2};
  cuuint32_t box[2] = {(cuuint32_t)box_k, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  const CUtensorMapSwizzle sw = swizzle_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                : swizzle_bytes == 64  ? CU_TENSOR_MAP_SWIZZLE_64B
                                : swizzle_bytes == 32  ? CU_TENSOR_MAP_SWIZZLE_32B
                                                       : CU_TENSOR_MAP_SWIZZLE_NONE;
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

namespace {

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

}  // namespace

int tc_gemm_ksplit(int M, int N, int K) {
  const int tiles = ((M + TG_M - 1) / TG_M) * ((N + TG_N - 1) / TG_N);
  const int nkc = (K + TG_K - 1) / TG_K;
  const int nsm = num_sms();
  int best = 1;
  double best_cost = 1e300;
  for (int ks = 1; ks <= 32 && ks <= nkc; ++ks) {
    const double waves = (double)((tiles * ks + nsm - 1) / nsm);
    const double cost = waves / ks * (1.0 + 0.01 * ks);
    if (cost < best_cost) {
      best_cost = cost;
      best = ks;
    }
  }
  return best;
}

int tc_gemm_split3(Ctx& c, const uint16_t* A, int M, const uint16_t* B, int N, int K, int kstride, int npairs,
                   const int* ps, const int* pt, int mode, float* part, int ksplit, double* C, long long ldc,
                   int* status) {
  if (kstride % 8 != 0 || K > kstride || npairs < 1 || npairs > kTGMaxPairs) {
    c.err = "tc_gemm: bad layout";
    return 1;
  }
  int nslA = 0, nslB = 0;
  for (int q = 0; q < npairs; ++q) {
    nslA = std::max(nslA, ps[q] + 1);
    nslB = std::max(nslB, pt[q] + 1);
  }
  CUtensorMap ma, mb;
  if (!tmap_bf16_2d(&ma, A, K, (long long)nslA * M, kstride, TG_K, TG_M, 128) ||
      !tmap_bf16_2d(&mb, B, K, (long long)nslB * N, kstride, TG_K, TG_N, 128)) {
    c.err = "tc_gemm: tensor map encoding failed";
    return 5;
  }
  TGParams p{};
  p.M = M;
  p.N = N;
  p.mt = (M + TG_M - 1) / TG_M;
  p.nt = (N + TG_N - 1) / TG_N;
  p.nkc = (K + TG_K - 1) / TG_K;
  if (mode == 1) ksplit = 1;
  ksplit = std::max(1, std::min(ksplit, p.nkc));
  p.kcps = (p.nkc + ksplit - 1) / ksplit;
  p.ksplit = (p.nkc + p.kcps - 1) / p.kcps;  // no empty split
  p.npairs = npairs;
  for (int q = 0; q < npairs; ++q) {
    p.ps[q] = ps[q];
    p.pt[q] = pt[q];
  }
  p.mode = mode;
  p.part = part;
  p.C = C;
  p.ldc = ldc;
  p.status = status;
  const int units = p.mt * p.nt * p.ksplit;
  const int grid = std::min(units, num_sms());
  allow_smem(k_tc_gemm, TG_SMEM);
  ProfScope ps_(c, "k_tc_gemm");
  k_tc_gemm<<<grid, TG_THREADS, TG_SMEM, c.stream>>>(ma, mb, p);
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

int tc_gemm_splits_used(int M, int N, int K, int ksplit) {
  const int nkc = (K + TG_K - 1) / TG_K;
  ksplit = std::max(1, std::min(ksplit, nkc));
  const int kcps = (nkc + ksplit - 1) / ksplit;
  return (nkc + kcps - 1) / kcps;
}

}  // namespace gbcp
