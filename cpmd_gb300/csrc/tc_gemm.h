// Split-bf16 tcgen05 GEMM (tc_gemm.cu): host interface.
#pragma once
#include <stdint.h>

struct CUtensorMap_st;

namespace gbcp {

struct Ctx;

// 2D bf16 tensor map over `rows` rows of K elements (row stride kstride elements,
// a multiple of 8), box of box_k x box_rows, swizzle 0 / 32 / 64 / 128 bytes.
bool tmap_bf16_2d(CUtensorMap_st* m, const void* base, int K, long long rows, int kstride, int box_k, int box_rows,
                  int swizzle_bytes);

constexpr int kTGMaxPairs = 6;

// K splits for an M x N output with K-long contraction that fill the SMs evenly.
int tc_gemm_ksplit(int M, int N, int K);
// Number of non-empty K splits the kernel actually runs for a requested ksplit.
int tc_gemm_splits_used(int M, int N, int K, int ksplit);

// D[m][n] = sum_q sum_k A_{ps[q]}[m][k] B_{pt[q]}[n][k]; slices are bf16 bit
// patterns, row-major with row stride `kstride` elements (a multiple of 8),
// slice s of A at rows [s*M, (s+1)*M).  mode 0: part[(split*N + n)*M + m] = D
// of each K split (ksplit requested; see tc_gemm_splits_used); mode 1:
// C[m + ldc*n] += D (FP64).  `status` (device int) becomes -2 if a bounded
// wait expired.  Queued on the context stream, no synchronisation.
int tc_gemm_split3(Ctx& c, const uint16_t* A, int M, const uint16_t* B, int N, int K, int kstride, int npairs,
                   const int* ps, const int* pt, int mode, float* part, int ksplit, double* C, long long ldc,
                   int* status);

}  // namespace gbcp
