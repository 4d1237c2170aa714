// Compile-time-planned batched 1D FFT on lines in shared memory.
//
// Same Stockham autosort passes as fft_core.cuh, but the transform length N,
// the radix sequence, the number of lines per CTA and the CTA size are
// template parameters, so every loop bound, divisor and stride is a constant
// and the butterfly loops unroll.  The mesh sizes of the supported cells
// (2,3,5-smooth, gfft_utils.mod.F90:39-84) each get a plan below; other sizes
// fall back to the run-time planned transform of fft_core.cuh.
#pragma once
#include "fft_core.cuh"

namespace gbcp {

template <int... Rs> struct Radices {};

// radix sequence per transform length (execution order)
template <int N> struct CtPlan { static constexpr bool ok = false; using type = Radices<>; };
#define GBCP_PLAN(NN, ...)                      \
  template <> struct CtPlan<NN> {               \
    static constexpr bool ok = true;            \
    using type = Radices<__VA_ARGS__>;          \
  };
GBCP_PLAN(32, 8, 4)
GBCP_PLAN(36, 4, 3, 3)
GBCP_PLAN(40, 8, 5)
GBCP_PLAN(48, 4, 4, 3)
GBCP_PLAN(60, 5, 4, 3)
GBCP_PLAN(64, 8, 8)
GBCP_PLAN(72, 8, 3, 3)
GBCP_PLAN(80, 5, 4, 4)
GBCP_PLAN(96, 8, 4, 3)
GBCP_PLAN(120, 8, 5, 3)
GBCP_PLAN(144, 4, 4, 3, 3)
GBCP_PLAN(240, 8, 5, 3, 2)
#undef GBCP_PLAN

__host__ __device__ constexpr int ct_stride(int n) { return (n % 2 == 0) ? n + 1 : n; }

// one pass, all constants known
template <bool INV, typename T, int N, int R, int NS, int NL, int NT>
__device__ __forceinline__ void ct_pass(const cx<T>* __restrict__ in, cx<T>* __restrict__ out,
                                        const cx<T>* __restrict__ tw) {
  constexpr int S = INV ? 1 : -1;
  constexpr int LS = ct_stride(N);
  constexpr int NR = N / R;
  constexpr int TOT = NL * NR;
  constexpr int TWMUL = N / (NS * R);
  constexpr int ITERS = (TOT + NT - 1) / NT;
#pragma unroll
  for (int it = 0; it < ITERS; ++it) {
    const int t = (int)threadIdx.x + it * NT;
    if ((TOT % NT == 0) || t < TOT) {
      const int l = t / NR;
      const int j = t - l * NR;
      const int k = (NS == 1) ? 0 : j % NS;
      const cx<T>* src = in + l * LS;
      cx<T>* dst = out + l * LS;
      cx<T> v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = src[j + r * NR];
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const cx<T> w = tw[k * r * TWMUL];
          v[r] = INV ? cmul(v[r], w) : cmulc(v[r], w);
        }
      }
      dft<S, R>(v);
      const int base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) dst[base + r * NS] = v[r];
    }
  }
}

template <bool INV, typename T, int N, int NL, int NT, int NS>
__device__ __forceinline__ cx<T>* ct_run(cx<T>* a, cx<T>*, const cx<T>*, Radices<>) {
  return a;
}

template <bool INV, typename T, int N, int NL, int NT, int NS, int R, int... Rest>
__device__ __forceinline__ cx<T>* ct_run(cx<T>* a, cx<T>* b, const cx<T>* tw, Radices<R, Rest...>) {
  ct_pass<INV, T, N, R, NS, NL, NT>(a, b, tw);
  __syncthreads();
  return ct_run<INV, T, N, NL, NT, NS * R>(b, a, tw, Radices<Rest...>{});
}

// Transform NL lines of length N held at a (line stride ct_stride(N)); b is
// scratch.  Returns the buffer holding the result.  Caller syncs before.
template <bool INV, typename T, int N, int NL, int NT>
__device__ __forceinline__ cx<T>* fft_ct(cx<T>* a, cx<T>* b, const cx<T>* tw) {
  return ct_run<INV, T, N, NL, NT, 1>(a, b, tw, typename CtPlan<N>::type{});
}

}  // namespace gbcp
