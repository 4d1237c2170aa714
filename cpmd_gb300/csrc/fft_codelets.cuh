// Register DFT codelets of length 2..20 (2,3,5-smooth) for the four-step FFT.
//
// dftn<S, R>(v) transforms R values held in registers in place,
// V[k] = sum_r v[r] e^{S 2 pi i r k / R} (S = +1 inverse, -1 forward), output in
// natural order.  Lengths 2, 3, 4, 5, 8 use the butterflies of fft_core.cuh;
// composite lengths with coprime factors (6 = 2*3, 10 = 2*5, 12 = 4*3,
// 15 = 3*5, 20 = 4*5) use the prime-factor (Good-Thomas) mapping, which needs
// no twiddle factors: with N = A*B, input x[(B a + A b) mod N], a DFT of length
// A over a, a DFT of length B over b, and output index
// (B (B^-1 mod A) k_a + A (A^-1 mod B) k_b) mod N (Chinese remainder theorem).
// Every index is a compile-time constant, so the codelets are pure register code.
#pragma once
#include "fft_core.cuh"

namespace gbcp {

__host__ __device__ constexpr int inv_mod(int a, int m) {
  for (int x = 1; x < m; ++x)
    if ((a * x) % m == 1) return x;
  return 1;
}

template <int S, int R, typename T> __device__ __forceinline__ void dftn(cx<T>* v);

template <int S, int A, int B, typename T> __device__ __forceinline__ void dft_pfa(cx<T>* v) {
  constexpr int N = A * B;
  constexpr int Binv = inv_mod(B % A, A), Ainv = inv_mod(A % B, B);
  cx<T> u[A][B];
#pragma unroll
  for (int a = 0; a < A; ++a)
#pragma unroll
    for (int b = 0; b < B; ++b) u[a][b] = v[(B * a + A * b) % N];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    cx<T> t[A];
#pragma unroll
    for (int a = 0; a < A; ++a) t[a] = u[a][b];
    dftn<S, A>(t);
#pragma unroll
    for (int a = 0; a < A; ++a) u[a][b] = t[a];
  }
#pragma unroll
  for (int ka = 0; ka < A; ++ka) {
    cx<T> t[B];
#pragma unroll
    for (int b = 0; b < B; ++b) t[b] = u[ka][b];
    dftn<S, B>(t);
#pragma unroll
    for (int kb = 0; kb < B; ++kb) v[(B * Binv * ka + A * Ainv * kb) % N] = t[kb];
  }
}

template <int S, int R, typename T> __device__ __forceinline__ void dftn(cx<T>* v) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2 || R == 3 || R == 4 || R == 5 || R == 8) {
    dft<S, R>(v);
  } else if constexpr (R == 6) {
    dft_pfa<S, 2, 3>(v);
  } else if constexpr (R == 10) {
    dft_pfa<S, 2, 5>(v);
  } else if constexpr (R == 12) {
    dft_pfa<S, 4, 3>(v);
  } else if constexpr (R == 15) {
    dft_pfa<S, 3, 5>(v);
  } else if constexpr (R == 20) {
    dft_pfa<S, 4, 5>(v);
  } else {
    static_assert(R == 2, "unsupported codelet length");
  }
}

}  // namespace gbcp
