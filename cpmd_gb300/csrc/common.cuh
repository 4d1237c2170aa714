// Shared device-side types for the GB300 wavefunction hot path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbcp {

// Complex number in registers / shared memory.  Layout matches double2 /
// float2 and the Fortran COMPLEX(real_8) interleaved (re, im) pair.
template <typename T> struct alignas(2 * sizeof(T)) cx {
  T x, y;
};

template <typename T> __host__ __device__ __forceinline__ cx<T> mk(T a, T b) { cx<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> __device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T> __device__ __forceinline__ cx<T> scl(cx<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
// multiply by +i (S=+1) or -i (S=-1)
template <int S, typename T> __device__ __forceinline__ cx<T> mul_si(cx<T> a) {
  return S > 0 ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}

// Status codes shared with the C ABI (include/cpmd_gb300.h).
enum DevStatus : int {
  DEV_OK = 0,
  DEV_NOT_SPD = 2,
  DEV_NONFINITE = 3,
};

}  // namespace gbcp
