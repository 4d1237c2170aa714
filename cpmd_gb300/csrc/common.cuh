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

// First statement of a kernel launched with launch_pdl: let the next kernel on
// the stream be scheduled, then wait until the previous one has finished and
// its writes are visible.  Harmless in a kernel launched the ordinary way.
__device__ __forceinline__ void pdl_entry() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Z stage of a vpsi on the states of the rhoofr before it: keep (null outside such
// a call) holds the states' checksums taken by both calls; equal, zbuf already holds
// the transforms and the kernel returns at once
__device__ __forceinline__ bool zk_kept(const unsigned long long* keep) {
  return keep != nullptr && keep[0] == keep[1];
}

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
// a + s b (scalar s)
template <typename T> __device__ __forceinline__ cx<T> cfma(cx<T> a, T s, cx<T> b) {
  return mk<T>(fma(s, b.x, a.x), fma(s, b.y, a.y));
}
// a + S i b (S = +1 or -1), without forming the swapped pair i b
template <int S, typename T> __device__ __forceinline__ cx<T> add_si(cx<T> a, cx<T> b) {
  return S > 0 ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x + b.y, a.y - b.x);
}

// FP32 complex values occupy a 64-bit register pair; sm_100-family packed
// instructions (add/sub/mul/fma .rn.f32x2) process both halves in one issue slot.
__device__ __forceinline__ unsigned long long f2_pack(cx<float> a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ cx<float> f2_unpack(unsigned long long r) {
  cx<float> a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
template <> __device__ __forceinline__ cx<float> operator+<float>(cx<float> a, cx<float> b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
template <> __device__ __forceinline__ cx<float> operator-<float>(cx<float> a, cx<float> b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
template <> __device__ __forceinline__ cx<float> scl<float>(cx<float> a, float s) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(mk<float>(s, s))));
  return f2_unpack(r);
}
template <> __device__ __forceinline__ cx<float> cfma<float>(cx<float> a, float s, cx<float> b) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_pack(b)), "l"(f2_pack(mk<float>(s, s))), "l"(f2_pack(a)));
  return f2_unpack(r);
}
// multiply by +i (S=+1) or -i (S=-1)
template <int S, typename T> __device__ __forceinline__ cx<T> mul_si(cx<T> a) {
  return S > 0 ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}

// ---- precision conversions on the integer pipe --------------------------
// On GB300 the FP64 pipe runs at 1/58 of the FP32 rate and also executes the
// F2F/I2F conversions to and from double; in the FP32 kernels those
// conversions alone kept the FP64 pipe a third busy.  These helpers convert
// by IEEE-754 bit manipulation with integer instructions instead.

// double -> float, round to nearest even; magnitudes below FLT_MIN flush to 0.
__device__ __forceinline__ float d2f_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int sign = (unsigned int)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (m ? 0x400000u : 0u));
  int ef = e - 1023 + 127;
  if (ef <= 0) return __uint_as_float(sign);
  unsigned int r = (unsigned int)(m >> 29);
  const unsigned int rem = (unsigned int)(m & 0x1FFFFFFFull);
  if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) {
    if (++r == 0x800000u) {
      r = 0;
      ++ef;
    }
  }
  if (ef >= 255) return __uint_as_float(sign | 0x7F800000u);
  return __uint_as_float(sign | ((unsigned int)ef << 23) | r);
}

// float -> double, exact; float subnormals flush to 0.
__device__ __forceinline__ double f2d_int(float y) {
  const unsigned int b = __float_as_uint(y);
  const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
  const int ef = (int)((b >> 23) & 0xFF);
  const unsigned long long m = b & 0x7FFFFFu;
  if (ef == 0) return __longlong_as_double((long long)sign);
  if (ef == 255) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull | (m << 29)));
  return __longlong_as_double((long long)(sign | ((unsigned long long)(ef - 127 + 1023) << 52) | (m << 29)));
}

template <typename T> __device__ __forceinline__ T from_double(double x);
template <> __device__ __forceinline__ double from_double<double>(double x) { return x; }
template <> __device__ __forceinline__ float from_double<float>(double x) { return d2f_int(x); }

// Status codes shared with the C ABI (include/cpmd_gb300.h).
enum DevStatus : int {
  DEV_OK = 0,
  DEV_NOT_SPD = 2,
  DEV_NONFINITE = 3,
};

}  // namespace gbcp
