// Batched 1D mixed-radix FFT on lines held in shared memory.
//
// Each CTA owns `nl` lines of length N in shared memory, line l at
// buf + l*ls (ls >= N; an odd ls spreads lines over the banks).  A transform is a sequence of Stockham autosort passes
// (radices 2, 3, 4, 5, 8, product = N), ping-ponging between two shared
// buffers; the result ends in natural order, no bit-reversal pass.  For a
// pass of radix R after sub-transforms of size Ns, butterfly j reads
// in[j + r*N/R], applies the twiddle w^(r*(j mod Ns)) with w = e^{s 2 pi i /(Ns R)},
// does an R-point DFT and writes out[(j div Ns)*Ns*R + (j mod Ns) + r*Ns]
// (Govindaraju et al., "High performance discrete Fourier transforms on
// graphics processors", SC'08, the formulation used here).
//
// Sign convention: INV = true is e^{+i} (CPMD invfftn, isign=-1, FFTW_BACKWARD),
// INV = false is e^{-i} (fwfftn).  No scaling inside; callers scale.
//
// Twiddles: `tw[m] = e^{+2 pi i m / N}` for m in [0, N), filled on the host
// in FP64 (std::cos/std::sin of a reduced angle) and rounded once to float for
// the FP32 path.  The butterfly constants below are exact decimal expansions
// of cos/sin of multiples of pi/4, 2pi/3 and 2pi/5.
#pragma once
#include "common.cuh"

namespace gbcp {

constexpr int kMaxPasses = 8;

struct FftPlan {
  int n;                  // transform length
  int npass;              // number of passes
  int radix[kMaxPasses];  // radices in execution order
};

#define GBCP_C5_1 0.30901699437494742410
#define GBCP_C5_2 (-0.80901699437494742410)
#define GBCP_S5_1 0.95105651629515357212
#define GBCP_S5_2 0.58778525229247312917
#define GBCP_S3 0.86602540378443864676
#define GBCP_R2 0.70710678118654752440

template <int S, typename T> __device__ __forceinline__ void dft2(cx<T>* v) {
  cx<T> a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}

template <int S, typename T> __device__ __forceinline__ void dft4(cx<T>& v0, cx<T>& v1, cx<T>& v2, cx<T>& v3) {
  const cx<T> a0 = v0 + v2, a1 = v0 - v2, a2 = v1 + v3, d = v1 - v3;
  v0 = a0 + a2;
  v2 = a0 - a2;
  v1 = add_si<S>(a1, d);
  v3 = add_si<-S>(a1, d);
}

template <int S, typename T> __device__ __forceinline__ void dft3(cx<T>* v) {
  const T hs = (T)GBCP_S3;
  const cx<T> t1 = v[1] + v[2];
  const cx<T> t2 = cfma(v[0], (T)-0.5, t1);
  const cx<T> d = scl(v[1] - v[2], hs);
  v[0] = v[0] + t1;
  v[1] = add_si<S>(t2, d);
  v[2] = add_si<-S>(t2, d);
}

template <int S, typename T> __device__ __forceinline__ void dft5(cx<T>* v) {
  const T c1 = (T)GBCP_C5_1, c2 = (T)GBCP_C5_2, s1 = (T)GBCP_S5_1, s2 = (T)GBCP_S5_2;
  const cx<T> a = v[1] + v[4], b = v[2] + v[3], c = v[1] - v[4], d = v[2] - v[3];
  const cx<T> v0 = v[0];
  const cx<T> p1 = cfma(cfma(v0, c1, a), c2, b);
  const cx<T> p2 = cfma(cfma(v0, c2, a), c1, b);
  const cx<T> q1 = cfma(scl(c, s1), s2, d);
  const cx<T> q2 = cfma(scl(c, s2), -s1, d);
  v[0] = (v0 + a) + b;
  v[1] = add_si<S>(p1, q1);
  v[4] = add_si<-S>(p1, q1);
  v[2] = add_si<S>(p2, q2);
  v[3] = add_si<-S>(p2, q2);
}

template <int S, typename T> __device__ __forceinline__ void dft8(cx<T>* v) {
  cx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  cx<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<S>(e0, e1, e2, e3);
  dft4<S>(o0, o1, o2, o3);
  const T r = (T)GBCP_R2;
  // w8 = e^{S i pi/4}: (1 + S i)/sqrt2 o1 and (-1 + S i)/sqrt2 o3
  const cx<T> w1o = scl(add_si<S>(o1, o1), r);
  const cx<T> w3o = scl(add_si<S>(mk<T>(-o3.x, -o3.y), o3), r);
  v[0] = e0 + o0;
  v[4] = e0 - o0;
  v[1] = e1 + w1o;
  v[5] = e1 - w1o;
  v[2] = add_si<S>(e2, o2);  // e2 +- S i o2
  v[6] = add_si<-S>(e2, o2);
  v[3] = e3 + w3o;
  v[7] = e3 - w3o;
}

// dft8 for inputs v[2] .. v[5] known to be zero (only v[0], v[1], v[6], v[7] are
// read): the first butterflies of both length-4 halves reduce to copies, 16 of the
// 56 real additions go
template <int S, typename T> __device__ __forceinline__ void dft8_lo(cx<T>* v) {
  const cx<T> x0 = v[0], x1 = v[1], x6 = v[6], x7 = v[7];
  const cx<T> e0 = x0 + x6, e2 = x0 - x6, e1 = add_si<-S>(x0, x6), e3 = add_si<S>(x0, x6);
  const cx<T> o0 = x1 + x7, o2 = x1 - x7, o1 = add_si<-S>(x1, x7), o3 = add_si<S>(x1, x7);
  const T r = (T)GBCP_R2;
  const cx<T> w1o = scl(add_si<S>(o1, o1), r);
  const cx<T> w3o = scl(add_si<S>(mk<T>(-o3.x, -o3.y), o3), r);
  v[0] = e0 + o0;
  v[4] = e0 - o0;
  v[1] = e1 + w1o;
  v[5] = e1 - w1o;
  v[2] = add_si<S>(e2, o2);
  v[6] = add_si<-S>(e2, o2);
  v[3] = e3 + w3o;
  v[7] = e3 - w3o;
}

template <int S, int R, typename T> __device__ __forceinline__ void dft(cx<T>* v) {
  if constexpr (R == 2) dft2<S>(v);
  else if constexpr (R == 3) dft3<S>(v);
  else if constexpr (R == 4) dft4<S>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 5) dft5<S>(v);
  else if constexpr (R == 8) dft8<S>(v);
}

// One Stockham pass of radix R over nl lines.
template <bool INV, int R, typename T>
__device__ __forceinline__ void fft_pass(const cx<T>* __restrict__ in, cx<T>* __restrict__ out, int N, int nl,
                                         int ls, int Ns, const cx<T>* __restrict__ tw) {
  constexpr int S = INV ? 1 : -1;
  const int NR = N / R;
  const int tot = nl * NR;
  const int twmul = N / (Ns * R);
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int l = t / NR;
    const int j = t - l * NR;
    const cx<T>* src = in + l * ls;
    cx<T>* dst = out + l * ls;
    const int k = j % Ns;
    cx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[j + r * NR];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        cx<T> w = tw[k * r * twmul];
        v[r] = INV ? cmul(v[r], w) : cmulc(v[r], w);
      }
    }
    dft<S, R>(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[base + r * Ns] = v[r];
  }
}

// Full transform of nl lines.  `a` holds the input; `b` is scratch of the same
// size.  Returns the buffer that holds the result.  Contains __syncthreads();
// every thread of the CTA must call it.  The caller syncs before the first
// pass (after filling `a`); the function syncs after each pass.
template <bool INV, typename T>
__device__ cx<T>* fft_lines(cx<T>* a, cx<T>* b, int nl, int ls, const FftPlan& p, const cx<T>* __restrict__ tw) {
  int Ns = 1;
  for (int s = 0; s < p.npass; ++s) {
    const int R = p.radix[s];
    switch (R) {
      case 8: fft_pass<INV, 8>(a, b, p.n, nl, ls, Ns, tw); break;
      case 5: fft_pass<INV, 5>(a, b, p.n, nl, ls, Ns, tw); break;
      case 4: fft_pass<INV, 4>(a, b, p.n, nl, ls, Ns, tw); break;
      case 3: fft_pass<INV, 3>(a, b, p.n, nl, ls, Ns, tw); break;
      default: fft_pass<INV, 2>(a, b, p.n, nl, ls, Ns, tw); break;
    }
    __syncthreads();
    cx<T>* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

}  // namespace gbcp
