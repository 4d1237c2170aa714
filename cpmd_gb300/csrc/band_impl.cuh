// Band loop of the Γ-point hot path: rhoofr and vpsi as a pruned 3D FFT.
//
// Reference data flow (rhoofr_utils.mod.F90:305-409, vpsi_utils.mod.F90:376-675):
// for each pair of states, pack c1 + i c2 on the sphere (state_utils.mod.F90:
// 165-189), inverse 3D FFT (fftmain_utils.mod.F90:90-104), accumulate density
// or multiply by V and transform forward (l.122-136), decode.
//
// GB300 data flow per batch of pairs (one launch per stage, all pairs of the
// batch in the grid):
//   Z stage  gather the sphere column (gx,gy) straight from c0, FFT along z
//            -> zbuf[pair][z][col]            (only sphere columns exist)
//   Y stage  per z-plane and gx slot, FFT along y
//            -> ybuf[pair][z][y][slot]        (only |gx| inside the sphere)
//   X stage  per (y,z) line, FFT along x, then
//            rhoofr: rho += f1/omega Re^2 + f2/omega Im^2 (registers, all pairs)
//            vpsi:   x V(r), forward FFT along x, keep the sphere slots
// and for vpsi the mirror Y and Z stages forward, then a decode kernel that
// forms fp/fm from +G/-G and adds the kinetic term into c2.
// psi(r) never reaches HBM.  The all-to-all of the reference
// (fftutil_utils.mod.F90:292-319) becomes the layout change between stages.
//
// The mesh sizes of the supported cells (2,3,5-smooth, the reference's own
// size table gfft_utils.mod.F90:39-84) run the four-step kernels of
// band_fs.cuh (register codelets, one shared-memory exchange per transform);
// any other size runs the Stockham kernels below with a run-time radix plan.
// This header is included by band64.cu and band32.cu, one per precision.
#pragma once
#include <algorithm>
#include <cmath>

#include "ctx.h"
#include "fft_core.cuh"

namespace gbcp {
namespace band {

constexpr int kThreads = 256;
constexpr int kElems = 2048;   // complex elements per CTA tile (lines * length)
constexpr int kMaxAcc = 16;    // density accumulators per thread (run-time plan)

__host__ __device__ constexpr int line_stride(int n) { return (n % 2 == 0) ? n + 1 : n; }
__device__ __forceinline__ int freq_of(int i, int n) { return (i < (n + 1) / 2) ? i : i - n; }
// frequency of index a + W b of a length-N transform, 0 <= a < W, b an unrolled
// loop index: the branch folds at compile time except for the one row of W that
// holds the Nyquist boundary
template <int N, int W> __device__ __forceinline__ int freq_split(int a, int b) {
  constexpr int h = (N + 1) / 2;
  const int i = a + W * b;
  if (W * b + W - 1 < h) return i;
  if (W * b >= h) return i - N;
  return i < h ? i : i - N;
}
// 0 <= v < n in one unsigned compare
__device__ __forceinline__ bool in_range(int v, int n) { return (unsigned)v < (unsigned)n; }
__device__ __forceinline__ int idx_of(int g, int n) { return g < 0 ? g + n : g; }

template <typename T>
__device__ __forceinline__ void load_tw(cx<T>* tw, const cx<T>* __restrict__ twg, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = twg[i];
}

template <bool INV, typename T, int NC>
__device__ __forceinline__ cx<T>* run_fft(cx<T>* a, cx<T>* b, int nl, int ls, const FftPlan& p,
                                          const cx<T>* tw) {
  return fft_lines<INV>(a, b, nl, ls, p, tw);
}

// stage geometry: length N, line stride LS, lines per CTA NL
#define GBCP_STAGE(NAXIS, NLRT)                                   \
  const int N = (NAXIS);                                          \
  const int ls = line_stride(N);                                  \
  const int nl = (NLRT);                                          \
  extern __shared__ __align__(16) unsigned char smem_raw[];       \
  cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);                 \
  cx<T>* a = tw + N;                                              \
  cx<T>* b = a + nl * ls;

// ---------------------------------------------------------------- rhoofr scalars in the Z-stage gather
// The gather of rhoofr's Z stage holds every coefficient of the pair once as a
// +G entry, so the kinetic energy E_kin = tpiba2 sum_i f_i sum_G hg |c_i(G)|^2
// (kin_energy_utils.mod.F90:93-108; the 1/2 and the x2 of the half sphere
// cancel) and the Γ norm csumg = sum_i f_i <c_i|c_i> (2|c|^2, Re c^2 at G = 0;
// dotp_utils.mod.F90:45-52, rhoofr_utils.mod.F90:607-635) are summed there, with
// no second read of c0.  Each CTA writes its two occupation-weighted totals to
// kpart[2 b], kpart[2 b + 1], b = global pair * (column blocks) + column block.
// FP64 kernels sum in FP64.  FP32 kernels square the FP32-rounded coefficients
// (relative rounding 2^-24 per coefficient, unbiased), add a thread's few terms
// (at most N1 per line it owns) in FP32 and combine the threads of a warp in
// double-float (Knuth's TwoSum), so the summation error stays far below the
// coefficient rounding and the FP64 pipe, 1/58 of the FP32 rate on GB300, is
// used once per warp.
__device__ __forceinline__ void df_add(float& hi, float& lo, float bh, float bl) {
  const float s = hi + bh;
  const float v = s - hi;
  float e = (hi - (s - v)) + (bh - v);
  e += lo + bl;
  hi = s + e;
  lo = e - (hi - s);
}

template <typename T> struct KinAcc;
template <> struct KinAcc<double> {
  double k1 = 0.0, n1 = 0.0, k2 = 0.0, n2 = 0.0;
  __device__ __forceinline__ void add(double hg, double, bool g0, double ux, double uy, double wx, double wy) {
    const double a1 = fma(ux, ux, uy * uy), a2 = fma(wx, wx, wy * wy);
    k1 = fma(hg, a1, k1);
    k2 = fma(hg, a2, k2);
    n1 += g0 ? ux * ux : 2.0 * a1;
    n2 += g0 ? wx * wx : 2.0 * a2;
  }
  // warp totals, FP64
  __device__ __forceinline__ void warp_totals(double (&o)[4]) {
    o[0] = k1; o[1] = n1; o[2] = k2; o[3] = n2;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
#pragma unroll
      for (int q = 0; q < 4; ++q) o[q] += __shfl_down_sync(0xffffffffu, o[q], d);
  }
};
template <> struct KinAcc<float> {
  float k1 = 0.f, n1 = 0.f, k2 = 0.f, n2 = 0.f;
  __device__ __forceinline__ void add(double, float hg, bool g0, float ux, float uy, float wx, float wy) {
    const float a1 = fmaf(ux, ux, uy * uy), a2 = fmaf(wx, wx, wy * wy);
    k1 = fmaf(hg, a1, k1);
    k2 = fmaf(hg, a2, k2);
    n1 += g0 ? ux * ux : 2.f * a1;
    n2 += g0 ? wx * wx : 2.f * a2;
  }
  // warp totals as double-float pairs (h + l)
  __device__ __forceinline__ void warp_totals(float (&h)[4], float (&l)[4]) {
    h[0] = k1; h[1] = n1; h[2] = k2; h[3] = n2;
#pragma unroll
    for (int q = 0; q < 4; ++q) l[q] = 0.f;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        df_add(h[q], l[q], __shfl_down_sync(0xffffffffu, h[q], d), __shfl_down_sync(0xffffffffu, l[q], d));
  }
};

// coefficient idx of c0 as stored (complex128, or complex64 with psi32) in the
// kernel's precision
template <typename T>
__device__ __forceinline__ void load_coef(const cx<double>* __restrict__ c0, int psi32, size_t idx, T& x, T& y) {
  if (psi32) {
    const cx<float> a = reinterpret_cast<const cx<float>*>(c0)[idx];
    x = (T)a.x;
    y = (T)a.y;
  } else {
    const cx<double> a = c0[idx];
    x = from_double<T>(a.x);
    y = from_double<T>(a.y);
  }
}

// One +G entry (e > 0) of the gather: u, w the two states' coefficients as the
// kernel holds them (FP64, or FP32-rounded).
__device__ __forceinline__ void kin_entry(KinAcc<double>& acc, const GeoDev& g, int ig, double ux, double uy,
                                          double wx, double wy) {
  acc.add(g.hg[ig], 0.0, g.geq0 && ig == 0, ux, uy, wx, wy);
}
__device__ __forceinline__ void kin_entry(KinAcc<float>& acc, const GeoDev& g, int ig, float ux, float uy, float wx,
                                          float wy) {
  acc.add(0.0, g.hg32[ig], g.geq0 && ig == 0, ux, uy, wx, wy);
}
// the same with hg taken from the Z-stage gather table (FP32); FP64 reads hg[ig]
__device__ __forceinline__ void kin_entry_t(KinAcc<double>& acc, const GeoDev& g, int ig, float, double ux, double uy,
                                            double wx, double wy) {
  kin_entry(acc, g, ig, ux, uy, wx, wy);
}
__device__ __forceinline__ void kin_entry_t(KinAcc<float>& acc, const GeoDev& g, int ig, float hge, float ux, float uy,
                                            float wx, float wy) {
  acc.add(0.0, hge, g.geq0 && ig == 0, ux, uy, wx, wy);
}

// CTA totals weighted by f1, f2 into out[0..1].  Every thread of the CTA calls it.
__device__ __forceinline__ void kin_flush(KinAcc<double>& acc, double f1, double f2, double* __restrict__ out) {
  __shared__ double wsum[kThreads / 32][4];
  double o[4];
  acc.warp_totals(o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 4; ++q) wsum[warp][q] = o[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
#pragma unroll
      for (int q = 0; q < 4; ++q) t[q] += wsum[w][q];
    out[0] = f1 * t[0] + f2 * t[2];
    out[1] = f1 * t[1] + f2 * t[3];
  }
}
// FP32 kernels: the warp and CTA sums stay double-float and out[0..1] receives
// (kin hi, kin lo, norm hi, norm lo) as four floats, converted by the fold
// (k_rho_scalars), so that the gather kernel issues almost no FP64 instruction
// (each holds an SM sub-partition for ~64 clocks on GB300)
__device__ __forceinline__ void df_mul_add(float& h, float& l, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  const float e = fmaf(al, bh, fmaf(ah, bl, fmaf(ah, bh, -p)));
  df_add(h, l, p, e);
}
__device__ __forceinline__ void kin_flush(KinAcc<float>& acc, double f1, double f2, double* __restrict__ out) {
  // one partial per warp (no CTA barrier, no serial CTA sum): out + 2 warp
  float h[4], l[4];
  acc.warp_totals(h, l);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    const float f1h = d2f_int(f1), f1l = d2f_int(f1 - f2d_int(f1h));
    const float f2h = d2f_int(f2), f2l = d2f_int(f2 - f2d_int(f2h));
    float kh = 0.f, kl = 0.f, nh = 0.f, nl = 0.f;
    df_mul_add(kh, kl, f1h, f1l, h[0], l[0]);
    df_mul_add(kh, kl, f2h, f2l, h[2], l[2]);
    df_mul_add(nh, nl, f1h, f1l, h[1], l[1]);
    df_mul_add(nh, nl, f2h, f2l, h[3], l[3]);
    reinterpret_cast<float4*>(out)[warp] = make_float4(kh, kl, nh, nl);
  }
}
// E_kin / norm partial slots per CTA of a Z-stage kernel: one (FP64), one per warp (FP32)
template <typename T> __host__ __device__ constexpr int kin_slots() { return sizeof(T) == 4 ? kThreads / 32 : 1; }

// ---------------------------------------------------------------- Z stage (inverse, gather)
template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) k_zinv(GeoDev g, FftPlan p, const cx<double>* __restrict__ c0, int psi32,
                                                  int ldc, int s0, int nstate, int nlrt, cx<T>* __restrict__ zbuf,
                                                  const cx<T>* __restrict__ twg, const double* __restrict__ f,
                                                  double* __restrict__ kpart, const unsigned long long* keep) {
  if (zk_kept(keep)) return;
  GBCP_STAGE(g.n3, nlrt)
  const int pair = blockIdx.y;
  const int col0 = blockIdx.x * nl;
  const int is1 = s0 + 2 * pair, is2 = is1 + 1;
  const bool two = is2 < nstate;
  const size_t o1 = (size_t)is1 * ldc, o2 = (size_t)(two ? is2 : is1) * ldc;
  KinAcc<T> kacc;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int l = idx / N, z = idx - l * N, col = col0 + l;
    cx<T> v = mk<T>(0, 0);
    if (col < g.ncol) {
      const int st = g.col_start[col], len = g.col_start[col + 1] - st;
      const int off = freq_of(z, N) - g.col_zlo[col];
      if (off >= 0 && off < len) {
        const int e = g.col_ent[st + off];
        if (e != 0) {
          const int ig = (e > 0 ? e : -e) - 1;
          T ux, uy, wx = 0, wy = 0;
          load_coef<T>(c0, psi32, o1 + ig, ux, uy);
          if (two) load_coef<T>(c0, psi32, o2 + ig, wx, wy);
          // +G: c1 + i c2 ; -G: conj(c1) + i conj(c2)
          v = (e > 0) ? mk<T>(ux - wy, uy + wx) : mk<T>(ux + wy, wx - uy);
          if (kpart && e > 0) kin_entry(kacc, g, ig, ux, uy, wx, wy);
        }
      }
    }
    a[l * ls + z] = v;
  }
  __syncthreads();
  const cx<T>* r = run_fft<true, T, NC>(a, b, nl, ls, p, tw);
  cx<T>* zb = zbuf + (size_t)pair * N * g.ncol;
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int z = idx / nl, l = idx - z * nl, col = col0 + l;
    if (col < g.ncol) zb[(size_t)z * g.ncol + col] = r[l * ls + z];
  }
  if (kpart)
    kin_flush(kacc, f[is1], two ? f[is2] : 0.0,
              kpart + 2 * kin_slots<T>() * ((size_t)(s0 / 2 + pair) * gridDim.x + blockIdx.x));
}

// ---------------------------------------------------------------- Y stage (inverse)
template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) k_yinv(GeoDev g, FftPlan p, const cx<T>* __restrict__ zbuf, int nlrt,
                                                  cx<T>* __restrict__ ybuf, const cx<T>* __restrict__ twg) {
  GBCP_STAGE(g.n2, nlrt)
  const int sb = blockIdx.x * nl, z = blockIdx.y, pair = blockIdx.z;
  const cx<T>* zrow = zbuf + ((size_t)pair * g.n3 + z) * g.ncol;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int l = idx / N, y = idx - l * N, s = sb + l;
    cx<T> v = mk<T>(0, 0);
    if (s < g.nslot) {
      const int off = freq_of(y, N) - g.slot_gylo[s];
      if (off >= 0 && off < g.slot_ncol[s]) v = zrow[g.slot_col0[s] + off];
    }
    a[l * ls + y] = v;
  }
  __syncthreads();
  const cx<T>* r = run_fft<true, T, NC>(a, b, nl, ls, p, tw);
  cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)N * g.nslot;
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int y = idx / nl, l = idx - y * nl, s = sb + l;
    if (s < g.nslot) yb[(size_t)y * g.nslot + s] = r[l * ls + y];
  }
}

// Load nl x-lines (y0..y0+nl) of plane z from ybuf, scattering slots to x.
template <typename T>
__device__ __forceinline__ void load_xlines(const GeoDev& g, const cx<T>* __restrict__ yb, int y0, int nl, int N,
                                            int ls, cx<T>* a) {
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int l = idx / N, x = idx - l * N, y = y0 + l;
    const int s = freq_of(x, N) - g.gxlo;
    cx<T> v = mk<T>(0, 0);
    if (y < g.n2 && s >= 0 && s < g.nslot) v = yb[(size_t)y * g.nslot + s];
    a[l * ls + x] = v;
  }
}

// ---------------------------------------------------------------- X stage + density
template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) k_xinv_rho(GeoDev g, FftPlan p, const cx<T>* __restrict__ ybuf,
                                                      int npairs, int s0, int nstate, const double* __restrict__ f,
                                                      double inv_omega, double* __restrict__ rho, int nlrt,
                                                      const cx<T>* __restrict__ twg) {
  GBCP_STAGE(g.n1, nlrt)
  constexpr int NACC = kMaxAcc;
  const int y0 = blockIdx.x * nl, z = blockIdx.y;
  load_tw(tw, twg, N);
  // density of this launch's pairs: FP64 in the FP64 path; FP32 in the mixed path, added once
  // per launch to the FP64 density (the per-pair FP64 accumulation would occupy the
  // FP64 pipe for ~4 operations per grid point and pair)
  T acc[NACC];
#pragma unroll
  for (int k = 0; k < NACC; ++k) acc[k] = (T)0;
  const int tot = nl * N;
  for (int pair = 0; pair < npairs; ++pair) {
    const int is1 = s0 + 2 * pair, is2 = is1 + 1;
    const T f1 = (T)(f[is1] * inv_omega);
    const T f2 = (T)((is2 < nstate) ? f[is2] * inv_omega : 0.0);
    const cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)g.n2 * g.nslot;
    load_xlines(g, yb, y0, nl, N, ls, a);
    __syncthreads();
    const cx<T>* r = run_fft<true, T, NC>(a, b, nl, ls, p, tw);
#pragma unroll
    for (int k = 0; k < NACC; ++k) {
      const int e = threadIdx.x + k * kThreads;
      if (e < tot) {
        const int l = e / N, x = e - l * N;
        const cx<T> v = r[l * ls + x];
        const T vr = v.x, vi = v.y;
        acc[k] += f1 * vr * vr + f2 * vi * vi;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < NACC; ++k) {
    const int e = threadIdx.x + k * kThreads;
    if (e < tot) {
      const int l = e / N, x = e - l * N, y = y0 + l;
      if (y < g.n2) rho[x + (size_t)g.k1 * (y + (size_t)g.k2 * z)] += (double)acc[k];
    }
  }
}

// ---------------------------------------------------------------- X stage: inverse, x V, forward
template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) k_xvx(GeoDev g, FftPlan p, cx<T>* __restrict__ ybuf,
                                                 const double* __restrict__ vpot, int nlrt,
                                                 const cx<T>* __restrict__ twg) {
  GBCP_STAGE(g.n1, nlrt)
  const int y0 = blockIdx.x * nl, z = blockIdx.y, pair = blockIdx.z;
  cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)g.n2 * g.nslot;
  load_tw(tw, twg, N);
  load_xlines(g, yb, y0, nl, N, ls, a);
  __syncthreads();
  cx<T>* r = run_fft<true, T, NC>(a, b, nl, ls, p, tw);
  cx<T>* o = (r == a) ? b : a;
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int l = idx / N, x = idx - l * N, y = y0 + l;
    const T v = (y < g.n2) ? from_double<T>(vpot[x + (size_t)g.k1 * (y + (size_t)g.k2 * z)]) : (T)0;
    r[l * ls + x] = scl(r[l * ls + x], v);
  }
  __syncthreads();
  const cx<T>* q = run_fft<false, T, NC>(r, o, nl, ls, p, tw);
  for (int idx = threadIdx.x; idx < nl * g.nslot; idx += kThreads) {
    const int l = idx / g.nslot, s = idx - l * g.nslot, y = y0 + l;
    if (y < g.n2) yb[(size_t)y * g.nslot + s] = q[l * ls + idx_of(g.gxlo + s, N)];
  }
}

// ---------------------------------------------------------------- Y stage (forward)
template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) k_yfwd(GeoDev g, FftPlan p, const cx<T>* __restrict__ ybuf, int nlrt,
                                                  cx<T>* __restrict__ zbuf, const cx<T>* __restrict__ twg) {
  GBCP_STAGE(g.n2, nlrt)
  const int sb = blockIdx.x * nl, z = blockIdx.y, pair = blockIdx.z;
  const cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)N * g.nslot;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int y = idx / nl, l = idx - y * nl, s = sb + l;
    a[l * ls + y] = (s < g.nslot) ? yb[(size_t)y * g.nslot + s] : mk<T>(0, 0);
  }
  __syncthreads();
  const cx<T>* r = run_fft<false, T, NC>(a, b, nl, ls, p, tw);
  cx<T>* zrow = zbuf + ((size_t)pair * g.n3 + z) * g.ncol;
  const int send = min(sb + nl, g.nslot);
  const int cbeg = g.slot_col0[sb];
  const int cend = g.slot_col0[send - 1] + g.slot_ncol[send - 1];
  for (int c = cbeg + threadIdx.x; c < cend; c += kThreads) {
    const int l = g.col_slot[c] - sb;
    zrow[c] = r[l * ls + idx_of(g.col_gy[c], N)];
  }
}

// ---------------------------------------------------------------- Z stage (forward, to sphere entries)
template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) k_zfwd(GeoDev g, FftPlan p, const cx<T>* __restrict__ zbuf, int nlrt,
                                                  T scale, cx<T>* __restrict__ qbuf,
                                                  const cx<T>* __restrict__ twg) {
  GBCP_STAGE(g.n3, nlrt)
  const int col0 = blockIdx.x * nl, pair = blockIdx.y;
  const cx<T>* zb = zbuf + (size_t)pair * N * g.ncol;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += kThreads) {
    const int z = idx / nl, l = idx - z * nl, col = col0 + l;
    a[l * ls + z] = (col < g.ncol) ? zb[(size_t)z * g.ncol + col] : mk<T>(0, 0);
  }
  __syncthreads();
  const cx<T>* r = run_fft<false, T, NC>(a, b, nl, ls, p, tw);
  const int cend = min(col0 + nl, g.ncol);
  const int ebeg = g.col_start[col0], eend = g.col_start[cend];
  cx<T>* qb = qbuf + (size_t)pair * g.nent;
  for (int e = ebeg + threadIdx.x; e < eend; e += kThreads) {
    const int col = g.ent_col[e];
    const int gz = g.col_zlo[col] + (e - g.col_start[col]);
    qb[e] = scl(r[(col - col0) * ls + idx_of(gz, N)], scale);
  }
}

#undef GBCP_STAGE

// ---------------------------------------------------------------- decode + kinetic (vpsi_utils.mod.F90:661-671)
static __global__ void k_v_to_float(const double* __restrict__ v, float* __restrict__ vf, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    vf[i] = d2f_int(v[i]);
}

template <typename T> __device__ __forceinline__ double to_double(T x);
template <> __device__ __forceinline__ double to_double<double>(double x) { return x; }
template <> __device__ __forceinline__ double to_double<float>(float x) { return f2d_int(x); }

// c2 += -f/2 (tpiba2 hg c0 + (Re fp, Im fm)) for state 1 and -f/2 (... + (Im fp, -Re fm))
// for state 2; fp/fm in the transform precision, the update in FP64 (two FMAs per
// component; kin = tpiba2 hg precomputed).
// psi32 (FP32 kernels only): c0 and c2 stored as complex64, the update in FP32.
template <typename T>
__global__ void k_decode(GeoDev g, const cx<T>* __restrict__ qbuf, const cx<double>* __restrict__ c0, int ldc,
                         cx<double>* __restrict__ c2, int ldc2, const double* __restrict__ f, int s0, int nstate,
                         const double* __restrict__ kin_g, int psi32) {
  const int ig = blockIdx.x * blockDim.x + threadIdx.x;
  const int pair = blockIdx.y;
  if (ig >= g.ngw) return;
  const int is1 = s0 + 2 * pair, is2 = is1 + 1;
  const cx<T>* qb = qbuf + (size_t)pair * g.nent;
  const cx<T> qp = qb[g.pos_plus[ig]], qm = qb[g.pos_minus[ig]];
  if (psi32) {
    const float kin = d2f_int(kin_g[ig]);
    const cx<float>* a0 = reinterpret_cast<const cx<float>*>(c0);
    cx<float>* a2 = reinterpret_cast<cx<float>*>(c2);
    const float q1x = (float)(qp.x + qm.x), q1y = (float)(qp.y - qm.y);
    const float q2x = (float)(qp.y + qm.y), q2y = (float)(qm.x - qp.x);
    float fi = d2f_int(f[is1]) * 0.5f;
    if (fi == 0.0f) fi = 1.0f;
    {
      const cx<float> c = a0[(size_t)is1 * ldc + ig];
      cx<float>& o = a2[(size_t)is1 * ldc2 + ig];
      o.x = fmaf(-fi, fmaf(kin, c.x, q1x), o.x);
      o.y = fmaf(-fi, fmaf(kin, c.y, q1y), o.y);
    }
    if (is2 < nstate) {
      float fip1 = d2f_int(f[is2]) * 0.5f;
      if (fip1 == 0.0f) fip1 = 1.0f;
      const cx<float> c = a0[(size_t)is2 * ldc + ig];
      cx<float>& o = a2[(size_t)is2 * ldc2 + ig];
      o.x = fmaf(-fip1, fmaf(kin, c.x, q2x), o.x);
      o.y = fmaf(-fip1, fmaf(kin, c.y, q2y), o.y);
    }
    return;
  }
  const double kin = kin_g[ig];
  double fi = f[is1] * 0.5;
  if (fi == 0.0) fi = 1.0;
  {
    const cx<double> c = c0[(size_t)is1 * ldc + ig];
    cx<double>& o = c2[(size_t)is1 * ldc2 + ig];
    o.x = fma(-fi, fma(kin, c.x, to_double<T>(qp.x + qm.x)), o.x);
    o.y = fma(-fi, fma(kin, c.y, to_double<T>(qp.y - qm.y)), o.y);
  }
  if (is2 < nstate) {
    double fip1 = f[is2] * 0.5;
    if (fip1 == 0.0) fip1 = 1.0;
    const cx<double> c = c0[(size_t)is2 * ldc + ig];
    cx<double>& o = c2[(size_t)is2 * ldc2 + ig];
    o.x = fma(-fip1, fma(kin, c.x, to_double<T>(qp.y + qm.y)), o.x);
    o.y = fma(-fip1, fma(kin, c.y, to_double<T>(qm.x - qp.x)), o.y);
  }
}

}  // namespace band
}  // namespace gbcp

#include "band_fs.cuh"
#include "band_plane.cuh"

namespace gbcp {
namespace band {

// =========================================================================== host side

inline int lines_rt(int n) { return std::max(1, std::min(64, kElems / n)); }

template <typename T> inline size_t stage_smem(int n, int nl) {
  return sizeof(cx<T>) * ((size_t)n + 2 * (size_t)nl * line_stride(n));
}


template <typename T> inline const cx<T>* tw_of(Ctx& c, int axis);
template <> inline const cx<double>* tw_of<double>(Ctx& c, int axis) { return c.tw64[axis]; }
template <> inline const cx<float>* tw_of<float>(Ctx& c, int axis) { return c.tw32[axis]; }

template <typename T> inline const cx<T>* twA_of(Ctx& c, int axis);
template <> inline const cx<double>* twA_of<double>(Ctx& c, int axis) { return c.twA64[axis]; }
template <> inline const cx<float>* twA_of<float>(Ctx& c, int axis) { return c.twA32[axis]; }
template <typename T> inline const cx<T>* twB_of(Ctx& c, int axis);
template <> inline const cx<double>* twB_of<double>(Ctx& c, int axis) { return c.twB64[axis]; }
template <> inline const cx<float>* twB_of<float>(Ctx& c, int axis) { return c.twB32[axis]; }

// Dispatch `FN<T, NC>(args...)` on the run-time length n: NC > 0 runs the
// four-step kernels of band_fs.cuh, NC = 0 the run-time planned Stockham kernels.
#define GBCP_DISPATCH(FN, T, n, ...)                        \
  switch (n) {                                              \
    case 32: return FN<T, 32>(__VA_ARGS__);                 \
    case 36: return FN<T, 36>(__VA_ARGS__);                 \
    case 40: return FN<T, 40>(__VA_ARGS__);                 \
    case 48: return FN<T, 48>(__VA_ARGS__);                 \
    case 60: return FN<T, 60>(__VA_ARGS__);                 \
    case 64: return FN<T, 64>(__VA_ARGS__);                 \
    case 72: return FN<T, 72>(__VA_ARGS__);                 \
    case 80: return FN<T, 80>(__VA_ARGS__);                 \
    case 96: return FN<T, 96>(__VA_ARGS__);                 \
    case 120: return FN<T, 120>(__VA_ARGS__);               \
    case 144: return FN<T, 144>(__VA_ARGS__);               \
    case 240: return FN<T, 240>(__VA_ARGS__);               \
    default: return FN<T, 0>(__VA_ARGS__);                  \
  }

// no_ybuf: the plane kernels run the y and x stages, ybuf is not needed
template <typename T> int ensure_band_buffers(Ctx& c, int npairs, bool no_ybuf = false) {
  const GeoDev& g = c.geo;
  const size_t zb = sizeof(cx<T>) * (size_t)npairs * g.n3 * g.ncol;
  const size_t yb = no_ybuf ? 16 : sizeof(cx<T>) * (size_t)npairs * g.n3 * g.n2 * g.nslot;
  const size_t qb = sizeof(cx<T>) * (size_t)npairs * g.nent;
  if (!ensure(c, c.zbuf, zb) || !ensure(c, c.ybuf, yb) || !ensure(c, c.qbuf, qb)) {
    c.err = "band workspace allocation failed";
    return 6;
  }
  return 0;
}

template <typename T, int N> constexpr size_t fs_smem(int buffers, int tables) {
  return sizeof(cx<T>) * ((size_t)tables * N + (size_t)buffers * FS<T, N>::L * FS<T, N>::LS);
}
// x stage: the conflict-free (pitch, stride) layout, one exchange buffer
template <typename T, int N> constexpr size_t fs_smem_x(int tables) {
  return sizeof(cx<T>) * ((size_t)tables * N + (size_t)FS<T, N>::L * FS<T, N>::XS);
}

// Column blocks of the Z stage (the grid's x extent), for the size of the
// per-CTA partials of rhoofr's scalars.
// The four-step gather over column/mirror pairs (k_zinv_fs<.., true>): on by
// default where the column set spans at least 48 blocks (the 120^3 and larger
// cells), GBCP_OPT_ZMIRROR forces it on or off (a batch turns it off)
template <typename T, int NC> bool zmirror_n(const Ctx& c) {
  if constexpr (NC > 0) return c.zmirror > 0 || (c.zmirror < 0 && (c.geo.ncol + FS<T, NC>::L - 1) / FS<T, NC>::L >= 48);
  else return false;
}
template <typename T, int NC> int zinv_blocks_n(const Ctx& c) {
  // four-step: column blocks, or blocks of primary columns, each with its mirrors
  if constexpr (NC > 0)
    return ((zmirror_n<T, NC>(c) ? (c.geo.ncol + 1) / 2 : c.geo.ncol) + FS<T, NC>::L - 1) / FS<T, NC>::L;
  else return (c.geo.ncol + lines_rt(c.geo.n3) - 1) / lines_rt(c.geo.n3);
}

// kpart (may be null): per-CTA partials of E_kin and the norm (rhoofr only)
template <typename T, int NC>
int launch_zinv(Ctx& c, const cx<double>* c0, int ldc, int s0, int nstate, int np, int poff, const double* f,
                double* kpart) {
  const GeoDev& g = c.geo;
  cx<T>* zb = static_cast<cx<T>*>(c.zbuf.p) + (size_t)poff * g.n3 * g.ncol;  // pair poff of the launch batch
  ProfScope ps_(c, c.zk_skip ? "k_zinv_kept" : "k_zinv");  // kept: returns at once if the checksums agree
  if constexpr (NC > 0) {
    const dim3 grid(zinv_blocks_n<T, NC>(c), np);
    if (zmirror_n<T, NC>(c)) {
      constexpr size_t sm = fs_smem<T, NC>(2, 1);
      allow_smem(k_zinv_fs<T, NC, true>, sm);
      k_zinv_fs<T, NC, true><<<grid, kThreads, sm, c.stream>>>(g, c0, c.psi32, ldc, s0, nstate, zb, twA_of<T>(c, 2), f,
                                                               kpart, c.zk_skip);
    } else {
      constexpr size_t sm = fs_smem<T, NC>(1, 1);
      allow_smem(k_zinv_fs<T, NC, false>, sm);
      k_zinv_fs<T, NC, false><<<grid, kThreads, sm, c.stream>>>(g, c0, c.psi32, ldc, s0, nstate, zb, twA_of<T>(c, 2), f,
                                                                kpart, c.zk_skip);
    }
  } else {
    const int nl = lines_rt(g.n3);
    const size_t sm = stage_smem<T>(g.n3, nl);
    allow_smem(k_zinv<T, 0>, sm);
    k_zinv<T, 0><<<dim3(zinv_blocks_n<T, 0>(c), np), kThreads, sm, c.stream>>>(g, c.plan[2], c0, c.psi32, ldc, s0, nstate, nl,
                                                                               zb, tw_of<T>(c, 2), f, kpart, c.zk_skip);
  }
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

template <typename T, int NC> int launch_yinv(Ctx& c, int np, int poff) {
  const GeoDev& g = c.geo;
  // pairs poff .. poff+np-1 of the launch batch
  const cx<T>* zb = static_cast<const cx<T>*>(c.zbuf.p) + (size_t)poff * g.n3 * g.ncol;
  cx<T>* yb = static_cast<cx<T>*>(c.ybuf.p) + (size_t)poff * g.n3 * g.n2 * g.nslot;
  ProfScope ps_(c, "k_yinv");
  if constexpr (NC > 0) {
    // FP32: plus the staged sphere columns of one block of slots
    const size_t sm = fs_smem<T, NC>(1, 1) + (sizeof(T) == 4 ? sizeof(cx<T>) * (size_t)g.yblk_cols : 0);
    auto go = [&](auto kern) {
      allow_smem(kern, sm);
      kern<<<dim3((g.nslot + FS<T, NC>::L - 1) / FS<T, NC>::L, g.n3, np), kThreads, sm, c.stream>>>(g, zb, yb,
                                                                                                twA_of<T>(c, 1));
    };
    if constexpr (FS<T, NC>::N1 == 8) {
      if (g.prune_y) go(k_yinv_fs<T, NC, true>);
      else go(k_yinv_fs<T, NC, false>);
    } else {
      go(k_yinv_fs<T, NC, false>);
    }
  } else {
    const int nl = lines_rt(g.n2);
    const size_t sm = stage_smem<T>(g.n2, nl);
    allow_smem(k_yinv<T, 0>, sm);
    k_yinv<T, 0><<<dim3((g.nslot + nl - 1) / nl, g.n3, np), kThreads, sm, c.stream>>>(g, c.plan[1], zb, nl, yb,
                                                                                       tw_of<T>(c, 1));
  }
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

// Pair chunks of the density x-stage: the count that minimises the busiest
// SM's work, ceil(tiles * P / SMs) CTAs of ceil(np / P) + 1 pair-times each (the
// +1 is the copy of the first pair and the partial-tile combine).
constexpr int kXrhoMaxChunks = 8;
inline int xrho_chunks(const Ctx& c, int tiles, int np) {
  if (c.xr_chunks > 0) return std::max(1, std::min({c.xr_chunks, np, kXrhoMaxChunks}));
  const long long nsm = c.nsm > 0 ? c.nsm : 152;
  int best = 1;
  long long best_cost = -1;
  for (int p = 1; p <= std::min(np, kXrhoMaxChunks); ++p) {
    const long long per_sm = ((long long)tiles * p + nsm - 1) / nsm;
    const long long cost = per_sm * ((np + p - 1) / p + 1);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = p;
    }
  }
  return best;
}

template <typename T, int NC>
int launch_xinv_rho(Ctx& c, int np, int s0, int nstate, const double* f, double* rho, int poff, int z0, int z1) {
  const GeoDev& g = c.geo;
  if (z1 < 0) z1 = g.n3;
  // pairs poff .. poff+np-1 of the launch batch (states from s0)
  const cx<T>* yb = static_cast<const cx<T>*>(c.ybuf.p) + (size_t)poff * g.n3 * g.n2 * g.nslot;
  if constexpr (NC > 0) {
    using P = FS<T, NC>;
    const int tiles_y = (g.n2 + P::L - 1) / P::L, tiles = tiles_y * g.n3;
    const int pchunk = (np + xrho_chunks(c, tiles, np) - 1) / xrho_chunks(c, tiles, np);
    const int nchunk = (np + pchunk - 1) / pchunk;
    const size_t sm = fs_smem_x<T, NC>(1) + sizeof(cx<T>) * (size_t)xrho_bufs<T>() * P::L * g.nslot;
    if (sm > (size_t)227 * 1024) {
      c.err = "density x-stage: shared-memory tile too large for this sphere";
      return 7;
    }
    T* part = nullptr;
    unsigned* tickets = nullptr;
    if (nchunk > 1) {
      // sized for the largest chunk count once, so that later launches never reallocate
      if (!ensure(c, c.xr_part, sizeof(T) * (size_t)tiles * kXrhoMaxChunks * P::TB * P::N2)) return 6;
      const size_t tb = sizeof(unsigned) * (size_t)tiles;
      if (!c.xr_tk.p || c.xr_tk.cap < tb) {
        if (!ensure(c, c.xr_tk, tb)) return 6;
        GBCP_CUDA_TRY(c, cudaMemsetAsync(c.xr_tk.p, 0, c.xr_tk.cap, c.stream));
      }
      part = static_cast<T*>(c.xr_part.p);
      tickets = static_cast<unsigned*>(c.xr_tk.p);
    }
    ProfScope ps_(c, "k_xinv_rho");
    auto go = [&](auto kern) {
      allow_smem(kern, sm);
      kern<<<dim3(nchunk, tiles_y, z1 - z0), kThreads, sm, c.stream>>>(g, yb, np, s0, nstate, f, 1.0 / c.omega, rho,
                                                                         twA_of<T>(c, 0), pchunk, part, tickets, z0);
    };
    if constexpr (FS<T, NC>::N1 == 8) {
      if (g.prune_x) go(k_xrho_fs<T, NC, true>);
      else go(k_xrho_fs<T, NC, false>);
    } else {
      go(k_xrho_fs<T, NC, false>);
    }
  } else {
    if (z0 != 0 || z1 != g.n3) return 7;  // planes are split in the four-step kernel only
    int nl = lines_rt(g.n1);
    while (nl > 1 && nl * g.n1 > kMaxAcc * kThreads) --nl;
    if (nl * g.n1 > kMaxAcc * kThreads) {
      c.err = "mesh too large for the density tile";
      return 7;
    }
    const size_t sm = stage_smem<T>(g.n1, nl);
    allow_smem(k_xinv_rho<T, 0>, sm);
    ProfScope ps_(c, "k_xinv_rho");
    k_xinv_rho<T, 0><<<dim3((g.n2 + nl - 1) / nl, g.n3), kThreads, sm, c.stream>>>(
        g, c.plan[0], yb, np, s0, nstate, f, 1.0 / c.omega, rho, nl, tw_of<T>(c, 0));
  }
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

template <typename T, int NC> int launch_xvx(Ctx& c, int np, const double* vpot, const T* vpotT) {
  const GeoDev& g = c.geo;
  cx<T>* yb = static_cast<cx<T>*>(c.ybuf.p);
  ProfScope ps_(c, "k_xvx");
  if constexpr (NC > 0) {
    constexpr size_t sm = fs_smem_x<T, NC>(2);
    auto go = [&](auto kern) {
      allow_smem(kern, sm);
      kern<<<dim3((g.n2 + FS<T, NC>::L - 1) / FS<T, NC>::L, g.n3, np), kThreads, sm, c.stream>>>(
          g, yb, vpotT, twA_of<T>(c, 0), twB_of<T>(c, 0));
    };
    if constexpr (FS<T, NC>::N1 == 8) {
      if (g.prune_x) go(k_xvx_fs<T, NC, true>);
      else go(k_xvx_fs<T, NC, false>);
    } else {
      go(k_xvx_fs<T, NC, false>);
    }
  } else {
    const int nl = lines_rt(g.n1);
    const size_t sm = stage_smem<T>(g.n1, nl);
    allow_smem(k_xvx<T, 0>, sm);
    k_xvx<T, 0><<<dim3((g.n2 + nl - 1) / nl, g.n3, np), kThreads, sm, c.stream>>>(g, c.plan[0], yb, vpot, nl,
                                                                                   tw_of<T>(c, 0));
  }
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

template <typename T, int NC> int launch_yfwd(Ctx& c, int np) {
  const GeoDev& g = c.geo;
  const cx<T>* yb = static_cast<const cx<T>*>(c.ybuf.p);
  cx<T>* zb = static_cast<cx<T>*>(c.zbuf.p);
  ProfScope ps_(c, "k_yfwd");
  if constexpr (NC > 0) {
    constexpr size_t sm = fs_smem<T, NC>(1, 1);
    allow_smem(k_yfwd_fs<T, NC>, sm);
    k_yfwd_fs<T, NC><<<dim3((g.nslot + FS<T, NC>::L - 1) / FS<T, NC>::L, g.n3, np), kThreads, sm, c.stream>>>(
        g, yb, zb, twA_of<T>(c, 1));
  } else {
    const int nl = lines_rt(g.n2);
    const size_t sm = stage_smem<T>(g.n2, nl);
    allow_smem(k_yfwd<T, 0>, sm);
    k_yfwd<T, 0><<<dim3((g.nslot + nl - 1) / nl, g.n3, np), kThreads, sm, c.stream>>>(g, c.plan[1], yb, nl, zb,
                                                                                       tw_of<T>(c, 1));
  }
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

template <typename T, int NC> int launch_zfwd(Ctx& c, int np, int poff) {
  const GeoDev& g = c.geo;
  const cx<T>* zb = static_cast<const cx<T>*>(c.zbuf.p) + (size_t)poff * g.n3 * g.ncol;  // pairs poff ..
  cx<T>* qb = static_cast<cx<T>*>(c.qbuf.p);
  const T scale = (T)(1.0 / ((double)g.n1 * g.n2 * g.n3));
  ProfScope ps_(c, "k_zfwd");
  if constexpr (NC > 0) {
    constexpr size_t sm = fs_smem<T, NC>(1, 1);
    allow_smem(k_zfwd_fs<T, NC>, sm);
    k_zfwd_fs<T, NC><<<dim3((g.ncol + FS<T, NC>::L - 1) / FS<T, NC>::L, np), kThreads, sm, c.stream>>>(
        g, zb, scale, qb, twA_of<T>(c, 2));
  } else {
    const int nl = lines_rt(g.n3);
    const size_t sm = stage_smem<T>(g.n3, nl);
    allow_smem(k_zfwd<T, 0>, sm);
    k_zfwd<T, 0><<<dim3((g.ncol + nl - 1) / nl, np), kThreads, sm, c.stream>>>(g, c.plan[2], zb, nl, scale, qb,
                                                                               tw_of<T>(c, 2));
  }
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

// ---- plane-fused Y and X stages (FP32, band_plane.cuh) ----
constexpr size_t kSmemMax = 227 * 1024;
// largest mesh length with plane kernels: a 240-point plane of a sphere that fills
// it does not fit in shared memory (and its density tile would spill registers)
constexpr int kPlaneMaxN = 144;
// whether the plane kernels run this context's band loop: FP32, four-step plan,
// equal x and y lengths, the plane fits in shared memory (GBCP_OPT_PLANE on)
template <typename T, int NC> bool plane_fits_n(const Ctx& c) {
  if constexpr (sizeof(T) == 4 && NC > 0 && NC <= kPlaneMaxN) {
    return c.nr[0] == c.nr[1] && PlaneLayout<NC>::bytes(3, c.geo.nslot) <= kSmemMax &&
           PlaneLayout<NC>::bytes(2, c.geo.nslot, 2) <= kSmemMax;
  } else {
    return false;
  }
}
template <typename T> bool plane_fits(const Ctx& c) {
  if (c.fft_engine == 2 || c.nr[0] != c.nr[1]) return false;
  GBCP_DISPATCH(plane_fits_n, T, c.nr[0], c)
}

template <typename T, int NC> int launch_plane_vx(Ctx& c, int np, int poff, const T* vpotT) {
  if constexpr (sizeof(T) == 4 && NC > 0 && NC <= kPlaneMaxN) {
    const GeoDev& g = c.geo;
    cx<float>* zb = static_cast<cx<float>*>(c.zbuf.p) + (size_t)poff * g.n3 * g.ncol;
    const size_t sm = PlaneLayout<NC>::bytes(3, g.nslot);
    ProfScope ps_(c, "k_plane_vx");
    auto go = [&](auto kern) {
      allow_smem(kern, sm);
      kern<<<dim3(g.n3, np), kThreads, sm, c.stream>>>(g, zb, reinterpret_cast<const float*>(vpotT),
                                                      twA_of<float>(c, 1), twA_of<float>(c, 0), twB_of<float>(c, 0));
    };
    // x and y have the same length here; the radix-8 plans prune each axis whose
    // sphere frequencies allow it
    if constexpr (FS<float, NC>::N1 == 8) {
      if (g.prune_x && g.prune_y) go(k_plane_vx_fs<NC, true, true>);
      else if (g.prune_x) go(k_plane_vx_fs<NC, true, false>);
      else if (g.prune_y) go(k_plane_vx_fs<NC, false, true>);
      else go(k_plane_vx_fs<NC, false, false>);
    } else {
      go(k_plane_vx_fs<NC, false, false>);
    }
    GBCP_LAUNCH_CHECK(c);
    return 0;
  } else {
    c.err = "plane kernels: FP32 four-step meshes only";
    return 7;
  }
}

// CTAs of the plane density kernel resident on one SM (measured once per mesh)
template <int NC> int plane_rho_ctas_per_sm(size_t sm) {
  static int n = 0;
  if (!n) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_plane_rho_fs<NC>, kPlaneRhoThreads, sm) != cudaSuccess ||
        n < 1) {
      cudaGetLastError();
      n = 1;
    }
  }
  return n;
}

template <typename T, int NC>
int launch_plane_rho(Ctx& c, int np, int s0, int nstate, const double* f, double* rho, int poff) {
  if constexpr (sizeof(T) == 4 && NC > 0 && NC <= kPlaneMaxN) {
    const GeoDev& g = c.geo;
    using PL = PlaneLayout<NC>;
    const cx<float>* zb = static_cast<const cx<float>*>(c.zbuf.p) + (size_t)poff * g.n3 * g.ncol;
    const size_t sm = PL::bytes(2, g.nslot, 2);
    allow_smem(k_plane_rho_fs<NC>, sm);
    // pair chunks: the count that minimises the busiest SM's work, as for the x-stage
    const int per_sm = plane_rho_ctas_per_sm<NC>(sm);
    const long long slots = (long long)(c.nsm > 0 ? c.nsm : 152) * per_sm;
    int nchunk = 1;
    long long best = -1;
    for (int q = 1; q <= std::min(np, kXrhoMaxChunks); ++q) {
      const long long cost = (((long long)g.n3 * q + slots - 1) / slots) * ((np + q - 1) / q + 1);
      if (best < 0 || cost < best) {
        best = cost;
        nchunk = q;
      }
    }
    if (c.xr_chunks > 0) nchunk = std::max(1, std::min({c.xr_chunks, np, kXrhoMaxChunks}));
    const int pchunk = (np + nchunk - 1) / nchunk;
    nchunk = (np + pchunk - 1) / pchunk;
    float* part = nullptr;
    unsigned* tickets = nullptr;
    if (nchunk > 1) {
      constexpr size_t tile = (size_t)2 * ((PL::NB + 1) / 2) * FS<float, NC>::TB * FS<float, NC>::N2;
      if (!ensure(c, c.xr_part, sizeof(float) * tile * (size_t)g.n3 * kXrhoMaxChunks)) return 6;
      const size_t tb = sizeof(unsigned) * (size_t)std::max(g.n3, 1);
      if (!c.xr_tk.p || c.xr_tk.cap < tb) {
        if (!ensure(c, c.xr_tk, tb)) return 6;
        GBCP_CUDA_TRY(c, cudaMemsetAsync(c.xr_tk.p, 0, c.xr_tk.cap, c.stream));
      }
      part = static_cast<float*>(c.xr_part.p);
      tickets = static_cast<unsigned*>(c.xr_tk.p);
    }
    ProfScope ps_(c, "k_plane_rho");
    k_plane_rho_fs<NC><<<dim3(nchunk, g.n3), kPlaneRhoThreads, sm, c.stream>>>(g, zb, np, s0, nstate, f, 1.0 / c.omega,
                                                                               rho,
                                                                       twA_of<float>(c, 1), twA_of<float>(c, 0),
                                                                       pchunk, part, tickets);
    GBCP_LAUNCH_CHECK(c);
    return 0;
  } else {
    c.err = "plane kernels: FP32 four-step meshes only";
    return 7;
  }
}

template <typename T>
int launch_decode(Ctx& c, int np, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f, int s0,
                  int nstate, int poff = 0) {
  const GeoDev& g = c.geo;
  ProfScope ps_(c, "k_decode");
  const cx<T>* qb = static_cast<const cx<T>*>(c.qbuf.p) + (size_t)poff * g.nent;  // pair poff of the launch batch
  k_decode<T><<<dim3((g.ngw + 255) / 256, np), 256, 0, c.stream>>>(g, qb, c0, ldc, c2, ldc2, f, s0, nstate, c.kin,
                                                                   c.psi32);
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

template <typename T>
int zinv(Ctx& c, const cx<double>* c0, int ldc, int s0, int nstate, int np, int poff = 0, const double* f = nullptr,
         double* kpart = nullptr) {
  GBCP_DISPATCH(launch_zinv, T, band_len(c, c.nr[2]), c, c0, ldc, s0, nstate, np, poff, f, kpart)
}
template <typename T> int zinv_blocks(const Ctx& c) { GBCP_DISPATCH(zinv_blocks_n, T, band_len(c, c.nr[2]), c) }
// E_kin / norm partial slots per pair
template <typename T> int kin_blocks(const Ctx& c) { return zinv_blocks<T>(c) * kin_slots<T>(); }
template <typename T> int yinv(Ctx& c, int np, int poff = 0) {
  GBCP_DISPATCH(launch_yinv, T, band_len(c, c.nr[1]), c, np, poff)
}
// planes z0 .. z1-1 (z1 < 0: to the last plane; other than all planes only in the four-step kernels)
template <typename T>
int xinv_rho(Ctx& c, int np, int s0, int nstate, const double* f, double* rho, int poff = 0, int z0 = 0, int z1 = -1) {
  GBCP_DISPATCH(launch_xinv_rho, T, band_len(c, c.nr[0]), c, np, s0, nstate, f, rho, poff, z0, z1)
}
// the density x-stage's z planes can be launched in slabs (four-step kernels)
template <typename T> bool xrho_slabs(const Ctx& c) {
  const int n = band_len(c, c.nr[0]);
  return c.fft_engine != 2 && (n == 32 || n == 36 || n == 40 || n == 48 || n == 60 || n == 64 || n == 72 || n == 80 ||
                               n == 96 || n == 120 || n == 144 || n == 240);
}
template <typename T> int xvx(Ctx& c, int np, const double* vpot, const T* vpotT) {
  GBCP_DISPATCH(launch_xvx, T, band_len(c, c.nr[0]), c, np, vpot, vpotT)
}
template <typename T> int yfwd(Ctx& c, int np) { GBCP_DISPATCH(launch_yfwd, T, band_len(c, c.nr[1]), c, np) }
template <typename T> int plane_vx(Ctx& c, int np, const T* vpotT, int poff = 0) {
  GBCP_DISPATCH(launch_plane_vx, T, c.nr[0], c, np, poff, vpotT)
}
template <typename T>
int plane_rho(Ctx& c, int np, int s0, int nstate, const double* f, double* rho, int poff = 0) {
  GBCP_DISPATCH(launch_plane_rho, T, c.nr[0], c, np, s0, nstate, f, rho, poff)
}
template <typename T> int zfwd(Ctx& c, int np, int poff = 0) {
  GBCP_DISPATCH(launch_zfwd, T, band_len(c, c.nr[2]), c, np, poff)
}

// Z stage of pairs [p0, p0 + np): one launch, or, with host staging, one launch per
// staging chunk after that chunk's columns have arrived
template <typename T> int zinv_staged(Ctx& c, const cx<double>* c0, int ldc, int p0, int nstate, int np) {
  if (!c.batch_ready) return zinv<T>(c, c0, ldc, 2 * p0, nstate, np);
  const std::vector<int>& b = c.stage_bounds;
  for (size_t q = 0; q + 1 < b.size(); ++q) {
    const int q0 = std::max(b[q], p0), q1 = std::min(b[q + 1], p0 + np);
    if (q1 <= q0) continue;
    GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.batch_ready[q], 0));
    const int rc = zinv<T>(c, c0, ldc, 2 * q0, nstate, q1 - q0, q0 - p0);
    if (rc) return rc;
  }
  return 0;
}

// pairs of the launch batch starting at pair p0: c.batch, or with host staging the staging chunk
inline int launch_pairs(const Ctx& c, int p0, int npairs_total) {
  if (c.batch_ready) {
    for (size_t q = 0; q + 1 < c.stage_bounds.size(); ++q)
      if (c.stage_bounds[q] == p0) return c.stage_bounds[q + 1] - p0;
  }
  return std::min(c.batch, npairs_total - p0);
}

// kpart (may be null): E_kin / norm partials, 2 * npairs * zinv_blocks<T>(c) doubles
template <typename T>
int rhoofr_t(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho, double* kpart) {
  const int npairs_total = (nstate + 1) / 2;
  const bool plane = (c.plane & 2) && plane_fits<T>(c);  // y and x stages fused per z-plane, no ybuf
  int rc = ensure_band_buffers<T>(c, std::min(c.batch, npairs_total), plane);
  if (rc) return rc;
  // the density x-stage of the pairs [g0, g1) of the launch batch starting at p0
  auto density = [&](int g0, int g1, int p0b) -> int {
    return plane ? plane_rho<T>(c, g1 - g0, 2 * g0, nstate, f, rho, g0 - p0b)
                 : xinv_rho<T>(c, g1 - g0, 2 * g0, nstate, f, rho, g0 - p0b);
  };
  // host staging, the call's last x-stage launch: in slabs of z planes, each followed
  // by its event, so that rho goes back slab by slab while the later ones compute
  // (band_rhoofr records the events at its end if no such launch ran)
  auto density_final = [&](int g0, int g1, int p0b) -> int {
    const int ns = c.rho_ev ? c.rho_slabs : 0;
    int r = 0;
    if (ns == 2 && !plane && xrho_slabs<T>(c) && c.rho_zsplit > 0 && c.rho_zsplit < c.geo.n3) {
      for (int i = 0; i < ns && !r; ++i) {
        r = xinv_rho<T>(c, g1 - g0, 2 * g0, nstate, f, rho, g0 - p0b, i ? c.rho_zsplit : 0,
                        i ? c.geo.n3 : c.rho_zsplit);
        if (!r) GBCP_CUDA_TRY(c, cudaEventRecord(c.rho_ev[i], c.stream));
      }
    } else {
      r = density(g0, g1, p0b);
      for (int i = 0; i < ns && !r; ++i) GBCP_CUDA_TRY(c, cudaEventRecord(c.rho_ev[i], c.stream));
    }
    c.rho_ev_set = !r;
    return r;
  };
  for (int p0 = 0, np = 0; p0 < npairs_total; p0 += np) {
    np = std::min(c.batch, npairs_total - p0);
    const int s0 = 2 * p0;
    if (!c.batch_ready) {
      if ((rc = zinv<T>(c, c0, ldc, s0, nstate, np, 0, f, kpart))) return rc;
      if (!plane && (rc = yinv<T>(c, np))) return rc;
      if ((rc = density(p0, p0 + np, p0))) return rc;
    } else {
      // host staging: Z and Y stages of each staging chunk as its states land; the
      // density x-stage (which gains most from many pairs per launch) in two groups
      // of chunks, the first overlapping the later uploads, the second the tail
      const std::vector<int>& b = c.stage_bounds;
      const size_t nq = b.size() - 1;
      const size_t ng = std::max<size_t>(1, std::min<size_t>(nq, c.stage_groups > 0 ? c.stage_groups : 2));
      const bool last_batch = p0 + np >= npairs_total;
      int g0 = p0;  // first pair of the x-stage group not yet launched
      for (size_t q = 0; q < nq; ++q) {
        const int q0 = std::max(b[q], p0), q1 = std::min(b[q + 1], p0 + np);
        if (q1 > q0) {
          GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.batch_ready[q], 0));
          if ((rc = zinv<T>(c, c0, ldc, 2 * q0, nstate, q1 - q0, q0 - p0, f, kpart))) return rc;
          if (!plane && (rc = yinv<T>(c, q1 - q0, q0 - p0))) return rc;
        }
        const int gend = std::min(b[q + 1], p0 + np);
        // group ends after chunks ceil(nq g / ng), g = 1 .. ng
        const bool group_end = ((q + 1) * ng) / nq != (q * ng) / nq || q + 1 == nq;
        if (group_end && gend > g0) {
          const bool fin = last_batch && gend == p0 + np;
          if ((rc = fin ? density_final(g0, gend, p0) : density(g0, gend, p0))) return rc;
          g0 = gend;
        }
      }
      if (g0 < p0 + np && (rc = last_batch ? density_final(g0, p0 + np, p0) : density(g0, p0 + np, p0))) return rc;
    }
  }
  return 0;
}

template <typename T>
int vpsi_t(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f, const double* vpot,
           int nstate) {
  const int npairs_total = (nstate + 1) / 2;
  const bool plane = (c.plane & 1) && plane_fits<T>(c);  // y and x stages fused per z-plane, no ybuf
  int rc = ensure_band_buffers<T>(c, std::min(c.batch, npairs_total), plane);
  if (rc) return rc;
  // V(r) in the transform precision, converted once per call before the first
  // x-stage (with host staging V(r) arrives behind the first chunk of states)
  const T* vT = reinterpret_cast<const T*>(vpot);
  auto prepare_v = [&]() -> int {
    if (c.vpot_ready) GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.vpot_ready, 0));
    if constexpr (sizeof(T) == 4) {
      const size_t nnr = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
      if (!ensure(c, c.st_vf, sizeof(float) * nnr)) return 6;
      ProfScope ps_(c, "k_v_to_float");
      k_v_to_float<<<std::max<size_t>(1, std::min<size_t>(2048, (nnr + 255) / 256)), 256, 0, c.stream>>>(
          vpot, static_cast<float*>(c.st_vf.p), nnr);
      GBCP_LAUNCH_CHECK(c);
      vT = reinterpret_cast<const T*>(c.st_vf.p);
    }
    return 0;
  };
  // host staging with the Z stage kept from rhoofr (all pairs in zbuf at their own
  // positions): no Z stage, each staging chunk's stages on its pairs of zbuf
  const bool hkeep = c.zk_host && plane;
  for (int p0 = 0, np = 0; p0 < npairs_total; p0 += np) {
    np = launch_pairs(c, p0, npairs_total);
    const int s0 = 2 * p0;
    if (!hkeep && (rc = zinv_staged<T>(c, c0, ldc, p0, nstate, np))) return rc;
    if (plane) {
      if (p0 == 0 && (rc = prepare_v())) return rc;
      if ((rc = plane_vx<T>(c, np, vT, hkeep ? p0 : 0))) return rc;
    } else {
      if ((rc = yinv<T>(c, np))) return rc;
      if (p0 == 0 && (rc = prepare_v())) return rc;
      if ((rc = xvx<T>(c, np, vpot, vT))) return rc;
      if ((rc = yfwd<T>(c, np))) return rc;
    }
    if ((rc = zfwd<T>(c, np, hkeep ? p0 : 0))) return rc;
    if (!c.batch_ready) {
      if ((rc = launch_decode<T>(c, np, c0, ldc, c2, ldc2, f, s0, nstate))) return rc;
    } else {
      // host staging: decode per staging chunk, each followed by its download
      const std::vector<int>& b = c.stage_bounds;
      for (size_t q = 0; q + 1 < b.size(); ++q) {
        const int q0 = std::max(b[q], p0), q1 = std::min(b[q + 1], p0 + np);
        if (q1 <= q0) continue;
        if (c.batch_c2_ready) GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.batch_c2_ready[q], 0));
        if ((rc = launch_decode<T>(c, q1 - q0, c0, ldc, c2, ldc2, f, 2 * q0, nstate, q0 - p0))) return rc;
        if (c.batch_done && (rc = c.batch_done((int)q))) return rc;
      }
    }
  }
  return 0;
}

}  // namespace band
}  // namespace gbcp
