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
#include <algorithm>
#include <cmath>

#include "ctx.h"

namespace gbcp {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxAcc = 16;  // density accumulators per thread in the X stage

__host__ __device__ inline int line_stride(int n) { return (n % 2 == 0) ? n + 1 : n; }
__device__ __forceinline__ int freq_of(int i, int n) { return (i < (n + 1) / 2) ? i : i - n; }
__device__ __forceinline__ int idx_of(int g, int n) { return g < 0 ? g + n : g; }

template <typename T> __device__ __forceinline__ cx<T> from_d(cx<double> v) { return mk<T>((T)v.x, (T)v.y); }

template <typename T>
__device__ __forceinline__ void load_tw(cx<T>* tw, const cx<T>* __restrict__ twg, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = twg[i];
}

// ---------------------------------------------------------------- Z stage (inverse, gather)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_zinv(GeoDev g, FftPlan p, const cx<double>* __restrict__ c0, int ldc,
                                                  int s0, int nstate, int nl, cx<T>* __restrict__ zbuf,
                                                  const cx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.n3, ls = line_stride(N);
  cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* a = tw + N;
  cx<T>* b = a + nl * ls;
  const int pair = blockIdx.y;
  const int col0 = blockIdx.x * nl;
  const int is1 = s0 + 2 * pair, is2 = is1 + 1;
  const bool two = is2 < nstate;
  const cx<double>* c1 = c0 + (size_t)is1 * ldc;
  const cx<double>* c2 = c0 + (size_t)(two ? is2 : is1) * ldc;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int l = idx / N, z = idx - l * N, col = col0 + l;
    cx<T> v = mk<T>(0, 0);
    if (col < g.ncol) {
      const int st = g.col_start[col], len = g.col_start[col + 1] - st;
      const int off = freq_of(z, N) - g.col_zlo[col];
      if (off >= 0 && off < len) {
        const int e = g.col_ent[st + off];
        if (e != 0) {
          const int ig = (e > 0 ? e : -e) - 1;
          const cx<double> u = c1[ig];
          const cx<double> w = two ? c2[ig] : mk<double>(0.0, 0.0);
          // +G: c1 + i c2 ; -G: conj(c1) + i conj(c2)
          v = (e > 0) ? mk<T>((T)(u.x - w.y), (T)(u.y + w.x)) : mk<T>((T)(u.x + w.y), (T)(w.x - u.y));
        }
      }
    }
    a[l * ls + z] = v;
  }
  __syncthreads();
  const cx<T>* r = fft_lines<true>(a, b, nl, ls, p, tw);
  cx<T>* zb = zbuf + (size_t)pair * N * g.ncol;
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int z = idx / nl, l = idx - z * nl, col = col0 + l;
    if (col < g.ncol) zb[(size_t)z * g.ncol + col] = r[l * ls + z];
  }
}

// ---------------------------------------------------------------- Y stage (inverse)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_yinv(GeoDev g, FftPlan p, const cx<T>* __restrict__ zbuf, int nl,
                                                  cx<T>* __restrict__ ybuf, const cx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.n2, ls = line_stride(N);
  cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* a = tw + N;
  cx<T>* b = a + nl * ls;
  const int sb = blockIdx.x * nl, z = blockIdx.y, pair = blockIdx.z;
  const cx<T>* zrow = zbuf + ((size_t)pair * g.n3 + z) * g.ncol;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int l = idx / N, y = idx - l * N, s = sb + l;
    cx<T> v = mk<T>(0, 0);
    if (s < g.nslot) {
      const int off = freq_of(y, N) - g.slot_gylo[s];
      if (off >= 0 && off < g.slot_ncol[s]) v = zrow[g.slot_col0[s] + off];
    }
    a[l * ls + y] = v;
  }
  __syncthreads();
  const cx<T>* r = fft_lines<true>(a, b, nl, ls, p, tw);
  cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)N * g.nslot;
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int y = idx / nl, l = idx - y * nl, s = sb + l;
    if (s < g.nslot) yb[(size_t)y * g.nslot + s] = r[l * ls + y];
  }
}

// Load nl x-lines (y0..y0+nl) of plane z from ybuf, scattering slots to x.
template <typename T>
__device__ __forceinline__ void load_xlines(const GeoDev& g, const cx<T>* __restrict__ yb, int y0, int nl, int ls,
                                            cx<T>* a) {
  const int N = g.n1;
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int l = idx / N, x = idx - l * N, y = y0 + l;
    const int s = freq_of(x, N) - g.gxlo;
    cx<T> v = mk<T>(0, 0);
    if (y < g.n2 && s >= 0 && s < g.nslot) v = yb[(size_t)y * g.nslot + s];
    a[l * ls + x] = v;
  }
}

// ---------------------------------------------------------------- X stage + density
template <typename T>
__global__ void __launch_bounds__(kThreads) k_xinv_rho(GeoDev g, FftPlan p, const cx<T>* __restrict__ ybuf,
                                                      int npairs, int s0, int nstate, const double* __restrict__ f,
                                                      double inv_omega, double* __restrict__ rho, int nl,
                                                      const cx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.n1, ls = line_stride(N);
  cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* a = tw + N;
  cx<T>* b = a + nl * ls;
  const int y0 = blockIdx.x * nl, z = blockIdx.y;
  load_tw(tw, twg, N);
  double acc[kMaxAcc];
#pragma unroll
  for (int k = 0; k < kMaxAcc; ++k) acc[k] = 0.0;
  const int tot = nl * N;
  for (int pair = 0; pair < npairs; ++pair) {
    const int is1 = s0 + 2 * pair, is2 = is1 + 1;
    const double f1 = f[is1] * inv_omega;
    const double f2 = (is2 < nstate) ? f[is2] * inv_omega : 0.0;
    const cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)g.n2 * g.nslot;
    load_xlines(g, yb, y0, nl, ls, a);
    __syncthreads();
    const cx<T>* r = fft_lines<true>(a, b, nl, ls, p, tw);
#pragma unroll
    for (int k = 0; k < kMaxAcc; ++k) {
      const int e = threadIdx.x + k * kThreads;
      if (e < tot) {
        const int l = e / N, x = e - l * N;
        const cx<T> v = r[l * ls + x];
        const double vr = (double)v.x, vi = (double)v.y;
        acc[k] += f1 * vr * vr + f2 * vi * vi;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < kMaxAcc; ++k) {
    const int e = threadIdx.x + k * kThreads;
    if (e < tot) {
      const int l = e / N, x = e - l * N, y = y0 + l;
      if (y < g.n2) rho[x + (size_t)g.k1 * (y + (size_t)g.k2 * z)] += acc[k];
    }
  }
}

// ---------------------------------------------------------------- X stage: inverse, x V, forward
template <typename T>
__global__ void __launch_bounds__(kThreads) k_xvx(GeoDev g, FftPlan p, cx<T>* __restrict__ ybuf,
                                                 const double* __restrict__ vpot, int nl,
                                                 const cx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.n1, ls = line_stride(N);
  cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* a = tw + N;
  cx<T>* b = a + nl * ls;
  const int y0 = blockIdx.x * nl, z = blockIdx.y, pair = blockIdx.z;
  cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)g.n2 * g.nslot;
  load_tw(tw, twg, N);
  load_xlines(g, yb, y0, nl, ls, a);
  __syncthreads();
  cx<T>* r = fft_lines<true>(a, b, nl, ls, p, tw);
  cx<T>* o = (r == a) ? b : a;
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int l = idx / N, x = idx - l * N, y = y0 + l;
    const T v = (y < g.n2) ? (T)vpot[x + (size_t)g.k1 * (y + (size_t)g.k2 * z)] : (T)0;
    r[l * ls + x] = scl(r[l * ls + x], v);
  }
  __syncthreads();
  const cx<T>* q = fft_lines<false>(r, o, nl, ls, p, tw);
  for (int idx = threadIdx.x; idx < nl * g.nslot; idx += blockDim.x) {
    const int l = idx / g.nslot, s = idx - l * g.nslot, y = y0 + l;
    if (y < g.n2) yb[(size_t)y * g.nslot + s] = q[l * ls + idx_of(g.gxlo + s, N)];
  }
}

// ---------------------------------------------------------------- Y stage (forward)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_yfwd(GeoDev g, FftPlan p, const cx<T>* __restrict__ ybuf, int nl,
                                                  cx<T>* __restrict__ zbuf, const cx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.n2, ls = line_stride(N);
  cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* a = tw + N;
  cx<T>* b = a + nl * ls;
  const int sb = blockIdx.x * nl, z = blockIdx.y, pair = blockIdx.z;
  const cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)N * g.nslot;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int y = idx / nl, l = idx - y * nl, s = sb + l;
    a[l * ls + y] = (s < g.nslot) ? yb[(size_t)y * g.nslot + s] : mk<T>(0, 0);
  }
  __syncthreads();
  const cx<T>* r = fft_lines<false>(a, b, nl, ls, p, tw);
  cx<T>* zrow = zbuf + ((size_t)pair * g.n3 + z) * g.ncol;
  const int send = min(sb + nl, g.nslot);
  const int cbeg = g.slot_col0[sb];
  const int cend = g.slot_col0[send - 1] + g.slot_ncol[send - 1];
  for (int c = cbeg + threadIdx.x; c < cend; c += blockDim.x) {
    const int l = g.col_slot[c] - sb;
    zrow[c] = r[l * ls + idx_of(g.col_gy[c], N)];
  }
}

// ---------------------------------------------------------------- Z stage (forward, to sphere entries)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_zfwd(GeoDev g, FftPlan p, const cx<T>* __restrict__ zbuf, int nl,
                                                  T scale, cx<T>* __restrict__ qbuf,
                                                  const cx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = g.n3, ls = line_stride(N);
  cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* a = tw + N;
  cx<T>* b = a + nl * ls;
  const int col0 = blockIdx.x * nl, pair = blockIdx.y;
  const cx<T>* zb = zbuf + (size_t)pair * N * g.ncol;
  load_tw(tw, twg, N);
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    const int z = idx / nl, l = idx - z * nl, col = col0 + l;
    a[l * ls + z] = (col < g.ncol) ? zb[(size_t)z * g.ncol + col] : mk<T>(0, 0);
  }
  __syncthreads();
  const cx<T>* r = fft_lines<false>(a, b, nl, ls, p, tw);
  const int cend = min(col0 + nl, g.ncol);
  const int ebeg = g.col_start[col0], eend = g.col_start[cend];
  cx<T>* qb = qbuf + (size_t)pair * g.nent;
  for (int e = ebeg + threadIdx.x; e < eend; e += blockDim.x) {
    const int col = g.ent_col[e];
    const int gz = g.col_zlo[col] + (e - g.col_start[col]);
    qb[e] = scl(r[(col - col0) * ls + idx_of(gz, N)], scale);
  }
}

// ---------------------------------------------------------------- decode + kinetic (vpsi_utils.mod.F90:661-671)
template <typename T>
__global__ void k_decode(GeoDev g, const cx<T>* __restrict__ qbuf, const cx<double>* __restrict__ c0, int ldc,
                         cx<double>* __restrict__ c2, int ldc2, const double* __restrict__ f, int s0, int nstate,
                         double tpiba2) {
  const int ig = blockIdx.x * blockDim.x + threadIdx.x;
  const int pair = blockIdx.y;
  if (ig >= g.ngw) return;
  const int is1 = s0 + 2 * pair, is2 = is1 + 1;
  const cx<T>* qb = qbuf + (size_t)pair * g.nent;
  const cx<T> qp = qb[g.pos_plus[ig]], qm = qb[g.pos_minus[ig]];
  const double fpx = (double)qp.x + (double)qm.x, fpy = (double)qp.y + (double)qm.y;
  const double fmx = (double)qp.x - (double)qm.x, fmy = (double)qp.y - (double)qm.y;
  const double kin = tpiba2 * g.hg[ig];
  double fi = f[is1] * 0.5;
  if (fi == 0.0) fi = 1.0;
  {
    const cx<double> c = c0[(size_t)is1 * ldc + ig];
    cx<double>& o = c2[(size_t)is1 * ldc2 + ig];
    o.x += -fi * (kin * c.x + fpx);
    o.y += -fi * (kin * c.y + fmy);
  }
  if (is2 < nstate) {
    double fip1 = f[is2] * 0.5;
    if (fip1 == 0.0) fip1 = 1.0;
    const cx<double> c = c0[(size_t)is2 * ldc + ig];
    cx<double>& o = c2[(size_t)is2 * ldc2 + ig];
    o.x += -fip1 * (kin * c.x + fpy);
    o.y += -fip1 * (kin * c.y - fmx);
  }
}

// ---------------------------------------------------------------- dense axis FFT (invfftn/fwfftn)
// grid (kr1, kr2, nr3) complex, transform along `axis` in place.
template <bool INV>
__global__ void __launch_bounds__(kThreads) k_axis_fft(cx<double>* __restrict__ grid, int axis, int n1, int n2,
                                                      int n3, int k1, int k2, FftPlan p, int nl, double scale,
                                                      const cx<double>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = p.n, ls = line_stride(N);
  cx<double>* tw = reinterpret_cast<cx<double>*>(smem_raw);
  cx<double>* a = tw + N;
  cx<double>* b = a + nl * ls;
  load_tw(tw, twg, N);
  // element address of (line l, position i)
  const size_t sy = k1, sz = (size_t)k1 * k2;
  size_t base0;
  int lcount;
  size_t lstep, pstep;
  if (axis == 0) {  // lines over (y,z), contiguous in x; tile = nl consecutive y at fixed z
    const int ytiles = (n2 + nl - 1) / nl;
    const int z = blockIdx.x / ytiles, y0 = (blockIdx.x % ytiles) * nl;
    base0 = y0 * sy + z * sz;
    lcount = min(nl, n2 - y0);
    lstep = sy;
    pstep = 1;
  } else if (axis == 1) {  // lines over (x,z); tile = nl consecutive x at fixed z
    const int xtiles = (n1 + nl - 1) / nl;
    const int z = blockIdx.x / xtiles, x0 = (blockIdx.x % xtiles) * nl;
    base0 = x0 + z * sz;
    lcount = min(nl, n1 - x0);
    lstep = 1;
    pstep = sy;
  } else {  // lines over (x,y); tile = nl consecutive x at fixed y
    const int xtiles = (n1 + nl - 1) / nl;
    const int y = blockIdx.x / xtiles, x0 = (blockIdx.x % xtiles) * nl;
    base0 = x0 + y * sy;
    lcount = min(nl, n1 - x0);
    lstep = 1;
    pstep = sz;
  }
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    int l, i;
    if (axis == 0) { l = idx / N; i = idx - l * N; } else { i = idx / nl; l = idx - i * nl; }
    a[l * ls + i] = (l < lcount) ? grid[base0 + l * lstep + i * pstep] : mk<double>(0.0, 0.0);
  }
  __syncthreads();
  const cx<double>* r = fft_lines<INV>(a, b, nl, ls, p, tw);
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    int l, i;
    if (axis == 0) { l = idx / N; i = idx - l * N; } else { i = idx / nl; l = idx - i * nl; }
    if (l < lcount) grid[base0 + l * lstep + i * pstep] = scl(r[l * ls + i], scale);
  }
}

// ---------------------------------------------------------------- reductions
// Per-block partial sums, then one block folds them (deterministic order).
__global__ void k_kin_partial(const cx<double>* __restrict__ c0, int ldc, int ngw, int nstate,
                              const double* __restrict__ f, const double* __restrict__ hg, int geq0,
                              double* __restrict__ part) {
  // grid.x = blocks over G, grid.y = state
  const int i = blockIdx.y;
  double sk = 0.0, sn = 0.0;
  const double fi = f[i];
  if (fi != 0.0) {
    for (int ig = blockIdx.x * blockDim.x + threadIdx.x; ig < ngw; ig += gridDim.x * blockDim.x) {
      const cx<double> c = c0[(size_t)i * ldc + ig];
      const double a2 = c.x * c.x + c.y * c.y;
      sk += hg[ig] * a2;
      sn += (geq0 && ig == 0) ? c.x * c.x : 2.0 * a2;  // dotp_utils.mod.F90:45-52
    }
  }
  __shared__ double rk[kThreads], rn[kThreads];
  rk[threadIdx.x] = fi * sk;
  rn[threadIdx.x] = fi * sn;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rk[threadIdx.x] += rk[threadIdx.x + s];
      rn[threadIdx.x] += rn[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int b = blockIdx.y * gridDim.x + blockIdx.x;
    part[2 * b] = rk[0];
    part[2 * b + 1] = rn[0];
  }
}

__global__ void k_fold2(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double r0[kThreads], r1[kThreads];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    a += part[2 * i];
    b += part[2 * i + 1];
  }
  r0[threadIdx.x] = a;
  r1[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      r0[threadIdx.x] += r0[threadIdx.x + s];
      r1[threadIdx.x] += r1[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = r0[0];
    out[1] = r1[0];
  }
}

__global__ void k_sum_partial(const double* __restrict__ x, size_t n, double* __restrict__ part) {
  double a = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a += x[i];
  __shared__ double r[kThreads];
  r[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) r[threadIdx.x] += r[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = r[0];
    part[2 * blockIdx.x + 1] = 0.0;
  }
}

}  // namespace

// --------------------------------------------------------------------------- host side

static int lines_for(int n, int target) { return std::max(1, std::min(64, target / n)); }

template <typename T> static size_t stage_smem(int n, int nl) {
  return sizeof(cx<T>) * ((size_t)n + 2 * (size_t)nl * line_stride(n));
}

template <typename T> static int target_elems() { return sizeof(T) == 8 ? 2048 : 4096; }

template <typename KernelT> static void allow_smem(KernelT k, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T> static const cx<T>* tw_of(Ctx& c, int axis);
template <> const cx<double>* tw_of<double>(Ctx& c, int axis) { return c.tw64[axis]; }
template <> const cx<float>* tw_of<float>(Ctx& c, int axis) { return c.tw32[axis]; }

template <typename T> static int ensure_band_buffers(Ctx& c, int npairs) {
  const GeoDev& g = c.geo;
  const size_t zb = sizeof(cx<T>) * (size_t)npairs * g.n3 * g.ncol;
  const size_t yb = sizeof(cx<T>) * (size_t)npairs * g.n3 * g.n2 * g.nslot;
  const size_t qb = sizeof(cx<T>) * (size_t)npairs * g.nent;
  if (!ensure(c, c.zbuf, zb) || !ensure(c, c.ybuf, yb) || !ensure(c, c.qbuf, qb)) {
    c.err = "band workspace allocation failed";
    return 6;
  }
  return 0;
}

// inverse Z and Y stages for pairs [s0/2, s0/2 + np)
template <typename T> static int run_inverse_zy(Ctx& c, const cx<double>* c0, int ldc, int s0, int nstate, int np) {
  const GeoDev& g = c.geo;
  cx<T>* zb = static_cast<cx<T>*>(c.zbuf.p);
  cx<T>* yb = static_cast<cx<T>*>(c.ybuf.p);
  {
    const int nl = c.tune.zl ? c.tune.zl : lines_for(g.n3, target_elems<T>());
    const size_t sm = stage_smem<T>(g.n3, nl);
    allow_smem(k_zinv<T>, sm);
    dim3 grid((g.ncol + nl - 1) / nl, np);
    {
      ProfScope ps_(c, "k_zinv");
      k_zinv<T><<<grid, kThreads, sm, c.stream>>>(g, c.plan[2], c0, ldc, s0, nstate, nl, zb, tw_of<T>(c, 2));
      GBCP_LAUNCH_CHECK(c);
    }
  }
  {
    const int nl = c.tune.yl ? c.tune.yl : std::min(g.nslot, lines_for(g.n2, target_elems<T>()));
    const size_t sm = stage_smem<T>(g.n2, nl);
    allow_smem(k_yinv<T>, sm);
    dim3 grid((g.nslot + nl - 1) / nl, g.n3, np);
    {
      ProfScope ps_(c, "k_yinv");
      k_yinv<T><<<grid, kThreads, sm, c.stream>>>(g, c.plan[1], zb, nl, yb, tw_of<T>(c, 1));
      GBCP_LAUNCH_CHECK(c);
    }
  }
  return 0;
}

template <typename T> static int xlines(Ctx& c) {
  const int n1 = c.geo.n1;
  int nl = c.tune.xl ? c.tune.xl : lines_for(n1, target_elems<T>());
  // the density accumulators cap the tile at kMaxAcc*kThreads elements
  while (nl > 1 && nl * n1 > kMaxAcc * kThreads) --nl;
  return nl;
}

template <typename T>
static int rhoofr_t(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho) {
  const GeoDev& g = c.geo;
  const int npairs_total = (nstate + 1) / 2;
  int rc = ensure_band_buffers<T>(c, std::min(c.batch, npairs_total));
  if (rc) return rc;
  const int nl = xlines<T>(c);
  if (nl * g.n1 > kMaxAcc * kThreads) {
    c.err = "mesh too large for the density tile";
    return 7;
  }
  const size_t sm = stage_smem<T>(g.n1, nl);
  allow_smem(k_xinv_rho<T>, sm);
  for (int p0 = 0; p0 < npairs_total; p0 += c.batch) {
    const int np = std::min(c.batch, npairs_total - p0);
    const int s0 = 2 * p0;
    rc = run_inverse_zy<T>(c, c0, ldc, s0, nstate, np);
    if (rc) return rc;
    dim3 grid((g.n2 + nl - 1) / nl, g.n3);
    {
      ProfScope ps_(c, "k_xinv_rho");
      k_xinv_rho<T><<<grid, kThreads, sm, c.stream>>>(g, c.plan[0], static_cast<const cx<T>*>(c.ybuf.p), np, s0,
                                                      nstate, f, 1.0 / c.omega, rho, nl, tw_of<T>(c, 0));
      GBCP_LAUNCH_CHECK(c);
    }
  }
  return 0;
}

template <typename T>
static int vpsi_t(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f,
                  const double* vpot, int nstate) {
  const GeoDev& g = c.geo;
  const int npairs_total = (nstate + 1) / 2;
  int rc = ensure_band_buffers<T>(c, std::min(c.batch, npairs_total));
  if (rc) return rc;
  cx<T>* zb = static_cast<cx<T>*>(c.zbuf.p);
  cx<T>* yb = static_cast<cx<T>*>(c.ybuf.p);
  cx<T>* qb = static_cast<cx<T>*>(c.qbuf.p);
  const T scale = (T)(1.0 / ((double)g.n1 * g.n2 * g.n3));
  for (int p0 = 0; p0 < npairs_total; p0 += c.batch) {
    const int np = std::min(c.batch, npairs_total - p0);
    const int s0 = 2 * p0;
    rc = run_inverse_zy<T>(c, c0, ldc, s0, nstate, np);
    if (rc) return rc;
    {
      const int nl = c.tune.xl ? c.tune.xl : lines_for(g.n1, target_elems<T>());
      const size_t sm = stage_smem<T>(g.n1, nl);
      allow_smem(k_xvx<T>, sm);
      dim3 grid((g.n2 + nl - 1) / nl, g.n3, np);
      {
        ProfScope ps_(c, "k_xvx");
        k_xvx<T><<<grid, kThreads, sm, c.stream>>>(g, c.plan[0], yb, vpot, nl, tw_of<T>(c, 0));
        GBCP_LAUNCH_CHECK(c);
      }
    }
    {
      const int nl = c.tune.yl ? c.tune.yl : std::min(g.nslot, lines_for(g.n2, target_elems<T>()));
      const size_t sm = stage_smem<T>(g.n2, nl);
      allow_smem(k_yfwd<T>, sm);
      dim3 grid((g.nslot + nl - 1) / nl, g.n3, np);
      {
        ProfScope ps_(c, "k_yfwd");
        k_yfwd<T><<<grid, kThreads, sm, c.stream>>>(g, c.plan[1], yb, nl, zb, tw_of<T>(c, 1));
        GBCP_LAUNCH_CHECK(c);
      }
    }
    {
      const int nl = c.tune.zl ? c.tune.zl : lines_for(g.n3, target_elems<T>());
      const size_t sm = stage_smem<T>(g.n3, nl);
      allow_smem(k_zfwd<T>, sm);
      dim3 grid((g.ncol + nl - 1) / nl, np);
      {
        ProfScope ps_(c, "k_zfwd");
        k_zfwd<T><<<grid, kThreads, sm, c.stream>>>(g, c.plan[2], zb, nl, scale, qb, tw_of<T>(c, 2));
        GBCP_LAUNCH_CHECK(c);
      }
    }
    {
      dim3 grid((g.ngw + 255) / 256, np);
      {
        ProfScope ps_(c, "k_decode");
        k_decode<T><<<grid, 256, 0, c.stream>>>(g, qb, c0, ldc, c2, ldc2, f, s0, nstate, c.tpiba2);
        GBCP_LAUNCH_CHECK(c);
      }
    }
  }
  return 0;
}

int band_rhoofr(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho) {
  GBCP_CUDA_TRY(c, cudaMemsetAsync(rho, 0, sizeof(double) * (size_t)c.kr[0] * c.kr[1] * c.kr[2], c.stream));
  if (nstate <= 0) return 0;
  return c.precision == 0 ? rhoofr_t<double>(c, c0, ldc, nstate, f, rho) : rhoofr_t<float>(c, c0, ldc, nstate, f, rho);
}

int band_vpsi(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f, const double* vpot,
              int nstate) {
  if (nstate <= 0) return 0;
  return c.precision == 0 ? vpsi_t<double>(c, c0, ldc, c2, ldc2, f, vpot, nstate)
                          : vpsi_t<float>(c, c0, ldc, c2, ldc2, f, vpot, nstate);
}

int dense_fft(Ctx& c, cx<double>* grid, bool inv) {
  const int n1 = c.nr[0], n2 = c.nr[1], n3 = c.nr[2], k1 = c.kr[0], k2 = c.kr[1];
  const double scale_last = inv ? 1.0 : 1.0 / ((double)n1 * n2 * n3);
  // inverse: x, y, z (fftnew sparse order); forward: z, y, x
  const int order_inv[3] = {0, 1, 2}, order_fw[3] = {2, 1, 0};
  for (int s = 0; s < 3; ++s) {
    const int axis = inv ? order_inv[s] : order_fw[s];
    const int n = c.nr[axis];
    const int nl = lines_for(n, 2048);
    const size_t sm = stage_smem<double>(n, nl);
    int nblk;
    if (axis == 0) nblk = ((n2 + nl - 1) / nl) * n3;
    else if (axis == 1) nblk = ((n1 + nl - 1) / nl) * n3;
    else nblk = ((n1 + nl - 1) / nl) * n2;
    const double sc = (s == 2) ? scale_last : 1.0;
    ProfScope ps_(c, "k_axis_fft");
    if (inv) {
      allow_smem(k_axis_fft<true>, sm);
      k_axis_fft<true><<<nblk, kThreads, sm, c.stream>>>(grid, axis, n1, n2, n3, k1, k2, c.plan[axis], nl, sc,
                                                           c.tw64[axis]);
    } else {
      allow_smem(k_axis_fft<false>, sm);
      k_axis_fft<false><<<nblk, kThreads, sm, c.stream>>>(grid, axis, n1, n2, n3, k1, k2, c.plan[axis], nl, sc,
                                                            c.tw64[axis]);
    }
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

int kin_energy(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* ekin, double* csumg) {
  const int gx = std::max(1, std::min(64, (c.ngw + kThreads - 1) / kThreads));
  const int nb = gx * nstate;
  if (!ensure(c, c.red, sizeof(double) * (2 * (size_t)nb + 2))) return 6;
  double* part = static_cast<double*>(c.red.p);
  {
    ProfScope ps_(c, "k_kin_partial");
    k_kin_partial<<<dim3(gx, nstate), kThreads, 0, c.stream>>>(c0, ldc, c.ngw, nstate, f, c.geo.hg, c.geq0, part);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_fold2");
    k_fold2<<<1, kThreads, 0, c.stream>>>(part, nb, part + 2 * nb);
    GBCP_LAUNCH_CHECK(c);
  }
  double h[2];
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(h, part + 2 * nb, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (ekin) *ekin = h[0] * c.tpiba2;
  if (csumg) *csumg = h[1];
  if (!std::isfinite(h[0]) || !std::isfinite(h[1])) {
    c.err = "non-finite kinetic energy / norm";
    return 3;
  }
  return 0;
}

int rho_sum(Ctx& c, const double* rho, double* sum) {
  const size_t n = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  const int nb = 296;
  if (!ensure(c, c.red, sizeof(double) * (2 * (size_t)nb + 2))) return 6;
  double* part = static_cast<double*>(c.red.p);
  {
    ProfScope ps_(c, "k_sum_partial");
    k_sum_partial<<<nb, kThreads, 0, c.stream>>>(rho, n, part);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_fold2");
    k_fold2<<<1, kThreads, 0, c.stream>>>(part, nb, part + 2 * nb);
    GBCP_LAUNCH_CHECK(c);
  }
  double h[2];
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(h, part + 2 * nb, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  *sum = h[0];
  if (!std::isfinite(h[0])) {
    c.err = "non-finite density";
    return 3;
  }
  return 0;
}

}  // namespace gbcp
