// Four-step band-loop stage kernels (compile-time mesh sizes).
//
// A line of length N = N1*N2 is transformed by two groups of threads with one
// shared-memory exchange in between:
//   step A  thread (line, n2) holds x[n2 + N2 n1], n1 < N1, in registers:
//           DFT of length N1, twiddle e^{S 2 pi i n2 k1 / N}, store T[k1][n2];
//   step B  thread (line, k1) reads T[k1][*]: DFT of length N2, giving
//           X[k1 + N1 k2], k2 < N2, in registers.
// The forward transform that vpsi applies after V(r) starts from that
// register layout (stride N1) without an exchange: DFT of length N2 over k2,
// twiddle e^{-2 pi i k1 j / N}, store, DFT of length N1, output X[j + N2 j2].
// The DFTs are the register codelets of fft_codelets.cuh.  Each stage kernel
// maps its two thread groups so that global loads and stores are coalesced.
//
// Plans (N1 x N2, lines per CTA L) keep both thread groups near 256 tasks.
#pragma once
#include "fft_codelets.cuh"
#include "fs_plan.h"

namespace gbcp {
namespace band {

template <typename T, int N> struct FS {
  static constexpr int N1 = fs_n1(N), N2 = N / N1, L = fs_lines(N);
  static constexpr int LS = N + ((N % 2 == 0) ? 1 : 0);  // y/z stages: odd line stride, rows of N2
  static constexpr int XP = fs_xpitch(N), XS = fs_xstride(N);  // x stage: row pitch, line stride
  static constexpr int TA = L * N2, TB = L * N1;
  static constexpr int IA = (TA + kThreads - 1) / kThreads, IB = (TB + kThreads - 1) / kThreads;
  static_assert(XP >= N2 && XS >= N1 * XP, "x-stage layout");
};

template <typename T> __device__ __forceinline__ cx<T> twmul(cx<T> v, cx<T> w, bool conj) {
  return conj ? cmulc(v, w) : cmul(v, w);
}

// step A on registers v[N1] of line position n2; writes T[k1][n2] = line[k1*PITCH + n2].
// PR (N1 = 8): the line's input lies within frequencies [-N/4, N/4), so v[2] .. v[5]
// (positions n2 + N2 n1, n1 = 2..5) are zero and are neither loaded nor transformed
template <int S, typename T, int N1, int N2, int PITCH = N2, bool PR = false>
__device__ __forceinline__ void fs_step_a(cx<T> (&v)[N1], int n2, const cx<T>* __restrict__ twA, cx<T>* line) {
  if constexpr (PR && N1 == 8)
    dft8_lo<S>(v);
  else
    dftn<S, N1>(v);
#pragma unroll
  for (int k1 = 0; k1 < N1; ++k1) {
    cx<T> r = v[k1];
    if (k1 > 0 && n2 > 0) r = twmul(r, twA[k1 * N2 + n2], S < 0);
    line[k1 * PITCH + n2] = r;
  }
}

// step B: read row k1 of the line, DFT of length N2
template <int S, typename T, int N1, int N2, int PITCH = N2>
__device__ __forceinline__ void fs_step_b(const cx<T>* line, int k1, cx<T> (&w)[N2]) {
#pragma unroll
  for (int n2 = 0; n2 < N2; ++n2) w[n2] = line[k1 * PITCH + n2];
  dftn<S, N2>(w);
}

// cp.async copies of complex elements (8 or 16 bytes), their commit and wait
template <typename T> __device__ __forceinline__ void cp_async_cx(cx<T>* dst, const cx<T>* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  if constexpr (sizeof(cx<T>) == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int NPEND> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(NPEND) : "memory");
}

template <typename T>
__device__ __forceinline__ void load_table(cx<T>* dst, const cx<T>* __restrict__ src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// ---------------------------------------------------------------- Z stage (inverse, gather)
// CTA (column block, pair): the gather of its L sphere columns straight from c0
// through the dense table g.zgat, pair packing, step A and step B.
// MIR: the full sphere's columns, sorted by (gx, gy), form a centrally symmetric
// set, so the mirror (-gx, -gy) of column c is column ncol - 1 - c and its entry
// at -z is the -G of the entry at z (code -e).  A CTA then takes L primary
// columns c < ceil(ncol / 2) and their mirrors: each coefficient and each
// gather-table entry is loaded once and feeds both lines (c1 + i c2 at +G, its
// conjugate packing at -G).  In the four-step layout the mirror of thread
// (n2, n1) is (N2 - n2, N1 - 1 - n1), or (0, (N1 - n1) mod N1) for n2 = 0, so the
// same thread runs step A of both lines.  The column (0, 0), its own mirror,
// keeps one line.  Half the CTAs with twice the work and shared memory each: a
// gain where the column set is large (a single 120^3 cell: 104 -> 90 us per
// 64-pair launch), a loss among the small concurrent kernels of a batch.
template <typename T, int N, bool MIR>
__global__ void __launch_bounds__(kThreads) k_zinv_fs(GeoDev g, const cx<double>* __restrict__ c0, int psi32, int ldc,
                                                     int s0, int nstate, cx<T>* __restrict__ zbuf,
                                                     const cx<T>* __restrict__ twAg, const double* __restrict__ f,
                                                     double* __restrict__ kpart, const unsigned long long* keep) {
  if (zk_kept(keep)) return;
  using P = FS<T, N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* twA = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* Ts = twA + N;  // lines l (primary) and, with MIR, L + l (mirror)
  const int col0 = blockIdx.x * P::L, pair = blockIdx.y;
  const int half = MIR ? (g.ncol + 1) / 2 : g.ncol;
  const int is1 = s0 + 2 * pair, is2 = is1 + 1;
  const bool two = is2 < nstate;
  const size_t o1 = (size_t)is1 * ldc, o2 = (size_t)(two ? is2 : is1) * ldc;
  KinAcc<T> kacc;
  load_table(twA, twAg, N);
  __syncthreads();
  // the gather table: one coalesced 8-byte load per (line, z), then the coefficients
  const int2* zg = g.zgat + (size_t)blockIdx.x * (P::N1 * P::N2 * P::L);
#pragma unroll
  for (int ia = 0; ia < P::IA; ++ia) {
    const int t = threadIdx.x + ia * kThreads;
    if (t < P::TA) {
      const int n2 = t / P::L, l = t - n2 * P::L, col = col0 + l;
      const bool prim = col < half, mir = MIR && prim && g.ncol - 1 - col != col;
      cx<T> v[P::N1], u[P::N1];
      int2 ce[P::N1];
#pragma unroll
      for (int n1 = 0; n1 < P::N1; ++n1) ce[n1] = prim ? zg[(n1 * P::N2 + n2) * P::L + l] : int2{0, 0};
#pragma unroll
      for (int n1 = 0; n1 < P::N1; ++n1) {
        const int e = ce[n1].x;
        cx<T> val = mk<T>(0, 0), mval = mk<T>(0, 0);
        if (e != 0) {
          const int ig = (e > 0 ? e : -e) - 1;
          T ux, uy, wx = 0, wy = 0;
          load_coef<T>(c0, psi32, o1 + ig, ux, uy);
          if (two) load_coef<T>(c0, psi32, o2 + ig, wx, wy);
          const cx<T> pp = mk<T>(ux - wy, uy + wx), pm = mk<T>(ux + wy, wx - uy);  // at +G, at -G
          val = e > 0 ? pp : pm;
          mval = e > 0 ? pm : pp;
          // each coefficient once: at +G, or with MIR at either sign outside the
          // self-mirror column
          if (kpart && (e > 0 || mir)) kin_entry_t(kacc, g, ig, __int_as_float(ce[n1].y), ux, uy, wx, wy);
        }
        v[n1] = val;
        u[n1] = mval;
      }
      fs_step_a<1, T, P::N1, P::N2>(v, n2, twA, Ts + l * P::LS);
      if constexpr (MIR) {
        cx<T> vm[P::N1];
        if (n2 == 0) {  // uniform per warp when L is a multiple of 32
#pragma unroll
          for (int n1 = 0; n1 < P::N1; ++n1) vm[(P::N1 - n1) % P::N1] = u[n1];
        } else {
#pragma unroll
          for (int n1 = 0; n1 < P::N1; ++n1) vm[P::N1 - 1 - n1] = u[n1];
        }
        fs_step_a<1, T, P::N1, P::N2>(vm, n2 == 0 ? 0 : P::N2 - n2, twA, Ts + (P::L + l) * P::LS);
      }
    }
  }
  __syncthreads();
  cx<T>* zb = zbuf + (size_t)pair * N * g.ncol;
#pragma unroll
  for (int ib = 0; ib < (MIR ? 2 : 1) * P::IB; ++ib) {
    const int t = threadIdx.x + (ib % P::IB) * kThreads, side = ib / P::IB;
    if (t < P::TB) {
      const int k1 = t / P::L, l = t - k1 * P::L, col = col0 + l;
      const bool ok = side == 0 ? col < half : (col < half && g.ncol - 1 - col != col);
      cx<T> w[P::N2];
      fs_step_b<1, T, P::N1, P::N2>(Ts + (side * P::L + l) * P::LS, k1, w);
      if (ok) {
        const int oc = side == 0 ? col : g.ncol - 1 - col;
#pragma unroll
        for (int k2 = 0; k2 < P::N2; ++k2) zb[(size_t)(k1 + P::N1 * k2) * g.ncol + oc] = w[k2];
      }
    }
  }
  if (kpart)
    kin_flush(kacc, f[is1], two ? f[is2] : 0.0,
              kpart + 2 * kin_slots<T>() * ((size_t)(s0 / 2 + pair) * gridDim.x + blockIdx.x));
}

// ---------------------------------------------------------------- Y stage (inverse)
template <typename T, int N, bool PR>
__global__ void __launch_bounds__(kThreads) k_yinv_fs(GeoDev g, const cx<T>* __restrict__ zbuf,
                                                     cx<T>* __restrict__ ybuf, const cx<T>* __restrict__ twAg) {
  using P = FS<T, N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* twA = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* Ts = twA + N;
  const int sb = blockIdx.x * P::L, z = blockIdx.y, pair = blockIdx.z;
  const cx<T>* zrow = zbuf + ((size_t)pair * g.n3 + z) * g.ncol;
  // FP32: the block's sphere columns (one contiguous run of zbuf) copied in with
  // cp.async, so that the scattered reads of step A hit shared memory
  constexpr bool STAGE = sizeof(T) == 4;
  cx<T>* zs = Ts + P::L * P::LS;
  const int cb = g.slot_col0[sb], ce = sb + P::L < g.nslot ? g.slot_col0[sb + P::L] : g.ncol;
  if constexpr (STAGE) {
    for (int e = cb + (int)threadIdx.x; e < ce; e += kThreads) cp_async_cx(zs + (e - cb), zrow + e);
    cp_async_commit();
  }
  load_table(twA, twAg, N);
  if constexpr (STAGE) cp_async_wait<0>();
  __syncthreads();
  const cx<T>* zsrc = STAGE ? zs - cb : zrow;
#pragma unroll
  for (int ia = 0; ia < P::IA; ++ia) {
    const int t = threadIdx.x + ia * kThreads;
    if (t < P::TA) {
      const int n2 = t / P::L, l = t - n2 * P::L, s = sb + l;
      int c0s = 0, gylo = 0, ncs = 0;
      if (s < g.nslot) {
        c0s = g.slot_col0[s];
        gylo = g.slot_gylo[s];
        ncs = g.slot_ncol[s];
      }
      cx<T> v[P::N1];
#pragma unroll
      for (int n1 = 0; n1 < P::N1; ++n1) {
        const int off = freq_split<N, P::N2>(n2, n1) - gylo;
        v[n1] = in_range(off, ncs) ? zsrc[c0s + off] : mk<T>(0, 0);
      }
      fs_step_a<1, T, P::N1, P::N2, P::N2, PR>(v, n2, twA, Ts + l * P::LS);
    }
  }
  __syncthreads();
  cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)N * g.nslot;
#pragma unroll
  for (int ib = 0; ib < P::IB; ++ib) {
    const int t = threadIdx.x + ib * kThreads;
    if (t < P::TB) {
      const int k1 = t / P::L, l = t - k1 * P::L, s = sb + l;
      cx<T> w[P::N2];
      fs_step_b<1, T, P::N1, P::N2>(Ts + l * P::LS, k1, w);
      if (s < g.nslot) {
#pragma unroll
        for (int k2 = 0; k2 < P::N2; ++k2) yb[(size_t)(k1 + P::N1 * k2) * g.nslot + s] = w[k2];
      }
    }
  }
}

// step A of an x-line: gather the sphere slots of row y (l-major thread map)
template <typename T, int N, bool PR = false>
__device__ __forceinline__ void xline_step_a(const GeoDev& g, const cx<T>* __restrict__ yb, int y0,
                                             const cx<T>* twA, cx<T>* Ts) {
  using P = FS<T, N>;
#pragma unroll
  for (int ia = 0; ia < P::IA; ++ia) {
    const int t = threadIdx.x + ia * kThreads;
    if (t < P::TA) {
      const int l = t / P::N2, n2 = t - l * P::N2, y = y0 + l;
      cx<T> v[P::N1];
#pragma unroll
      for (int n1 = 0; n1 < P::N1; ++n1) {
        const int s = freq_split<N, P::N2>(n2, n1) - g.gxlo;
        v[n1] = (y < g.n2 && in_range(s, g.nslot)) ? yb[(size_t)y * g.nslot + s] : mk<T>(0, 0);
      }
      fs_step_a<1, T, P::N1, P::N2, P::XP, PR>(v, n2, twA, Ts + l * P::XS);
    }
  }
}

// ---------------------------------------------------------------- X stage + density
// asynchronous global -> shared copy of one complex (LDGSTS; completes without a wait loop)
// slab buffers of the density x-stage: two (copy of the next pair overlaps the
// current one) in FP32, one in FP64 (shared memory)
template <typename T> __host__ __device__ constexpr int xrho_bufs() { return sizeof(T) == 4 ? 2 : 1; }

// CTA (chunk, y-block, z): the x-lines y0 .. y0+L-1 of plane z for the pairs
// [chunk*pchunk, ..).  Each pair's slots of those lines are one contiguous run of
// ybuf (L rows of nslot), copied to shared memory with cp.async one pair ahead.
// The CTA's density contribution sum_pairs f1 |Re psi|^2 + f2 |Im psi|^2 builds
// up in registers (T).  With one chunk it is added to rho directly; with
// several, each CTA stores its partial tile, and the last CTA of the tile to
// finish (ticket counter) adds the partials in chunk order: the result does not
// depend on the order the CTAs run in.
template <typename T, int N, bool PR>
__global__ void __launch_bounds__(kThreads) k_xrho_fs(GeoDev g, const cx<T>* __restrict__ ybuf, int npairs, int s0,
                                                     int nstate, const double* __restrict__ f, double inv_omega,
                                                     double* __restrict__ rho, const cx<T>* __restrict__ twAg,
                                                     int pchunk, T* __restrict__ part, unsigned* __restrict__ tickets,
                                                     int z0) {
  using P = FS<T, N>;
  constexpr int NBUF = xrho_bufs<T>();
  static_assert(P::IB == 1, "density tile: one step-B task per thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* twA = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* Ts = twA + N;
  cx<T>* slab = Ts + P::L * P::XS;
  const int nslot = g.nslot, slab_n = P::L * nslot;
  const int nchunk = gridDim.x, chunk = blockIdx.x, y0 = blockIdx.y * P::L, z = z0 + blockIdx.z;  // planes z0 ..
  const int p0 = chunk * pchunk, p1 = min(npairs, p0 + pchunk);
  const int nel = min(P::L, g.n2 - y0) * nslot;
  load_table(twA, twAg, N);
  T acc[P::N2];
#pragma unroll
  for (int k2 = 0; k2 < P::N2; ++k2) acc[k2] = (T)0;
  __shared__ T fw[2 * kMaxBatch];
  __shared__ int last_sh;
  for (int i = threadIdx.x; i < 2 * (p1 - p0); i += kThreads) {
    const int is = s0 + 2 * p0 + i;
    fw[i] = from_double<T>(is < nstate ? f[is] * inv_omega : 0.0);
  }
  auto issue = [&](int pair, int buf) {
    const cx<T>* src = ybuf + (((size_t)pair * g.n3 + z) * g.n2 + y0) * (size_t)nslot;
    cx<T>* dst = slab + buf * slab_n;
    for (int e = threadIdx.x; e < nel; e += kThreads) cp_async_cx(dst + e, src + e);
    cp_async_commit();
  };
  const int t = threadIdx.x;
  const int lb = t / P::N1, k1 = t - lb * P::N1;
  if (p0 < p1) issue(p0, 0);
  for (int pair = p0; pair < p1; ++pair) {
    const int buf = (NBUF == 2) ? ((pair - p0) & 1) : 0;
    if (NBUF == 2 && pair + 1 < p1) {
      issue(pair + 1, buf ^ 1);  // buffer buf^1 was last read before the previous mid-pair barrier
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // slab of this pair in shared memory; previous step B done with Ts
    const cx<T>* sl = slab + buf * slab_n;
#pragma unroll
    for (int ia = 0; ia < P::IA; ++ia) {
      const int ta = threadIdx.x + ia * kThreads;
      if (ta < P::TA) {
        const int l = ta / P::N2, n2 = ta - l * P::N2, y = y0 + l;
        cx<T> v[P::N1];
#pragma unroll
        for (int n1 = 0; n1 < P::N1; ++n1) {
          const int s = freq_split<N, P::N2>(n2, n1) - g.gxlo;
          v[n1] = (y < g.n2 && in_range(s, nslot)) ? sl[l * nslot + s] : mk<T>(0, 0);
        }
        fs_step_a<1, T, P::N1, P::N2, P::XP, PR>(v, n2, twA, Ts + l * P::XS);
      }
    }
    __syncthreads();
    if (NBUF == 1 && pair + 1 < p1) issue(pair + 1, 0);  // slab read by every thread; overlaps step B
    const T f1 = fw[2 * (pair - p0)], f2 = fw[2 * (pair - p0) + 1];
    if (t < P::TB) {
      cx<T> w[P::N2];
      fs_step_b<1, T, P::N1, P::N2, P::XP>(Ts + lb * P::XS, k1, w);
#pragma unroll
      for (int k2 = 0; k2 < P::N2; ++k2) acc[k2] += f1 * w[k2].x * w[k2].x + f2 * w[k2].y * w[k2].y;
    }
  }
  const int y = y0 + lb;
  double* rrow = rho + (size_t)g.k1 * ((y < g.n2 ? y : 0) + (size_t)g.k2 * z);
  if (nchunk == 1) {
    if (t < P::TB && y < g.n2) {
#pragma unroll
      for (int k2 = 0; k2 < P::N2; ++k2) rrow[k1 + P::N1 * k2] += to_double<T>(acc[k2]);
    }
    return;
  }
  const int tile = z * gridDim.y + blockIdx.y;
  T* mine = part + ((size_t)tile * nchunk + chunk) * (P::TB * P::N2);
  if (t < P::TB) {
#pragma unroll
    for (int k2 = 0; k2 < P::N2; ++k2) mine[k2 * P::TB + t] = acc[k2];
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last_sh = (atomicAdd(&tickets[tile], 1u) == (unsigned)(nchunk - 1));
  __syncthreads();
  if (!last_sh) return;
  __threadfence();
  if (t < P::TB && y < g.n2) {
    const T* tp = part + (size_t)tile * nchunk * (P::TB * P::N2);
#pragma unroll
    for (int k2 = 0; k2 < P::N2; ++k2) {
      if constexpr (sizeof(T) == 4) {
        // chunk order in double-float (two FP64 additions per element instead of nchunk + 1)
        float h = 0.f, l = 0.f;
        for (int q = 0; q < nchunk; ++q) df_add(h, l, __ldcg(tp + (size_t)q * (P::TB * P::N2) + k2 * P::TB + t), 0.f);
        rrow[k1 + P::N1 * k2] += f2d_int(h) + f2d_int(l);
      } else {
        double sum = 0.0;
        for (int q = 0; q < nchunk; ++q) sum += to_double<T>(__ldcg(tp + (size_t)q * (P::TB * P::N2) + k2 * P::TB + t));
        rrow[k1 + P::N1 * k2] += sum;
      }
    }
  }
  if (threadIdx.x == 0) tickets[tile] = 0u;  // ready for the next launch
}

// ---------------------------------------------------------------- X stage: inverse, x V, forward
template <typename T, int N, bool PR>
__global__ void __launch_bounds__(kThreads) k_xvx_fs(GeoDev g, cx<T>* __restrict__ ybuf,
                                                    const T* __restrict__ vpot, const cx<T>* __restrict__ twAg,
                                                    const cx<T>* __restrict__ twBg) {
  using P = FS<T, N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* twA = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* twB = twA + N;
  cx<T>* Ts = twB + N;  // one exchange buffer: step B reads and rewrites only its own row k1
  const int y0 = blockIdx.x * P::L, z = blockIdx.y, pair = blockIdx.z;
  cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)g.n2 * g.nslot;
  load_table(twA, twAg, N);
  load_table(twB, twBg, N);
  __syncthreads();
  xline_step_a<T, N, PR>(g, yb, y0, twA, Ts);
  __syncthreads();
#pragma unroll
  for (int ib = 0; ib < P::IB; ++ib) {
    const int t = threadIdx.x + ib * kThreads;
    if (t < P::TB) {
      const int l = t / P::N1, k1 = t - l * P::N1, y = y0 + l;
      cx<T> w[P::N2];
      fs_step_b<1, T, P::N1, P::N2, P::XP>(Ts + l * P::XS, k1, w);
      const T* vrow = vpot + (size_t)g.k1 * ((y < g.n2 ? y : 0) + (size_t)g.k2 * z);
#pragma unroll
      for (int k2 = 0; k2 < P::N2; ++k2) w[k2] = scl(w[k2], (y < g.n2) ? vrow[k1 + P::N1 * k2] : (T)0);
      // forward: DFT over k2 (stride-N1 elements), twiddle, back into row k1
      dftn<-1, P::N2>(w);
      cx<T>* line = Ts + l * P::XS;
#pragma unroll
      for (int j = 0; j < P::N2; ++j) {
        cx<T> r = w[j];
        if (j > 0 && k1 > 0) r = cmulc(r, twB[j * P::N1 + k1]);
        line[k1 * P::XP + j] = r;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int ia = 0; ia < P::IA; ++ia) {
    const int t = threadIdx.x + ia * kThreads;
    if (t < P::TA) {
      const int l = t / P::N2, j = t - l * P::N2, y = y0 + l;
      const cx<T>* line = Ts + l * P::XS;
      cx<T> u[P::N1];
#pragma unroll
      for (int k1 = 0; k1 < P::N1; ++k1) u[k1] = line[k1 * P::XP + j];
      dftn<-1, P::N1>(u);
      if (y < g.n2) {
#pragma unroll
        for (int j2 = 0; j2 < P::N1; ++j2) {
          // PR: outputs 2 .. 5 lie outside the sphere's x range (and go unused)
          if (!(PR && P::N1 == 8 && j2 >= 2 && j2 <= 5)) {
            const int s = freq_split<N, P::N2>(j, j2) - g.gxlo;
            if (in_range(s, g.nslot)) yb[(size_t)y * g.nslot + s] = u[j2];
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------- Y stage (forward)
template <typename T, int N>
__global__ void __launch_bounds__(kThreads) k_yfwd_fs(GeoDev g, const cx<T>* __restrict__ ybuf,
                                                     cx<T>* __restrict__ zbuf, const cx<T>* __restrict__ twAg) {
  using P = FS<T, N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* twA = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* Ts = twA + N;
  const int sb = blockIdx.x * P::L, z = blockIdx.y, pair = blockIdx.z;
  const cx<T>* yb = ybuf + ((size_t)pair * g.n3 + z) * (size_t)N * g.nslot;
  load_table(twA, twAg, N);
  __syncthreads();
#pragma unroll
  for (int ia = 0; ia < P::IA; ++ia) {
    const int t = threadIdx.x + ia * kThreads;
    if (t < P::TA) {
      const int n2 = t / P::L, l = t - n2 * P::L, s = sb + l;
      cx<T> v[P::N1];
#pragma unroll
      for (int n1 = 0; n1 < P::N1; ++n1)
        v[n1] = (s < g.nslot) ? yb[(size_t)(n2 + P::N2 * n1) * g.nslot + s] : mk<T>(0, 0);
      fs_step_a<-1, T, P::N1, P::N2>(v, n2, twA, Ts + l * P::LS);
    }
  }
  __syncthreads();
  cx<T>* zrow = zbuf + ((size_t)pair * g.n3 + z) * g.ncol;
#pragma unroll
  for (int ib = 0; ib < P::IB; ++ib) {
    const int t = threadIdx.x + ib * kThreads;
    if (t < P::TB) {
      const int k1 = t / P::L, l = t - k1 * P::L, s = sb + l;
      cx<T> w[P::N2];
      fs_step_b<-1, T, P::N1, P::N2>(Ts + l * P::LS, k1, w);
      if (s < g.nslot) {
        const int c0s = g.slot_col0[s], gylo = g.slot_gylo[s], ncs = g.slot_ncol[s];
#pragma unroll
        for (int k2 = 0; k2 < P::N2; ++k2) {
          const int off = freq_split<N, P::N1>(k1, k2) - gylo;
          if (in_range(off, ncs)) zrow[c0s + off] = w[k2];
        }
      }
    }
  }
}

// ---------------------------------------------------------------- Z stage (forward, to sphere entries)
template <typename T, int N>
__global__ void __launch_bounds__(kThreads) k_zfwd_fs(GeoDev g, const cx<T>* __restrict__ zbuf, T scale,
                                                     cx<T>* __restrict__ qbuf, const cx<T>* __restrict__ twAg) {
  using P = FS<T, N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* twA = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* Ts = twA + N;
  const int col0 = blockIdx.x * P::L, pair = blockIdx.y;
  const cx<T>* zb = zbuf + (size_t)pair * N * g.ncol;
  load_table(twA, twAg, N);
  __syncthreads();
#pragma unroll
  for (int ia = 0; ia < P::IA; ++ia) {
    const int t = threadIdx.x + ia * kThreads;
    if (t < P::TA) {
      const int n2 = t / P::L, l = t - n2 * P::L, col = col0 + l;
      cx<T> v[P::N1];
#pragma unroll
      for (int n1 = 0; n1 < P::N1; ++n1)
        v[n1] = (col < g.ncol) ? zb[(size_t)(n2 + P::N2 * n1) * g.ncol + col] : mk<T>(0, 0);
      fs_step_a<-1, T, P::N1, P::N2>(v, n2, twA, Ts + l * P::LS);
    }
  }
  __syncthreads();
  cx<T>* qb = qbuf + (size_t)pair * g.nent;
#pragma unroll
  for (int ib = 0; ib < P::IB; ++ib) {
    const int t = threadIdx.x + ib * kThreads;
    if (t < P::TB) {
      const int k1 = t / P::L, l = t - k1 * P::L, col = col0 + l;
      cx<T> w[P::N2];
      fs_step_b<-1, T, P::N1, P::N2>(Ts + l * P::LS, k1, w);
      if (col < g.ncol) {
        const int st = g.col_start[col], len = g.col_start[col + 1] - st, zlo = g.col_zlo[col];
#pragma unroll
        for (int k2 = 0; k2 < P::N2; ++k2) {
          const int off = freq_split<N, P::N1>(k1, k2) - zlo;
          if (in_range(off, len)) qb[st + off] = scl(w[k2], scale);
        }
      }
    }
  }
}

}  // namespace band
}  // namespace gbcp
