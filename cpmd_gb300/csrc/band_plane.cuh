// Plane-fused Y and X stages of the FP32 band loop.
//
// The three-stage band loop (band_fs.cuh) writes the y-transformed slot lines of
// every z-plane to HBM (ybuf: 405 MB per 64-pair launch of the 120^3 cell) and
// reads them back in the x-stage, and vpsi does it twice more on the way back.
// Here one CTA keeps the whole z-plane of one pair in shared memory: the slot
// lines Pl[s][y] (nslot lines of P::LS complex), inverse y-transforms of the
// sphere columns straight from zbuf, then the x-rows block by block (the
// x-stage of band_fs.cuh, reading and writing Pl instead of ybuf), and for vpsi
// the forward y-transforms back into zbuf.  Only zbuf (sphere columns) and
// V(r) / rho touch HBM.  Used for FP32 transforms where the plane fits in
// shared memory (nslot * (N + 1) + one exchange tile: the 120^3 and 144^3
// cells, not 240^3) and the x and y lengths are equal.
#pragma once

namespace gbcp {
namespace band {

// shared-memory layout of a plane CTA, in complex elements: twiddle tables, one
// exchange tile X (the y-stage LS layout or the x-stage XS layout), the plane
template <int N> struct PlaneLayout {
  using P = FS<float, N>;
  static constexpr int XEL = (P::L * P::LS > P::L * P::XS) ? P::L * P::LS : P::L * P::XS;
  static constexpr int NB = (N + P::L - 1) / P::L;  // x-row blocks of a plane
  // `tiles` exchange tiles (one per group of kThreads threads)
  __host__ __device__ static constexpr size_t bytes(int tables, int nslot, int tiles = 1) {
    return sizeof(cx<float>) * ((size_t)tables * N + (size_t)tiles * XEL + (size_t)nslot * P::LS);
  }
};

// inverse y-transforms of the slot lines of one z-plane: zrow (sphere columns of
// the plane) -> Pl[s * LS + y]; ends with a barrier.  The CTA is nh groups of
// kThreads threads (tt = thread within the group, h = group); group h transforms
// the slot-line blocks h, h + nh, ... in its own exchange tile X, every group
// running the same number of barriers.
template <int N, bool PR = false>
__device__ __forceinline__ void plane_yinv(const GeoDev& g, const cx<float>* __restrict__ zrow, const cx<float>* twy,
                                           cx<float>* Pl, cx<float>* X, int tt = threadIdx.x, int h = 0, int nh = 1) {
  using P = FS<float, N>;
  const int nblk = (g.nslot + P::L - 1) / P::L;
  for (int it = 0; it < (nblk + nh - 1) / nh; ++it) {
    const int sb = (it * nh + h) * P::L;  // past the last block: every s >= nslot, nothing is written
#pragma unroll
    for (int ia = 0; ia < P::IA; ++ia) {
      const int t = tt + ia * kThreads;
      if (t < P::TA) {
        const int n2 = t / P::L, l = t - n2 * P::L, s = sb + l;
        int c0s = 0, gylo = 0, ncs = 0;
        if (s < g.nslot) {
          c0s = g.slot_col0[s];
          gylo = g.slot_gylo[s];
          ncs = g.slot_ncol[s];
        }
        cx<float> v[P::N1];
#pragma unroll
        for (int n1 = 0; n1 < P::N1; ++n1) {
          const int off = freq_split<N, P::N2>(n2, n1) - gylo;
          v[n1] = in_range(off, ncs) ? zrow[c0s + off] : mk<float>(0, 0);
        }
        fs_step_a<1, float, P::N1, P::N2, P::N2, PR>(v, n2, twy, X + l * P::LS);
      }
    }
    __syncthreads();
#pragma unroll
    for (int ib = 0; ib < P::IB; ++ib) {
      const int t = tt + ib * kThreads;
      if (t < P::TB) {
        const int k1 = t / P::L, l = t - k1 * P::L, s = sb + l;
        cx<float> w[P::N2];
        fs_step_b<1, float, P::N1, P::N2>(X + l * P::LS, k1, w);
        if (s < g.nslot) {
          cx<float>* pl = Pl + (size_t)s * P::LS;
#pragma unroll
          for (int k2 = 0; k2 < P::N2; ++k2) pl[k1 + P::N1 * k2] = w[k2];
        }
      }
    }
    __syncthreads();
  }
}

// step A of the inverse x-transform of rows y0 .. y0+L-1: the slots of row y from Pl
template <int N, bool PR = false>
__device__ __forceinline__ void plane_xrow_a(const GeoDev& g, const cx<float>* Pl, int y0, const cx<float>* twx,
                                             cx<float>* X, int tt = threadIdx.x) {
  using P = FS<float, N>;
#pragma unroll
  for (int ia = 0; ia < P::IA; ++ia) {
    const int t = tt + ia * kThreads;
    if (t < P::TA) {
      const int l = t / P::N2, n2 = t - l * P::N2, y = y0 + l;
      cx<float> v[P::N1];
#pragma unroll
      for (int n1 = 0; n1 < P::N1; ++n1) {
        const int s = freq_split<N, P::N2>(n2, n1) - g.gxlo;
        v[n1] = (y < N && in_range(s, g.nslot)) ? Pl[(size_t)s * P::LS + y] : mk<float>(0, 0);
      }
      fs_step_a<1, float, P::N1, P::N2, P::XP, PR>(v, n2, twx, X + l * P::XS);
    }
  }
}

// CTA (z, pair): vpsi's y-inverse, x-inverse, x V(r), x-forward and y-forward of
// one z-plane, zbuf row in place
template <int N, bool PRX, bool PRY>
__global__ void __launch_bounds__(kThreads, 2) k_plane_vx_fs(GeoDev g, cx<float>* __restrict__ zbuf,
                                                            const float* __restrict__ vpot,
                                                            const cx<float>* __restrict__ twAyg,
                                                            const cx<float>* __restrict__ twAxg,
                                                            const cx<float>* __restrict__ twBxg) {
  using P = FS<float, N>;
  using PL = PlaneLayout<N>;
  static_assert(P::IB == 1, "x rows: one step-B task per thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<float>* twy = reinterpret_cast<cx<float>*>(smem_raw);
  cx<float>* twx = twy + N;
  cx<float>* twbx = twx + N;
  cx<float>* X = twbx + N;
  cx<float>* Pl = X + PL::XEL;
  const int z = blockIdx.x, pair = blockIdx.y;
  cx<float>* zrow = zbuf + ((size_t)pair * g.n3 + z) * g.ncol;
  // the plane's sphere columns (one contiguous run of zbuf) copied in with cp.async
  // into the end of Pl, which no y-inverse block writes before the last one has
  // read them; the y-inverse then reads shared memory instead of scattered HBM
  // lines.  Where the plane leaves no such room, it reads zbuf directly.
  const int nblk = (g.nslot + P::L - 1) / P::L;
  const int zs_off = g.nslot * P::LS - g.ncol;
  const bool stage = zs_off >= (nblk - 1) * P::L * P::LS;  // the same in every thread
  const cx<float>* zsrc = zrow;
  if (stage) {
    cx<float>* zs = Pl + zs_off;
    for (int e = threadIdx.x; e < g.ncol; e += kThreads) cp_async_cx(zs + e, zrow + e);
    cp_async_commit();
    zsrc = zs;
  }
  load_table(twy, twAyg, N);
  load_table(twx, twAxg, N);
  load_table(twbx, twBxg, N);
  if (stage) cp_async_wait<0>();
  __syncthreads();
  plane_yinv<N, PRY>(g, zsrc, twy, Pl, X);
  for (int y0 = 0; y0 < N; y0 += P::L) {
    // this thread's V(r) values of step B, loaded before step A so that their
    // latency passes during it
    float vr[P::N2];
    {
      const int t = threadIdx.x;
      const int l = t / P::N1, k1 = t - l * P::N1, y = y0 + l;
      const float* vrow = vpot + (size_t)g.k1 * ((y < N ? y : 0) + (size_t)g.k2 * z);
#pragma unroll
      for (int k2 = 0; k2 < P::N2; ++k2) vr[k2] = (t < P::TB && y < N) ? __ldg(vrow + k1 + P::N1 * k2) : 0.f;
    }
    plane_xrow_a<N, PRX>(g, Pl, y0, twx, X);
    __syncthreads();
    // step B: inverse over k2, x V(r), forward over k2, twiddle, back into row k1
    if (threadIdx.x < P::TB) {
      const int t = threadIdx.x;
      const int l = t / P::N1, k1 = t - l * P::N1;
      cx<float> w[P::N2];
      fs_step_b<1, float, P::N1, P::N2, P::XP>(X + l * P::XS, k1, w);
#pragma unroll
      for (int k2 = 0; k2 < P::N2; ++k2) w[k2] = scl(w[k2], vr[k2]);
      dftn<-1, P::N2>(w);
      cx<float>* line = X + l * P::XS;
#pragma unroll
      for (int j = 0; j < P::N2; ++j) {
        cx<float> r = w[j];
        if (j > 0 && k1 > 0) r = cmulc(r, twbx[j * P::N1 + k1]);
        line[k1 * P::XP + j] = r;
      }
    }
    __syncthreads();
    // forward over N1; the sphere's x range back into the plane (rows y0.. only)
#pragma unroll
    for (int ia = 0; ia < P::IA; ++ia) {
      const int t = threadIdx.x + ia * kThreads;
      if (t < P::TA) {
        const int l = t / P::N2, j = t - l * P::N2, y = y0 + l;
        const cx<float>* line = X + l * P::XS;
        cx<float> u[P::N1];
#pragma unroll
        for (int k1 = 0; k1 < P::N1; ++k1) u[k1] = line[k1 * P::XP + j];
        dftn<-1, P::N1>(u);
        if (y < N) {
#pragma unroll
          for (int j2 = 0; j2 < P::N1; ++j2) {
            // PRX: outputs 2 .. 5 lie outside the sphere's x range (and go unused)
            if (!(PRX && P::N1 == 8 && j2 >= 2 && j2 <= 5)) {
              const int s = freq_split<N, P::N2>(j, j2) - g.gxlo;
              if (in_range(s, g.nslot)) Pl[(size_t)s * P::LS + y] = u[j2];
            }
          }
        }
      }
    }
    __syncthreads();
  }
  // forward y-transforms of the slot lines; keep the sphere columns.  The columns
  // are gathered in the start of Pl, whose first block of slot lines step A has
  // consumed before the first step B writes there (ncol <= L LS), then written to
  // zbuf as one contiguous run; otherwise straight to zbuf.
  const bool ostage = g.ncol <= P::L * P::LS;  // the same in every thread
  cx<float>* zdst = ostage ? Pl : zrow;
  for (int sb = 0; sb < g.nslot; sb += P::L) {
#pragma unroll
    for (int ia = 0; ia < P::IA; ++ia) {
      const int t = threadIdx.x + ia * kThreads;
      if (t < P::TA) {
        const int n2 = t / P::L, l = t - n2 * P::L, s = sb + l;
        cx<float> v[P::N1];
#pragma unroll
        for (int n1 = 0; n1 < P::N1; ++n1)
          v[n1] = (s < g.nslot) ? Pl[(size_t)s * P::LS + n2 + P::N2 * n1] : mk<float>(0, 0);
        fs_step_a<-1, float, P::N1, P::N2>(v, n2, twy, X + l * P::LS);
      }
    }
    __syncthreads();
#pragma unroll
    for (int ib = 0; ib < P::IB; ++ib) {
      const int t = threadIdx.x + ib * kThreads;
      if (t < P::TB) {
        const int k1 = t / P::L, l = t - k1 * P::L, s = sb + l;
        cx<float> w[P::N2];
        fs_step_b<-1, float, P::N1, P::N2>(X + l * P::LS, k1, w);
        if (s < g.nslot) {
          const int c0s = g.slot_col0[s], gylo = g.slot_gylo[s], ncs = g.slot_ncol[s];
#pragma unroll
          for (int k2 = 0; k2 < P::N2; ++k2) {
            const int off = freq_split<N, P::N1>(k1, k2) - gylo;
            if (in_range(off, ncs)) zdst[c0s + off] = w[k2];
          }
        }
      }
    }
    __syncthreads();
  }
  if (ostage)
    for (int e = threadIdx.x; e < g.ncol; e += kThreads) zrow[e] = Pl[e];
}

// CTA (chunk, z): rhoofr's y-inverse and x-inverse of plane z for the pairs
// [chunk*pchunk, ..).  Two groups of kThreads threads share the plane, each with
// its own exchange tile: the slot-line blocks and the x-row blocks alternate
// between them, so every barrier covers two blocks' work and twice the warps are
// resident.  The density of the plane builds up in registers (the x-stage map of
// k_xrho_fs; row blocks b = h, h + 2, ... of group h).  One chunk: added to rho
// directly; several: partial planes, and the last CTA of the plane to finish
// (ticket counter) adds them in chunk order, so rho does not depend on the order
// the CTAs run in.
constexpr int kPlaneRhoThreads = 2 * kThreads;
template <int N>
__global__ void __launch_bounds__(kPlaneRhoThreads, 1) k_plane_rho_fs(GeoDev g, const cx<float>* __restrict__ zbuf,
                                                                     int npairs, int s0, int nstate,
                                                                     const double* __restrict__ f, double inv_omega,
                                                                     double* __restrict__ rho,
                                                                     const cx<float>* __restrict__ twAyg,
                                                                     const cx<float>* __restrict__ twAxg, int pchunk,
                                                                     float* __restrict__ part,
                                                                     unsigned* __restrict__ tickets) {
  using P = FS<float, N>;
  using PL = PlaneLayout<N>;
  constexpr int NB = PL::NB;
  constexpr int NBH = (NB + 1) / 2;  // row blocks of one group
  static_assert(P::IB == 1, "density rows: one step-B task per thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<float>* twy = reinterpret_cast<cx<float>*>(smem_raw);
  cx<float>* twx = twy + N;
  const int h = threadIdx.x / kThreads, tt = threadIdx.x - h * kThreads;
  cx<float>* X = twx + N + h * PL::XEL;
  cx<float>* Pl = twx + N + 2 * PL::XEL;
  __shared__ float fw[2 * kMaxBatch];
  __shared__ int last_sh;
  const int nchunk = gridDim.x, chunk = blockIdx.x, z = blockIdx.y;
  const int p0 = chunk * pchunk, p1 = min(npairs, p0 + pchunk);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    twy[i] = twAyg[i];
    twx[i] = twAxg[i];
  }
  for (int i = threadIdx.x; i < 2 * (p1 - p0); i += blockDim.x) {
    const int is = s0 + 2 * p0 + i;
    fw[i] = d2f_int(is < nstate ? f[is] * inv_omega : 0.0);
  }
  __syncthreads();
  const int lb = tt / P::N1, k1 = tt - lb * P::N1;
  float acc[NBH][P::N2];
#pragma unroll
  for (int b = 0; b < NBH; ++b)
#pragma unroll
    for (int k2 = 0; k2 < P::N2; ++k2) acc[b][k2] = 0.f;
  for (int pair = p0; pair < p1; ++pair) {
    plane_yinv<N>(g, zbuf + ((size_t)pair * g.n3 + z) * g.ncol, twy, Pl, X, tt, h, 2);
    const float f1 = fw[2 * (pair - p0)], f2 = fw[2 * (pair - p0) + 1];
#pragma unroll
    for (int bh = 0; bh < NBH; ++bh) {
      const int b = 2 * bh + h;  // this group's row block (past the last one: rows >= N, zeros)
      plane_xrow_a<N>(g, Pl, b * P::L, twx, X, tt);
      __syncthreads();
      if (tt < P::TB) {
        cx<float> w[P::N2];
        fs_step_b<1, float, P::N1, P::N2, P::XP>(X + lb * P::XS, k1, w);
#pragma unroll
        for (int k2 = 0; k2 < P::N2; ++k2) acc[bh][k2] += f1 * w[k2].x * w[k2].x + f2 * w[k2].y * w[k2].y;
      }
      __syncthreads();
    }
  }
  if (nchunk == 1) {
    if (tt < P::TB) {
#pragma unroll
      for (int bh = 0; bh < NBH; ++bh) {
        const int y = (2 * bh + h) * P::L + lb;
        if (y < N) {
          double* rrow = rho + (size_t)g.k1 * (y + (size_t)g.k2 * z);
#pragma unroll
          for (int k2 = 0; k2 < P::N2; ++k2) rrow[k1 + P::N1 * k2] += f2d_int(acc[bh][k2]);
        }
      }
    }
    return;
  }
  constexpr int TILE = 2 * NBH * P::TB * P::N2;
  float* mine = part + ((size_t)z * nchunk + chunk) * TILE;
  if (tt < P::TB) {
#pragma unroll
    for (int bh = 0; bh < NBH; ++bh)
#pragma unroll
      for (int k2 = 0; k2 < P::N2; ++k2) mine[((h * NBH + bh) * P::N2 + k2) * P::TB + tt] = acc[bh][k2];
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last_sh = (atomicAdd(&tickets[z], 1u) == (unsigned)(nchunk - 1));
  __syncthreads();
  if (!last_sh) return;
  __threadfence();
  if (tt < P::TB) {
    const float* tp = part + (size_t)z * nchunk * TILE;
#pragma unroll
    for (int bh = 0; bh < NBH; ++bh) {
      const int y = (2 * bh + h) * P::L + lb;
      if (y >= N) continue;
      double* rrow = rho + (size_t)g.k1 * (y + (size_t)g.k2 * z);
#pragma unroll
      for (int k2 = 0; k2 < P::N2; ++k2) {
        double sum = 0.0;
        for (int q = 0; q < nchunk; ++q)
          sum += f2d_int(__ldcg(tp + (size_t)q * TILE + ((h * NBH + bh) * P::N2 + k2) * P::TB + tt));
        rrow[k1 + P::N1 * k2] += sum;
      }
    }
  }
  if (threadIdx.x == 0) tickets[z] = 0u;  // ready for the next launch
}

}  // namespace band
}  // namespace gbcp
