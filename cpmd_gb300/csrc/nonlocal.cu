// Non-local projector contractions (FP64 path): rnlsm1 and fnonloc.
//
// rnlsm1 (rnlsm1_utils.mod.F90:83-167): for every projector iv and atom ia
//   scr(G) = (-i)^l twnl(G,iv) eigr(G,ia), G=0 halved,
//   fnl(ia,iv,i) = 2 sum_{real view} scr * c0(:,i)       (dgemm 'T','N')
// fnonloc (fnonloc_utils.mod.F90:306-354): for every projector iv
//   auxc(G,i) = sum_ia eigr(G,ia) fnl(ia,iv,i)            (dgemm 'N','N')
//   c2(G,i) += twnl(G,iv) (-i)^l (-f_i wsg(iv)) auxc(G,i)
//
// GB300 form: all projectors of the species in ONE GEMM each (the reference
// builds scr per (iv) and calls dgemm per projector).
//  * FP64 (the drop-in): SIMT FP64 GEMMs with the (-i)^l twnl eigr operand
//    generated tile by tile in shared memory; rnlsm1 is a split-K reduction
//    over G, fnonloc accumulates straight into c2.
//  * mixed precision: the operands are converted to FP32 and split into three
//    bf16 slices (x = x0 + x1 + x2) in HBM, K-major, and the product runs on the
//    tcgen05 tensor cores through TMA (tc_gemm.cu) as the six slice pairs
//    s + t <= 2 accumulated in FP32 -- the accuracy of an FP32 GEMM.
//      rnlsm1:  fnl (P x n) = 2 scr^T c over K = 2 ngw real rows, split-K
//               partials folded in FP64;
//      fnonloc: c2 (2 ngw x n, real view) += Y Z over K = P projectors,
//               Y = (-i)^l twnl eigr, Z = -f wsg fnl, FP64 read-modify-write.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.h"
#include "tc_gemm.h"

namespace gbcp {

namespace {

constexpr int TS = 64;
constexpr int BK = 16;
constexpr int NT = 256;
constexpr int kMaxProj = 64;

struct ProjInfo {
  int nat, ngh;
  // the caller's fnl / dfnl layout: fnl(ia, iv, i) at ia + lda (iv + ldp i), dfnl(ia, iv, k, i)
  // at ia + lda (iv + ldp (k + 3 i)) -- the reference's global fnl(imagp, ions1%nat, nhxs, n)
  // seen from a species block fnl(1, isa0+1, 1, 1) (rnlsm1_utils.mod.F90:156-165)
  int lda, ldp;
  int lmod4[kMaxProj];  // angular momentum mod 4 per projector
  // rnlsm2 (dfnl = d fnl / d R): rows p = ia + nat (iv + ngh k) for the three directions k,
  // operand (-i)^(l+1) twnl eigr tpiba G_k (rnlsm2_utils.mod.F90:190-240)
  int deriv;
  const short4* gm;     // Miller indices of the sphere (deriv only)
  double tpiba;
};

// offset of row p = ia + nat (iv + ngh k) of state i in the caller's fnl (kdim 1) or dfnl (kdim 3)
__device__ __forceinline__ size_t fnl_at(const ProjInfo& pi, size_t p, size_t i, int kdim) {
  const size_t ia = p % pi.nat, q = p / pi.nat;
  const size_t iv = q % pi.ngh, k = q / pi.ngh;
  return ia + (size_t)pi.lda * (iv + (size_t)pi.ldp * (k + (size_t)kdim * i));
}

// (-i)^l * z
__device__ __forceinline__ cx<double> phase_l(int l, cx<double> z) {
  switch (l & 3) {
    case 0: return z;
    case 1: return mk<double>(z.y, -z.x);
    case 2: return mk<double>(-z.x, -z.y);
    default: return mk<double>(-z.y, z.x);
  }
}

// projector operand row p at sphere index G: (-i)^l eigr times the real factor t = twnl,
// or for rnlsm2 (-i)^(l+1) eigr times t = twnl tpiba G_k
__device__ __forceinline__ cx<double> proj_operand(const ProjInfo& pi, const double* __restrict__ twnl,
                                                   const cx<double>* __restrict__ eigr, int ngw, int p, int G,
                                                   double& t) {
  const int ia = p % pi.nat, iv = (p / pi.nat) % pi.ngh;
  t = twnl[(size_t)iv * ngw + G];
  int l = pi.lmod4[iv];
  if (pi.deriv) {
    const int kd = p / (pi.nat * pi.ngh);
    const short4 m = pi.gm[G];
    t *= pi.tpiba * (double)(kd == 0 ? m.x : kd == 1 ? m.y : m.z);
    l += 1;
  }
  return phase_l(l, eigr[(size_t)ia * ngw + G]);
}


// fnl partials: part[split][p][i], p = ia + nat*iv, K over real view 2*ngw
__global__ void __launch_bounds__(NT) k_rnlsm1_part(const double* __restrict__ c0r, int ldr, int ngw, int nstate,
                                                    ProjInfo pi, const double* __restrict__ twnl,
                                                    const cx<double>* __restrict__ eigr, int geq0, int kchunk,
                                                    double* __restrict__ part) {
  __shared__ double As[BK][TS + 1];
  __shared__ double Bs[BK][TS + 1];
  const int P = pi.nat * pi.ngh * (pi.deriv ? 3 : 1);
  const int p0 = blockIdx.x * TS, i0 = blockIdx.y * TS, split = blockIdx.z;
  const int K = 2 * ngw;
  const int k0 = split * kchunk, k1 = min(K, k0 + kchunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int kb = k0; kb < k1; kb += BK) {
    for (int q = 0; q < 4; ++q) {
      const int kk = threadIdx.x % 16, cc = threadIdx.x / 16 + 16 * q;
      const int k = kb + kk;
      // projector operand (generated)
      double av = 0.0;
      const int p = p0 + cc;
      if (k < k1 && p < P) {
        const int G = k >> 1;
        double t;
        const cx<double> s = proj_operand(pi, twnl, eigr, ngw, p, G, t);
        if (geq0 && G == 0) t *= 0.5;
        av = t * ((k & 1) ? s.y : s.x);
      }
      As[kk][cc] = av;
      const int i = i0 + cc;
      Bs[kk][cc] = (k < k1 && i < nstate) ? c0r[k + (size_t)i * ldr] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][ty + 16 * u];
        b[u] = Bs[kk][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
  double* out = part + (size_t)split * P * nstate;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int p = p0 + ty + 16 * u, i = i0 + tx + 16 * v;
      if (p < P && i < nstate) out[p + (size_t)P * i] = acc[u][v];
    }
}

// partials part[split][p + P i] folded in split order into the caller's layout
__global__ void k_rnlsm1_fold(const double* __restrict__ part, int nsplit, size_t P, size_t n, ProjInfo pi, int kdim,
                              double* __restrict__ fnl) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += part[(size_t)p * n + e];
    fnl[fnl_at(pi, e % P, e / P, kdim)] = 2.0 * s;
  }
}

// c2 real view (rows 2*ngw) += A_r (rows x P) * B (P x n),
// A[G][p] = (-i)^l twnl(G,iv) eigr(G,ia); B[p][i] = fnl[p + P i] * (-f_i' wsg(iv))
__global__ void __launch_bounds__(NT) k_fnonloc(double* __restrict__ c2r, int ldr, int ngw, int nstate, ProjInfo pi,
                                                const double* __restrict__ twnl, const cx<double>* __restrict__ eigr,
                                                const double* __restrict__ fnl, const double* __restrict__ f,
                                                const double* __restrict__ wsg) {
  __shared__ double As[BK][TS + 1];
  __shared__ double Bs[BK][TS + 1];
  const int P = pi.nat * pi.ngh;
  const int rows = 2 * ngw;
  const int r0 = blockIdx.x * TS, i0 = blockIdx.y * TS;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int kb = 0; kb < P; kb += BK) {
    for (int q = 0; q < 4; ++q) {
      // A tile: 64 rows x 16 projectors; thread -> (row = tid % 64, k = tid / 64 + 4 q)
      const int rr = threadIdx.x % 64, kk = threadIdx.x / 64 + 4 * q;
      const int r = r0 + rr, p = kb + kk;
      double av = 0.0;
      if (r < rows && p < P) {
        const int ia = p % pi.nat, iv = p / pi.nat;
        const int G = r >> 1;
        const cx<double> s = phase_l(pi.lmod4[iv], eigr[(size_t)ia * ngw + G]);
        const double t = twnl[(size_t)iv * ngw + G];
        av = t * ((r & 1) ? s.y : s.x);
      }
      As[kk][rr] = av;
      // B tile: 16 projectors x 64 states
      const int cc = threadIdx.x % 64, kp = threadIdx.x / 64 + 4 * q;
      const int i = i0 + cc, p2 = kb + kp;
      double bv = 0.0;
      if (i < nstate && p2 < P) {
        const int iv = p2 / pi.nat;
        double ffi = f[i];
        if (ffi < 1e-5) ffi = 1.0;
        bv = fnl[fnl_at(pi, p2, i, 1)] * (-ffi * wsg[iv]);
      }
      Bs[kp][cc] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][tx + 16 * u];
        b[u] = Bs[kk][ty + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = r0 + tx + 16 * u, i = i0 + ty + 16 * v;
      if (r < rows && i < nstate) c2r[r + (size_t)i * ldr] += acc[u][v];
    }
}

bool make_info(Ctx& c, int nat, int ngh, const int* nghtol, int lda, int ldp, ProjInfo& pi) {
  if (nat <= 0 || ngh <= 0 || ngh > kMaxProj) {
    c.err = "projectors: need 0 < ngh <= 64 and nat > 0";
    return false;
  }
  pi.nat = nat;
  pi.ngh = ngh;
  pi.lda = lda > 0 ? lda : nat;
  pi.ldp = ldp > 0 ? ldp : ngh;
  if (pi.lda < nat || pi.ldp < ngh) {
    c.err = "projectors: fnl leading dimensions below nat / ngh";
    return false;
  }
  pi.deriv = 0;
  pi.gm = nullptr;
  pi.tpiba = 0.0;
  for (int i = 0; i < ngh; ++i) pi.lmod4[i] = ((nghtol[i] % 4) + 4) % 4;
  return true;
}

// ---------------------------------------------------------------- mixed precision: bf16 slices
__device__ __forceinline__ uint32_t bf16_rn(float x) {
  const uint32_t u = __float_as_uint(x);
  return (u + 0x7FFFu + ((u >> 16) & 1u)) >> 16;
}
// x = x0 + x1 + x2 (bf16 bit patterns), each the bf16 rounding of the remainder
__device__ __forceinline__ void split3(float x, uint32_t (&h)[3]) {
  h[0] = bf16_rn(x);
  float r = x - __uint_as_float(h[0] << 16);
  h[1] = bf16_rn(r);
  r = r - __uint_as_float(h[1] << 16);
  h[2] = bf16_rn(r);
}
__device__ __forceinline__ void phase_lf(int l, float& re, float& im) {
  const float x = re, y = im;
  switch (l & 3) {
    case 0: break;
    case 1: re = y; im = -x; break;
    case 2: re = -x; im = -y; break;
    default: re = -y; im = x; break;
  }
}

// rnlsm1 A operand: slice s, row p = ia + nat*iv, columns (2G, 2G+1) = scr(G) with G = 0 halved
__global__ void __launch_bounds__(256) k_nl_scr3(const double* __restrict__ twnl, const cx<double>* __restrict__ eigr,
                                                 int ngw, ProjInfo pi, int geq0, size_t kstride,
                                                 uint32_t* __restrict__ A) {
  const int G = blockIdx.x * 256 + threadIdx.x, a = blockIdx.y;
  if (G >= ngw) return;
  const size_t P = (size_t)pi.nat * pi.ngh * (pi.deriv ? 3 : 1);
  const cx<double> e = eigr[G + (size_t)ngw * a];
  const float ex = d2f_int(e.x), ey = d2f_int(e.y);
  const float half = (geq0 && G == 0) ? 0.5f : 1.0f;
  float gk[3] = {1.f, 1.f, 1.f};
  if (pi.deriv) {
    const short4 m = pi.gm[G];
    const float tp = d2f_int(pi.tpiba);
    gk[0] = tp * (float)m.x;
    gk[1] = tp * (float)m.y;
    gk[2] = tp * (float)m.z;
  }
  const int nk = pi.deriv ? 3 : 1;
  for (int iv = 0; iv < pi.ngh; ++iv) {
    const float tw0 = d2f_int(twnl[G + (size_t)ngw * iv]) * half;
    for (int kd = 0; kd < nk; ++kd) {
      const float tw = tw0 * gk[kd];
      float re = tw * ex, im = tw * ey;
      phase_lf(pi.lmod4[iv] + pi.deriv, re, im);
      uint32_t hr[3], hi[3];
      split3(re, hr);
      split3(im, hi);
      const size_t p = (size_t)a + (size_t)pi.nat * (iv + (size_t)pi.ngh * kd);
#pragma unroll
      for (int s = 0; s < 3; ++s) A[((s * P + p) * kstride) / 2 + G] = hr[s] | (hi[s] << 16);
    }
  }
}

// rnlsm1 B operand: slice s, row i, columns (2G, 2G+1) = c0(G, i)
__global__ void __launch_bounds__(256) k_nl_c3(const cx<double>* __restrict__ c0, int ldc, int ngw, int nstate,
                                               size_t kstride, uint32_t* __restrict__ B) {
  const int G = blockIdx.x * 256 + threadIdx.x, i = blockIdx.y;
  if (G >= ngw) return;
  const cx<double> v = c0[G + (size_t)ldc * i];
  uint32_t hr[3], hi[3];
  split3(d2f_int(v.x), hr);
  split3(d2f_int(v.y), hi);
#pragma unroll
  for (int s = 0; s < 3; ++s) B[(((size_t)s * nstate + i) * kstride) / 2 + G] = hr[s] | (hi[s] << 16);
}

// fnl(p, i) = 2 sum_split part[(split n + i) P + p], written in the caller's layout
__global__ void k_nl_fnl_fold(const float* __restrict__ part, int nsplit, size_t P, size_t Pn, ProjInfo pi, int kdim,
                              double* __restrict__ fnl) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < Pn; e += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nsplit; ++k) s += f2d_int(part[k * Pn + e]);
    fnl[fnl_at(pi, e % P, e / P, kdim)] = 2.0 * s;
  }
}

// fnonloc A operand: slice s, row 2G + c (c = re, im), column p = ia + nat*iv: Y(G, p)
__global__ void __launch_bounds__(256) k_nl_y3(const double* __restrict__ twnl, const cx<double>* __restrict__ eigr,
                                               int ngw, ProjInfo pi, size_t kstride, uint16_t* __restrict__ A) {
  __shared__ float2 es[32][33];
  __shared__ float tws[kMaxProj][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int G0 = blockIdx.x * 32, a0 = blockIdx.y * 32;
  for (int j = ty; j < 32; j += 8) {
    const int a = a0 + j, G = G0 + tx;
    float2 v = make_float2(0.f, 0.f);
    if (a < pi.nat && G < ngw) {
      const cx<double> e = eigr[G + (size_t)ngw * a];
      v = make_float2(d2f_int(e.x), d2f_int(e.y));
    }
    es[j][tx] = v;
  }
  for (int iv = ty; iv < pi.ngh; iv += 8) tws[iv][tx] = (G0 + tx < ngw) ? d2f_int(twnl[G0 + tx + (size_t)ngw * iv]) : 0.f;
  __syncthreads();
  const size_t rows = 2 * (size_t)ngw;
  const int a = a0 + tx;
  if (a >= pi.nat) return;
  for (int gg = ty; gg < 32; gg += 8) {
    const int G = G0 + gg;
    if (G >= ngw) break;
    const float2 e = es[tx][gg];
    for (int iv = 0; iv < pi.ngh; ++iv) {
      float re = tws[iv][gg] * e.x, im = tws[iv][gg] * e.y;
      phase_lf(pi.lmod4[iv], re, im);
      uint32_t hr[3], hi[3];
      split3(re, hr);
      split3(im, hi);
      const size_t p = (size_t)a + (size_t)pi.nat * iv;
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        A[(s * rows + 2 * (size_t)G) * kstride + p] = (uint16_t)hr[s];
        A[(s * rows + 2 * (size_t)G + 1) * kstride + p] = (uint16_t)hi[s];
      }
    }
  }
}

// fnonloc B operand: slice s, row i, column p: Z(p, i) = -f_i wsg(iv) fnl(p, i), f < 1e-5 counted as 1
__global__ void k_nl_z3(const double* __restrict__ fnl, const double* __restrict__ f, const double* __restrict__ wsg,
                        ProjInfo pi, size_t P, int nstate, size_t kstride, uint16_t* __restrict__ B) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < P * nstate; e += (size_t)gridDim.x * blockDim.x) {
    const size_t i = e / P, p = e % P;
    const int iv = (int)(p / pi.nat);
    const double fi = f[i] < 1e-5 ? 1.0 : f[i];
    uint32_t h[3];
    split3(d2f_int(-fi * wsg[iv] * fnl[fnl_at(pi, p, i, 1)]), h);
#pragma unroll
    for (int s = 0; s < 3; ++s) B[((size_t)s * nstate + i) * kstride + p] = (uint16_t)h[s];
  }
}

constexpr int kPairS[6] = {0, 0, 1, 0, 1, 2};
constexpr int kPairT[6] = {0, 1, 0, 2, 1, 0};

size_t round8(size_t x) { return (x + 7) & ~size_t(7); }

int check_status(Ctx& c) {
  int st = 0;
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(&st, c.d_info, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (st == -2) {
    c.err = "projector GEMM: tensor-core pipeline wait expired";
    return 4;
  }
  return 0;
}

int rnlsm1_tc(Ctx& c, const cx<double>* c0, int ldc, int nstate, const ProjInfo& pi, const double* twnl,
              const cx<double>* eigr, double* fnl) {
  const int P = pi.nat * pi.ngh * (pi.deriv ? 3 : 1);
  const int K = 2 * c.ngw;
  const size_t ks = round8((size_t)K);
  if (!ensure(c, c.nl_ta, 2 * 3 * ks * (size_t)P) || !ensure(c, c.nl_tb, 2 * 3 * ks * (size_t)nstate)) return 6;
  const int ksplit = tc_gemm_splits_used(P, nstate, K, tc_gemm_ksplit(P, nstate, K));
  if (!ensure(c, c.nl_tp, sizeof(float) * (size_t)ksplit * P * nstate)) return 6;
  {
    ProfScope ps_(c, "k_nl_slices");
    k_nl_scr3<<<dim3((c.ngw + 255) / 256, pi.nat), 256, 0, c.stream>>>(twnl, eigr, c.ngw, pi, c.geq0, ks,
                                                                      static_cast<uint32_t*>(c.nl_ta.p));
    GBCP_LAUNCH_CHECK(c);
    k_nl_c3<<<dim3((c.ngw + 255) / 256, nstate), 256, 0, c.stream>>>(c0, ldc, c.ngw, nstate, ks,
                                                                    static_cast<uint32_t*>(c.nl_tb.p));
    GBCP_LAUNCH_CHECK(c);
  }
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, sizeof(int), c.stream));
  int rc = tc_gemm_split3(c, static_cast<const uint16_t*>(c.nl_ta.p), P, static_cast<const uint16_t*>(c.nl_tb.p),
                          nstate, K, (int)ks, 6, kPairS, kPairT, 0, static_cast<float*>(c.nl_tp.p), ksplit, nullptr,
                          0, c.d_info);
  if (rc) return rc;
  {
    ProfScope ps_(c, "k_nl_fnl_fold");
    k_nl_fnl_fold<<<1024, 256, 0, c.stream>>>(static_cast<const float*>(c.nl_tp.p), ksplit, (size_t)P,
                                              (size_t)P * nstate, pi, pi.deriv ? 3 : 1, fnl);
    GBCP_LAUNCH_CHECK(c);
  }
  return check_status(c);
}

int fnonloc_tc(Ctx& c, cx<double>* c2, int ldc2, int nstate, const double* f, const ProjInfo& pi,
               const double* twnl, const cx<double>* eigr, const double* fnl, const double* wsg) {
  const int P = pi.nat * pi.ngh;
  const int M = 2 * c.ngw;
  const size_t ks = round8((size_t)P);
  if (!ensure(c, c.nl_ta, 2 * 3 * ks * (size_t)M) || !ensure(c, c.nl_tb, 2 * 3 * ks * (size_t)nstate)) return 6;
  {
    ProfScope ps_(c, "k_nl_slices");
    k_nl_y3<<<dim3((c.ngw + 31) / 32, (pi.nat + 31) / 32), 256, 0, c.stream>>>(twnl, eigr, c.ngw, pi, ks,
                                                                              static_cast<uint16_t*>(c.nl_ta.p));
    GBCP_LAUNCH_CHECK(c);
    k_nl_z3<<<1024, 256, 0, c.stream>>>(fnl, f, wsg, pi, (size_t)P, nstate, ks, static_cast<uint16_t*>(c.nl_tb.p));
    GBCP_LAUNCH_CHECK(c);
  }
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, sizeof(int), c.stream));
  int rc = tc_gemm_split3(c, static_cast<const uint16_t*>(c.nl_ta.p), M, static_cast<const uint16_t*>(c.nl_tb.p),
                          nstate, P, (int)ks, 6, kPairS, kPairT, 1, nullptr, 1, reinterpret_cast<double*>(c2),
                          2 * (long long)ldc2, c.d_info);
  if (rc) return rc;
  return check_status(c);
}

// projector GEMMs on the tensor cores: mixed precision unless the FP64 SIMT engine is forced
bool use_tc_projectors(const Ctx& c) { return c.precision == 1 && c.gemm_mode != 0; }

}  // namespace

namespace {

// fnl (or dfnl) = 2 scr^T c0 in FP64 on the SIMT units (split-K over G, folded in order)
int rnlsm1_simt(Ctx& c, const cx<double>* c0, int ldc, int nstate, const ProjInfo& pi, const double* twnl,
                const cx<double>* eigr, double* fnl) {
  const int P = pi.nat * pi.ngh * (pi.deriv ? 3 : 1);
  const int K = 2 * c.ngw;
  const int tiles = ((P + TS - 1) / TS) * ((nstate + TS - 1) / TS);
  int nsplit = std::max(1, std::min(512, (4 * 152 + tiles - 1) / tiles));
  int kchunk = (K + nsplit - 1) / nsplit;
  kchunk = ((kchunk + BK - 1) / BK) * BK;
  nsplit = (K + kchunk - 1) / kchunk;
  const size_t n = (size_t)P * nstate;
  if (!ensure(c, c.nl_a, sizeof(double) * n * nsplit)) return 6;
  double* part = static_cast<double*>(c.nl_a.p);
  dim3 grid((P + TS - 1) / TS, (nstate + TS - 1) / TS, nsplit);
  {
    ProfScope ps_(c, "k_rnlsm1_part");
    k_rnlsm1_part<<<grid, NT, 0, c.stream>>>(reinterpret_cast<const double*>(c0), 2 * ldc, c.ngw, nstate, pi, twnl, eigr,
                                              c.geq0, kchunk, part);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_rnlsm1_fold");
    k_rnlsm1_fold<<<512, 256, 0, c.stream>>>(part, nsplit, (size_t)P, n, pi, pi.deriv ? 3 : 1, fnl);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

}  // namespace

int nl_rnlsm1(Ctx& c, const cx<double>* c0, int ldc, int nstate, int nat, int ngh, const int* nghtol_host,
              const double* twnl, const cx<double>* eigr, double* fnl, int lda, int ldp) {
  ProjInfo pi;
  if (!make_info(c, nat, ngh, nghtol_host, lda, ldp, pi)) return 1;
  if (use_tc_projectors(c)) return rnlsm1_tc(c, c0, ldc, nstate, pi, twnl, eigr, fnl);
  return rnlsm1_simt(c, c0, ldc, nstate, pi, twnl, eigr, fnl);
}

namespace {

// fion(k, ia) -= sum_i sum_iv 2 wsg(iv) f_i dfnl(ia,iv,k,i) fnl(ia,iv,i), states with |f| > 1e-12
// (rnlfor_utils.mod.F90:283-330, KB branch); one CTA per atom, fixed-order reduction
__global__ void __launch_bounds__(256) k_rnlfor(int nstate, const double* __restrict__ f, int nat, int ngh,
                                                int lda, int ldp, const double* __restrict__ wsg,
                                                const double* __restrict__ fnl, const double* __restrict__ dfnl,
                                                double* __restrict__ fion) {
  const int ia = blockIdx.x;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int t = threadIdx.x; t < nstate * ngh; t += blockDim.x) {
    const int i = t / ngh, iv = t - i * ngh;
    const double w = f[i];
    if (!(fabs(w) > 1e-12)) continue;
    const double a = 2.0 * wsg[iv] * w * fnl[(size_t)ia + (size_t)lda * (iv + (size_t)ldp * i)];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      acc[k] = fma(a, dfnl[(size_t)ia + (size_t)lda * (iv + (size_t)ldp * (k + 3 * (size_t)i))], acc[k]);
  }
  __shared__ double red[3][256];
#pragma unroll
  for (int k = 0; k < 3; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
#pragma unroll
      for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 3) fion[3 * (size_t)ia + threadIdx.x] -= red[threadIdx.x][0];
}

}  // namespace

int nl_rnlsm2(Ctx& c, const cx<double>* c0, int ldc, int nstate, int nat, int ngh, const int* nghtol_host,
              const double* twnl, const cx<double>* eigr, double* dfnl, int lda, int ldp) {
  ProjInfo pi;
  if (!make_info(c, nat, ngh, nghtol_host, lda, ldp, pi)) return 1;
  pi.deriv = 1;
  pi.gm = c.wmill;
  pi.tpiba = std::sqrt(c.tpiba2);
  if (use_tc_projectors(c)) return rnlsm1_tc(c, c0, ldc, nstate, pi, twnl, eigr, dfnl);
  return rnlsm1_simt(c, c0, ldc, nstate, pi, twnl, eigr, dfnl);
}

int nl_rnlfor(Ctx& c, int nstate, const double* f, int nat, int ngh, const double* wsg, const double* fnl,
              const double* dfnl, double* fion, int lda, int ldp) {
  lda = lda > 0 ? lda : nat;
  ldp = ldp > 0 ? ldp : ngh;
  if (nat <= 0 || ngh <= 0 || nstate <= 0 || lda < nat || ldp < ngh) {
    c.err = "rnlfor: bad sizes or fnl leading dimensions";
    return 1;
  }
  ProfScope ps_(c, "k_rnlfor");
  k_rnlfor<<<nat, 256, 0, c.stream>>>(nstate, f, nat, ngh, lda, ldp, wsg, fnl, dfnl, fion);
  GBCP_LAUNCH_CHECK(c);
  return 0;
}

int nl_fnonloc(Ctx& c, cx<double>* c2, int ldc2, int nstate, const double* f, int nat, int ngh, const int* nghtol_host,
               const double* twnl, const cx<double>* eigr, const double* fnl, const double* wsg, int lda, int ldp) {
  ProjInfo pi;
  if (!make_info(c, nat, ngh, nghtol_host, lda, ldp, pi)) return 1;
  if (use_tc_projectors(c)) return fnonloc_tc(c, c2, ldc2, nstate, f, pi, twnl, eigr, fnl, wsg);
  const int rows = 2 * c.ngw;
  dim3 grid((rows + TS - 1) / TS, (nstate + TS - 1) / TS);
  {
    ProfScope ps_(c, "k_fnonloc");
    k_fnonloc<<<grid, NT, 0, c.stream>>>(reinterpret_cast<double*>(c2), 2 * ldc2, c.ngw, nstate, pi, twnl, eigr, fnl, f,
                                         wsg);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

}  // namespace gbcp
