// Non-local projector contractions (FP64 path): rnlsm1 and fnonloc.
//
// rnlsm1 (rnlsm1_utils.mod.F90:83-167): for every projector iv and atom ia
//   scr(G) = (-i)^l twnl(G,iv) eigr(G,ia), G=0 halved,
//   fnl(ia,iv,i) = 2 sum_{real view} scr * c0(:,i)       (dgemm 'T','N')
// fnonloc (fnonloc_utils.mod.F90:306-354): for every projector iv
//   auxc(G,i) = sum_ia eigr(G,ia) fnl(ia,iv,i)            (dgemm 'N','N')
//   c2(G,i) += twnl(G,iv) (-i)^l (-f_i wsg(iv)) auxc(G,i)
//
// GB300 form: all projectors of the species in ONE GEMM each, with the
// (-i)^l twnl eigr operand generated tile by tile in shared memory instead of
// being materialised (the reference builds scr per (iv) and calls dgemm per
// projector).  rnlsm1 is a split-K reduction over G; fnonloc accumulates
// straight into c2.
#include <algorithm>
#include <vector>

#include "ctx.h"

namespace gbcp {

namespace {

constexpr int TS = 64;
constexpr int BK = 16;
constexpr int NT = 256;
constexpr int kMaxProj = 64;

struct ProjInfo {
  int nat, ngh;
  int lmod4[kMaxProj];  // angular momentum mod 4 per projector
};

// (-i)^l * z
__device__ __forceinline__ cx<double> phase_l(int l, cx<double> z) {
  switch (l & 3) {
    case 0: return z;
    case 1: return mk<double>(z.y, -z.x);
    case 2: return mk<double>(-z.x, -z.y);
    default: return mk<double>(-z.y, z.x);
  }
}

// fnl partials: part[split][p][i], p = ia + nat*iv, K over real view 2*ngw
__global__ void __launch_bounds__(NT) k_rnlsm1_part(const double* __restrict__ c0r, int ldr, int ngw, int nstate,
                                                    ProjInfo pi, const double* __restrict__ twnl,
                                                    const cx<double>* __restrict__ eigr, int geq0, int kchunk,
                                                    double* __restrict__ part) {
  __shared__ double As[BK][TS + 1];
  __shared__ double Bs[BK][TS + 1];
  const int P = pi.nat * pi.ngh;
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
        const int ia = p % pi.nat, iv = p / pi.nat;
        const int G = k >> 1;
        cx<double> s = phase_l(pi.lmod4[iv], eigr[(size_t)ia * ngw + G]);
        double t = twnl[(size_t)iv * ngw + G];
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

__global__ void k_rnlsm1_fold(const double* __restrict__ part, int nsplit, size_t n, double* __restrict__ fnl) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += part[(size_t)p * n + e];
    fnl[e] = 2.0 * s;
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
        bv = fnl[p2 + (size_t)P * i] * (-ffi * wsg[iv]);
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

bool make_info(Ctx& c, int nat, int ngh, const int* nghtol, ProjInfo& pi) {
  if (nat <= 0 || ngh <= 0 || ngh > kMaxProj) {
    c.err = "projectors: need 0 < ngh <= 64 and nat > 0";
    return false;
  }
  pi.nat = nat;
  pi.ngh = ngh;
  for (int i = 0; i < ngh; ++i) pi.lmod4[i] = ((nghtol[i] % 4) + 4) % 4;
  return true;
}

}  // namespace

int nl_rnlsm1(Ctx& c, const cx<double>* c0, int ldc, int nstate, int nat, int ngh, const int* nghtol_host,
              const double* twnl, const cx<double>* eigr, double* fnl) {
  ProjInfo pi;
  if (!make_info(c, nat, ngh, nghtol_host, pi)) return 1;
  const int P = nat * ngh;
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
    k_rnlsm1_fold<<<512, 256, 0, c.stream>>>(part, nsplit, n, fnl);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

int nl_fnonloc(Ctx& c, cx<double>* c2, int ldc2, int nstate, const double* f, int nat, int ngh, const int* nghtol_host,
               const double* twnl, const cx<double>* eigr, const double* fnl, const double* wsg) {
  ProjInfo pi;
  if (!make_info(c, nat, ngh, nghtol_host, pi)) return 1;
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
