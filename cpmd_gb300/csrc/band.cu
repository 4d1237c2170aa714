// Band-loop dispatch (precision) plus the dense 3D FFT (invfftn/fwfftn) and
// the FP64 reductions of rhoofr (kinetic energy, charge sums).
//
// The pruned band-loop kernels themselves live in band_impl.cuh, instantiated
// once per precision in band64.cu and band32.cu.
#include <algorithm>
#include <cmath>

#include "ctx.h"

namespace gbcp {

int band_rhoofr_fp64(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho,
                     double* kpart);
int band_vpsi_fp64(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f,
                   const double* vpot, int nstate);
int band_rhoofr_fp32(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho,
                     double* kpart);
int band_zinv_blocks_fp64(const Ctx& c);
int band_zinv_blocks_fp32(const Ctx& c);
int band_vpsi_fp32(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f,
                   const double* vpot, int nstate);

namespace {

constexpr int kThreads = 256;

__host__ __device__ inline int line_stride(int n) { return (n % 2 == 0) ? n + 1 : n; }

template <typename T>
__device__ __forceinline__ void load_tw(cx<T>* tw, const cx<T>* __restrict__ twg, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = twg[i];
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

// dot-product partials of two real arrays
__global__ void k_dot_partial(const double* __restrict__ x, const double* __restrict__ y, size_t n,
                              double* __restrict__ part) {
  double a = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a += x[i] * y[i];
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

// out = scale * sum_i part[2 i] (one CTA, deterministic order)
__global__ void k_fold_scaled(const double* __restrict__ part, int n, double scale, double* __restrict__ out) {
  __shared__ double r[kThreads];
  double a = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a += part[2 * i];
  r[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) r[threadIdx.x] += r[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = scale * r[0];
}

// First fold level of rhoofr's scalars: CTA b sums the 2-component partials
// [b*chunk, (b+1)*chunk) in index order into out[2b], out[2b+1].
__global__ void k_fold2_ranges(const double* __restrict__ part, int n, int chunk, double* __restrict__ out) {
  __shared__ double r0[kThreads], r1[kThreads];
  const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  double a = 0.0, b = 0.0;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
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
    out[2 * blockIdx.x] = r0[0];
    out[2 * blockIdx.x + 1] = r1[0];
  }
}

// Last level: out = {tpiba2 * sum kin, sum norm, rscale * sum rho} from nk
// 2-component kinetic/norm partials and nr density partials (k_sum_partial).
__global__ void k_rho_scalars(const double* __restrict__ kp, int nk, const double* __restrict__ rp, int nr,
                              double tpiba2, double rscale, double* __restrict__ out) {
  __shared__ double r0[kThreads], r1[kThreads], r2[kThreads];
  double a = 0.0, b = 0.0, d = 0.0;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    a += kp[2 * i];
    b += kp[2 * i + 1];
  }
  for (int i = threadIdx.x; i < nr; i += blockDim.x) d += rp[2 * i];
  r0[threadIdx.x] = a;
  r1[threadIdx.x] = b;
  r2[threadIdx.x] = d;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      r0[threadIdx.x] += r0[threadIdx.x + s];
      r1[threadIdx.x] += r1[threadIdx.x + s];
      r2[threadIdx.x] += r2[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = tpiba2 * r0[0];
    out[1] = r1[0];
    out[2] = rscale * r2[0];
  }
}

}  // namespace
static int lines_for(int n, int target) { return std::max(1, std::min(64, target / n)); }

template <typename T> static size_t stage_smem(int n, int nl) {
  return sizeof(cx<T>) * ((size_t)n + 2 * (size_t)nl * line_stride(n));
}


int band_rhoofr(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho,
                double* scalars) {
  const size_t nnr = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  GBCP_CUDA_TRY(c, cudaMemsetAsync(rho, 0, sizeof(double) * nnr, c.stream));
  if (nstate <= 0) {
    if (scalars) GBCP_CUDA_TRY(c, cudaMemsetAsync(scalars, 0, 3 * sizeof(double), c.stream));
    return 0;
  }
  // partials of E_kin / norm: one pair of doubles per Z-stage CTA of every pair,
  // then one per first-level fold CTA, then the density sum's partials
  const int npairs = (nstate + 1) / 2;
  const int nkb = npairs * (c.precision == 0 ? band_zinv_blocks_fp64(c) : band_zinv_blocks_fp32(c));
  const int kchunk = 4096, nk1 = (nkb + kchunk - 1) / kchunk, nrp = 296;
  double* kpart = nullptr;
  if (scalars) {
    if (!ensure(c, c.red, sizeof(double) * 2 * ((size_t)nkb + nk1 + nrp))) return 6;
    kpart = static_cast<double*>(c.red.p);
  }
  const int rc = c.precision == 0 ? band_rhoofr_fp64(c, c0, ldc, nstate, f, rho, kpart)
                                  : band_rhoofr_fp32(c, c0, ldc, nstate, f, rho, kpart);
  if (rc || !scalars) return rc;
  double* k1 = kpart + 2 * (size_t)nkb;
  double* rp = k1 + 2 * (size_t)nk1;
  {
    ProfScope ps_(c, "k_fold2_ranges");
    k_fold2_ranges<<<nk1, kThreads, 0, c.stream>>>(kpart, nkb, kchunk, k1);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_sum_partial");
    k_sum_partial<<<nrp, kThreads, 0, c.stream>>>(rho, nnr, rp);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_rho_scalars");
    k_rho_scalars<<<1, kThreads, 0, c.stream>>>(k1, nk1, rp, nrp, c.tpiba2,
                                                c.omega / ((double)c.nr[0] * c.nr[1] * c.nr[2]), scalars);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

int band_vpsi(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f, const double* vpot,
              int nstate) {
  if (nstate <= 0) return 0;
  return c.precision == 0 ? band_vpsi_fp64(c, c0, ldc, c2, ldc2, f, vpot, nstate)
                          : band_vpsi_fp32(c, c0, ldc, c2, ldc2, f, vpot, nstate);
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

int kin_energy_async(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* dev_out) {
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
    ProfScope ps_(c, "k_fold_scaled");
    k_fold_scaled<<<1, kThreads, 0, c.stream>>>(part, nb, c.tpiba2, dev_out);
    GBCP_LAUNCH_CHECK(c);
  }
  return 0;
}

int vrho_async(Ctx& c, const double* rho, const double* vpot, double* dev_out) {
  const size_t n = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  const int nb = 296;
  if (!ensure(c, c.red2, sizeof(double) * (2 * (size_t)nb + 2))) return 6;
  double* part = static_cast<double*>(c.red2.p);
  {
    ProfScope ps_(c, "k_dot_partial");
    k_dot_partial<<<nb, kThreads, 0, c.stream>>>(rho, vpot, n, part);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_fold_scaled");
    k_fold_scaled<<<1, kThreads, 0, c.stream>>>(part, nb, c.omega / ((double)c.nr[0] * c.nr[1] * c.nr[2]), dev_out);
    GBCP_LAUNCH_CHECK(c);
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
