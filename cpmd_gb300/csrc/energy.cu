// Energy functional of the local-potential Kohn-Sham model and its adjoint.
//
//   E[psi, V, R] = E_kin + E_loc + E_H + E_xc + E_ext
//
//   rho(r)   = sum_i f_i/Omega psi_i(r)^2            band loop (rhoofr)
//   rho(G)   = fwfftn(rho)                           vofrhoa_utils.mod.F90:90-96
//   V_ion(G) = sum_a vps(G, sp_a) e^{-iG.R_a}        eicalc_utils.mod.F90:33-173,
//              (e^{-iG.R} from per-axis tables ei1*ei2*ei3, phfac_utils.mod.F90:195)
//   E_loc    = Omega sum_G conj(rho(G)) V_ion(G)     ppener_utils.mod.F90:58-99,
//              vofrhoa_utils.mod.F90:125 (EPSEU = 2 Re(eps) Omega, G = 0 once)
//   E_H      = Omega sum_{G != 0, half} 4 pi |rho(G)|^2 / G^2   (ppener: eh, scg)
//   E_xc     = Omega/N sum_r rho eps_xc(rho): Slater exchange (alpha = 2/3,
//              cp_lda_exchange_utils.mod.F90:74-97) + Perdew-Zunger correlation
//              (cp_lda_correlation_utils.mod.F90:474-513); or, with the PBE option,
//              Omega/N sum_r f(rho, |grad rho|^2) of Perdew-Burke-Ernzerhof 1996 on
//              Perdew-Wang 1992 correlation, grad rho from rho(G) by FFT and
//              v_xc = df/drho - div(2 df/dsigma grad rho), the divergence by FFT too
//              (the reference's graden + gcener route, vofrhob_utils.mod.F90:80-471,
//              gcener_utils.mod.F90:60-304)
//   E_ext    = Omega/N sum_r V_ext(r) rho(r)  (optional mesh potential)
//
// Adjoint (nothing of psi(r) is stored: the band loop recomputes it):
//   dE/dc*   C2 = vpsi(c0, 0, f, V_eff), V_eff = V_ion + V_H + v_xc + V_ext,
//            the reference's CP force (vpsi_utils.mod.F90:661-671)
//   dE/dV(r) = rho(r) Omega / N
//   F_a      = 2 Omega sum_{G != 0, half} Re[e^{-iG.R_a} vps conj(rho(G)) iG]
//              potfor_utils.mod.F90:91-110
//
// Everything outside the band loop is FP64 whatever the context precision:
// the dense FFTs of rho and V, the structure factors, the energy reductions
// and the Hartree sum.  The cell is cubic with edge 2 pi / sqrt(tpiba2).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.h"

namespace gbcp {

namespace {

constexpr int kET = 256;     // threads per CTA
constexpr int kAT = 8;       // atoms per force CTA
constexpr double kRhoXcMin = 1.0e-30;
constexpr double kG2Min = 1.0e-12;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum of v over the CTA (kET threads); valid in thread 0
__device__ __forceinline__ double cta_sum(double v, double* sh) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (l < kET / 32) ? sh[l] : 0.0;
    r = warp_sum(r);
  }
  return r;
}

__global__ void k_rho_to_grid(const double* __restrict__ rho, cx<double>* __restrict__ grid, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    grid[i] = mk<double>(rho[i], 0.0);
}

// ei[(j*3 + d)*w + m + mmax] = e^{-i tpiba m tau_d} of atom order[j], w = 2 mmax + 1
__global__ void k_ei_table(const double* __restrict__ tau, const int* __restrict__ order, int nat, int mmax,
                           double tpiba, cx<double>* __restrict__ ei) {
  const int w = 2 * mmax + 1;
  const size_t total = (size_t)nat * 3 * w;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(i / (3 * (size_t)w));
    const int d = (int)((i / w) % 3);
    const int m = (int)(i % w) - mmax;
    double s, co;
    sincos(tpiba * (double)m * tau[3 * (size_t)order[j] + d], &s, &co);
    ei[i] = mk<double>(co, -s);
  }
}

__device__ __forceinline__ cx<double> phase(const cx<double>* __restrict__ ei, int j, int w, short4 m) {
  const cx<double>* e = ei + (size_t)j * 3 * w + (w >> 1);
  return cmul(cmul(e[m.x], e[w + m.y]), e[2 * w + m.z]);
}

// Per half-sphere G: V_ion(G), the Hartree and local energies, and
// V_ion + V_H written at +G and (conjugated) at -G of the zeroed grid vg.
__global__ void __launch_bounds__(kET) k_pot_g(int nhg, const int* __restrict__ dpos, const int* __restrict__ dneg,
                                               const short4* __restrict__ dmill, const double* __restrict__ dg2,
                                               const cx<double>* __restrict__ rhog, int nsp,
                                               const int* __restrict__ sp_start, const double* __restrict__ vps,
                                               int mmax, const cx<double>* __restrict__ ei,
                                               cx<double>* __restrict__ vg, double* __restrict__ part) {
  __shared__ double sh[kET / 32];
  const int w = 2 * mmax + 1;
  double eloc = 0.0, eh = 0.0;
  for (int g = blockIdx.x * kET + threadIdx.x; g < nhg; g += gridDim.x * kET) {
    const cx<double> rg = rhog[dpos[g]];
    const short4 m = dmill[g];
    cx<double> vion = mk<double>(0.0, 0.0);
    for (int s = 0; s < nsp; ++s) {
      cx<double> sf = mk<double>(0.0, 0.0);
      for (int j = sp_start[s]; j < sp_start[s + 1]; ++j) sf = sf + phase(ei, j, w, m);
      vion = vion + scl(sf, vps[g + (size_t)nhg * s]);
    }
    const double g2 = dg2[g];
    const double wg = g2 < kG2Min ? 1.0 : 2.0;
    eloc += wg * (rg.x * vion.x + rg.y * vion.y);
    const double scg = g2 < kG2Min ? 0.0 : 4.0 * M_PI / g2;
    eh += scg * (rg.x * rg.x + rg.y * rg.y);
    const cx<double> v = vion + scl(rg, scg);
    vg[dneg[g]] = mk<double>(v.x, -v.y);
    vg[dpos[g]] = v;
  }
  const double a = cta_sum(eloc, sh);
  const double b = cta_sum(eh, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// rho * eps_xc and v_xc (Slater alpha = 2/3 + Perdew-Zunger 1981, unpolarised)
__device__ __forceinline__ void lda_pz(double rho, double& e, double& v) {
  if (!(rho > kRhoXcMin)) {
    e = 0.0;
    v = 0.0;
    return;
  }
  const double cx_ = 0.98474502184269654;  // (3/pi)^(1/3): v_x = -cx rho^(1/3), eps_x = 3/4 v_x
  const double r13 = cbrt(rho);
  const double vx = -cx_ * r13;
  const double ex = 0.75 * vx;
  const double rs = 0.62035049089940009 / r13;  // (3/(4 pi))^(1/3) / rho^(1/3)
  double ec, vc;
  if (rs < 1.0) {
    const double a = 0.0311, b = -0.048, c = 0.0020, d = -0.0116;
    const double xln = log(rs);
    ec = a * xln + b + c * rs * xln + d * rs;
    vc = a * xln + (b - a / 3.0) + 2.0 / 3.0 * c * rs * xln + (2.0 * d - c) / 3.0 * rs;
  } else {
    const double gc = -0.1423, b1 = 1.0529, b2 = 0.3334;
    const double x = sqrt(rs);
    const double ox = 1.0 + b1 * x + b2 * rs;
    const double dox = 1.0 + 7.0 / 6.0 * b1 * x + 4.0 / 3.0 * b2 * rs;
    ec = gc / ox;
    vc = ec * dox / ox;
  }
  e = rho * (ex + ec);
  v = vx + vc;
}

// PBE, unpolarised: f = rho (eps_x + eps_c), df/drho, df/dsigma (sigma = |grad rho|^2);
// nothing below kRhoGgaMin.  Perdew, Burke, Ernzerhof, Phys. Rev. Lett. 77, 3865 (1996);
// correlation on Perdew, Wang, Phys. Rev. B 45, 13244 (1992).
constexpr double kRhoGgaMin = 1.0e-10;
__device__ __forceinline__ void pbe(double rho, double sigma, double& f, double& fr, double& fs) {
  if (!(rho > kRhoGgaMin)) {
    f = fr = fs = 0.0;
    return;
  }
  const double pi = 3.14159265358979323846;
  // exchange
  const double ax = -0.73855876638202234;     // -(3/4) (3/pi)^(1/3)
  const double cs = 0.026121172985233605;     // 1 / (4 (3 pi^2)^(2/3))
  const double kap = 0.804, mu = 0.2195149727645171;
  const double r13 = cbrt(rho), r43 = rho * r13;
  const double s2 = cs * sigma / (r43 * r43);
  const double den = kap + mu * s2;
  const double F = 1.0 + kap - kap * kap / den;
  const double dF = kap * kap * mu / (den * den);
  const double fx = ax * r43 * F;
  const double fx_r = (4.0 / 3.0) * ax * r13 * F + ax * r43 * dF * (-(8.0 / 3.0) * s2 / rho);
  const double fx_s = ax * r43 * dF * cs / (r43 * r43);
  // correlation: PW92
  const double A = 0.0310907, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  const double rs = 0.62035049089940009 / r13;  // (3/(4 pi rho))^(1/3)
  const double srs = sqrt(rs);
  const double Q = b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs;
  const double dQ = 0.5 * b1 / srs + b2 + 1.5 * b3 * srs + 2.0 * b4 * rs;
  const double L = log1p(1.0 / (2.0 * A * Q));
  const double ec = -2.0 * A * (1.0 + a1 * rs) * L;
  const double dec_rs = -2.0 * A * a1 * L + (1.0 + a1 * rs) * dQ / (Q * Q * (1.0 + 1.0 / (2.0 * A * Q)));
  const double dec_r = dec_rs * (-rs / (3.0 * rho));
  // gradient correction H(rs, t)
  const double beta = 0.06672455060314922, gam = 0.031090690869654895;  // (1 - ln 2) / pi^2
  const double ct = pi / (16.0 * 3.0936677262801355);                   // pi / (16 (3 pi^2)^(1/3))
  const double y = ct * sigma / (rho * rho * r13);
  const double E = exp(-ec / gam);
  const double Aa = (beta / gam) / (E - 1.0);
  const double dAa = (beta / (gam * gam)) * E / ((E - 1.0) * (E - 1.0));
  const double Nn = 1.0 + Aa * y, Dd = 1.0 + Aa * y + Aa * Aa * y * y;
  const double Bb = (beta / gam) * y * Nn / Dd;
  const double H = gam * log1p(Bb);
  const double dB_y = (beta / gam) * (Nn / Dd + y * (Aa * Dd - Nn * (Aa + 2.0 * Aa * Aa * y)) / (Dd * Dd));
  const double dB_A = (beta / gam) * y * (y * Dd - Nn * (y + 2.0 * Aa * y * y)) / (Dd * Dd);
  const double dH_y = gam * dB_y / (1.0 + Bb), dH_A = gam * dB_A / (1.0 + Bb);
  const double fc = rho * (ec + H);
  const double fc_r = (ec + H) + rho * (dec_r + dH_A * dAa * dec_r + dH_y * (-(7.0 / 3.0) * y / rho));
  const double fc_s = rho * dH_y * ct / (rho * rho * r13);
  f = fx + fc;
  fr = fx_r + fc_r;
  fs = fx_s + fc_s;
}

// i tpiba m of mesh index i on an axis of length n (Nyquist of an even n -> 0)
__device__ __forceinline__ double deriv_freq(int i, int n) {
  if ((n & 1) == 0 && 2 * i == n) return 0.0;
  return (double)(2 * i < n + 1 ? i : i - n);
}

// g3[d] = i tpiba m_d rho(G), d = x, y, z, on the (k1, k2, n3) FFT grid
__global__ void k_grad_g(const cx<double>* __restrict__ rg, cx<double>* __restrict__ g3, int n1, int n2, int n3,
                         int k1, int k2, double tpiba) {
  const size_t ng = (size_t)k1 * k2 * n3;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ng; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % k1), y = (int)((i / k1) % k2), z = (int)(i / ((size_t)k1 * k2));
    const bool in = x < n1 && y < n2;
    const cx<double> v = in ? rg[i] : mk<double>(0.0, 0.0);
    const double m[3] = {in ? deriv_freq(x, n1) : 0.0, in ? deriv_freq(y, n2) : 0.0, in ? deriv_freq(z, n3) : 0.0};
#pragma unroll
    for (int d = 0; d < 3; ++d) g3[d * ng + i] = mk<double>(-tpiba * m[d] * v.y, tpiba * m[d] * v.x);
  }
}

// sum_d i tpiba m_d h_d(G) into g3[0]
__global__ void k_div_g(cx<double>* __restrict__ g3, int n1, int n2, int n3, int k1, int k2, double tpiba) {
  const size_t ng = (size_t)k1 * k2 * n3;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ng; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % k1), y = (int)((i / k1) % k2), z = (int)(i / ((size_t)k1 * k2));
    const bool in = x < n1 && y < n2;
    const double m[3] = {in ? deriv_freq(x, n1) : 0.0, in ? deriv_freq(y, n2) : 0.0, in ? deriv_freq(z, n3) : 0.0};
    double re = 0.0, im = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const cx<double> h = g3[d * ng + i];
      re -= tpiba * m[d] * h.y;
      im += tpiba * m[d] * h.x;
    }
    g3[i] = mk<double>(re, im);
  }
}

// PBE per mesh point: V_eff = Re(vr) + df/drho (+ V_ext), dE/dV, partial sums of f and
// V_ext rho; g3[d] (grad rho in the real parts) is overwritten by h_d = 2 df/dsigma d_d rho
__global__ void __launch_bounds__(kET) k_xc_pbe(const double* __restrict__ rho, const cx<double>* __restrict__ vr,
                                                const double* __restrict__ vext, cx<double>* __restrict__ g3,
                                                int n1, int n2, int n3, int k1, int k2, int k3, double dscale,
                                                double* __restrict__ veff, double* __restrict__ dvloc,
                                                double* __restrict__ part) {
  __shared__ double sh[kET / 32];
  const size_t n = (size_t)k1 * k2 * k3, ng = (size_t)k1 * k2 * n3;
  double exc = 0.0, eext = 0.0;
  for (size_t i = blockIdx.x * (size_t)kET + threadIdx.x; i < n; i += (size_t)gridDim.x * kET) {
    const int x = (int)(i % k1);
    const int y = (int)((i / k1) % k2);
    const int z = (int)(i / ((size_t)k1 * k2));
    double ve = 0.0, dv = 0.0;
    if (x < n1 && y < n2 && z < n3) {
      const double r = rho[i];
      const double gx = g3[i].x, gy = g3[ng + i].x, gz = g3[2 * ng + i].x;
      double f, fr, fs;
      pbe(r, gx * gx + gy * gy + gz * gz, f, fr, fs);
      exc += f;
      ve = vr[i].x + fr;
      if (vext) {
        ve += vext[i];
        eext += vext[i] * r;
      }
      dv = r * dscale;
      g3[i] = mk<double>(2.0 * fs * gx, 0.0);
      g3[ng + i] = mk<double>(2.0 * fs * gy, 0.0);
      g3[2 * ng + i] = mk<double>(2.0 * fs * gz, 0.0);
    } else if (i < ng) {
      g3[i] = g3[ng + i] = g3[2 * ng + i] = mk<double>(0.0, 0.0);
    }
    veff[i] = ve;
    if (dvloc) dvloc[i] = dv;
  }
  const double a = cta_sum(exc, sh);
  const double b = cta_sum(eext, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// V_eff -= div(h) on the mesh points
__global__ void k_sub_div(const cx<double>* __restrict__ div, int n1, int n2, int n3, int k1, int k2,
                          double* __restrict__ veff) {
  const size_t ng = (size_t)k1 * k2 * n3;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ng; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % k1), y = (int)((i / k1) % k2);
    if (x < n1 && y < n2) veff[i] -= div[i].x;
  }
}

// V_eff = Re(vr) + v_xc + V_ext and dE/dV = rho Omega/N on the padded mesh;
// partial sums of rho eps_xc and V_ext rho
__global__ void __launch_bounds__(kET) k_xc(const double* __restrict__ rho, const cx<double>* __restrict__ vr,
                                            const double* __restrict__ vext, int n1, int n2, int n3, int k1, int k2,
                                            int k3, double dscale, double* __restrict__ veff,
                                            double* __restrict__ dvloc, double* __restrict__ part) {
  __shared__ double sh[kET / 32];
  const size_t n = (size_t)k1 * k2 * k3;
  double exc = 0.0, eext = 0.0;
  for (size_t i = blockIdx.x * (size_t)kET + threadIdx.x; i < n; i += (size_t)gridDim.x * kET) {
    const int x = (int)(i % k1);
    const int y = (int)((i / k1) % k2);
    const int z = (int)(i / ((size_t)k1 * k2));
    double ve = 0.0, dv = 0.0;
    if (x < n1 && y < n2 && z < n3) {
      const double r = rho[i];
      double e, v;
      lda_pz(r, e, v);
      exc += e;
      ve = vr[i].x + v;
      if (vext) {
        ve += vext[i];
        eext += vext[i] * r;
      }
      dv = r * dscale;
    }
    veff[i] = ve;
    if (dvloc) dvloc[i] = dv;
  }
  const double a = cta_sum(exc, sh);
  const double b = cta_sum(eext, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// Force partial sums: CTA (chunk, tile) covers a slice of G for kAT atoms;
// part[((chunk * nat) + j) * 3 + d] = sum_G -Im(e^{-iG.R_j} vps conj(rho(G))) m_d
__global__ void __launch_bounds__(kET) k_forces(int nhg, const int* __restrict__ dpos,
                                                const short4* __restrict__ dmill, const double* __restrict__ dg2,
                                                const cx<double>* __restrict__ rhog, int nat,
                                                const int* __restrict__ jsp, const double* __restrict__ vps,
                                                int mmax, const cx<double>* __restrict__ ei,
                                                double* __restrict__ part) {
  __shared__ double sh[kET / 32];
  const int w = 2 * mmax + 1;
  const int j0 = blockIdx.y * kAT;
  const int per = (nhg + gridDim.x - 1) / gridDim.x;
  const int g0 = blockIdx.x * per, g1 = min(nhg, g0 + per);
  double acc[kAT][3];
#pragma unroll
  for (int k = 0; k < kAT; ++k) acc[k][0] = acc[k][1] = acc[k][2] = 0.0;
  for (int g = g0 + threadIdx.x; g < g1; g += kET) {
    if (dg2[g] < kG2Min) continue;
    const cx<double> rg = rhog[dpos[g]];
    const short4 m = dmill[g];
#pragma unroll
    for (int k = 0; k < kAT; ++k) {
      const int j = j0 + k;
      if (j < nat) {
        const cx<double> t = scl(cmulc(phase(ei, j, w, m), rg), vps[g + (size_t)nhg * jsp[j]]);
        acc[k][0] -= t.y * (double)m.x;
        acc[k][1] -= t.y * (double)m.y;
        acc[k][2] -= t.y * (double)m.z;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kAT; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double s = cta_sum(acc[k][d], sh);
      if (threadIdx.x == 0 && j0 + k < nat) part[((size_t)blockIdx.x * nat + j0 + k) * 3 + d] = s;
    }
}

__global__ void k_forces_fold(const double* __restrict__ part, int nchunk, int nat, const int* __restrict__ order,
                              double scale, double* __restrict__ fion) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nat) return;
  double s = 0.0;
  for (int ch = 0; ch < nchunk; ++ch) s += part[(size_t)ch * 3 * nat + i];
  const int j = i / 3, d = i % 3;
  fion[3 * (size_t)order[j] + d] = scale * s;
}

// out[k] = sum_i part[2 i + k], k = 0, 1 (one CTA)
__global__ void __launch_bounds__(kET) k_fold_pairs(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double sh[kET / 32];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += kET) {
    a += part[2 * i];
    b += part[2 * i + 1];
  }
  a = cta_sum(a, sh);
  b = cta_sum(b, sh);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}

}  // namespace

// Density -> potential (the reference's vofrho: vofrhoa_utils.mod.F90:41-144 with the
// vofrhob xc step): from rho(r) (padded layout, device) to V_eff(r) = V_ion + V_H + v_xc
// (+ vext), dE/dV = rho Omega / N (dvloc, may be null), the local-potential forces
// (fion, may be null) and the energy partial sums, left on the device in sums[0..3]
// = {E_loc / Omega, E_H / Omega, sum eps_xc rho, sum vext rho} (no host synchronisation).
int vofrho(Ctx& c, const double* rho, int nat, int nsp, const int* isp_host, const double* tau, const double* vps,
           const double* vext, double* veff, double* dvloc, double* fion, double** sums_out) {
  if (c.nhg <= 0) {
    c.err = "energy: no density sphere (gbcp_set_dens_sphere)";
    return 1;
  }
  const int n1 = c.nr[0], n2 = c.nr[1], n3 = c.nr[2], k1 = c.kr[0], k2 = c.kr[1], k3 = c.kr[2];
  const size_t nnr1 = (size_t)k1 * k2 * k3;
  const size_t ngrid = (size_t)k1 * k2 * n3;
  const double nmesh = (double)n1 * n2 * n3;
  const double tpiba = std::sqrt(c.tpiba2);
  int rc;

  // atoms sorted by species: order[j] = atom, sp_start[s] = first sorted index of species s
  std::vector<int> idx(2 * (size_t)nat + nsp + 1);
  int* order = idx.data();
  int* jsp = order + nat;
  int* sp_start = jsp + nat;
  {
    int j = 0;
    for (int s = 0; s < nsp; ++s) {
      sp_start[s] = j;
      for (int a = 0; a < nat; ++a)
        if (isp_host[a] == s) {
          order[j] = a;
          jsp[j] = s;
          ++j;
        }
    }
    sp_start[nsp] = j;
    if (j != nat) {
      c.err = "energy: species index out of range";
      return 1;
    }
  }
  if (!ensure(c, c.en_idx, sizeof(int) * idx.size())) return 6;
  int* d_idx = static_cast<int*>(c.en_idx.p);
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(d_idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, c.stream));
  const int* d_order = d_idx;
  const int* d_jsp = d_idx + nat;
  const int* d_spstart = d_idx + 2 * nat;

  // rho(G)
  if (!ensure(c, c.en_a, sizeof(cx<double>) * ngrid) || !ensure(c, c.en_b, sizeof(cx<double>) * ngrid)) return 6;
  cx<double>* ga = static_cast<cx<double>*>(c.en_a.p);
  cx<double>* gb = static_cast<cx<double>*>(c.en_b.p);
  {
    ProfScope ps_(c, "k_rho_to_grid");
    k_rho_to_grid<<<std::min<size_t>(4096, (ngrid + kET - 1) / kET), kET, 0, c.stream>>>(rho, ga, ngrid);
    GBCP_LAUNCH_CHECK(c);
  }
  if ((rc = dense_fft(c, ga, false))) return rc;

  // structure-factor tables
  const int w = 2 * c.dmax + 1;
  if (!ensure(c, c.en_ei, sizeof(cx<double>) * (size_t)std::max(nat, 1) * 3 * w)) return 6;
  cx<double>* ei = static_cast<cx<double>*>(c.en_ei.p);
  if (nat > 0) {
    ProfScope ps_(c, "k_ei_table");
    const size_t tot = (size_t)nat * 3 * w;
    k_ei_table<<<std::max<size_t>(1, std::min<size_t>(1024, (tot + kET - 1) / kET)), kET, 0, c.stream>>>(
        tau, d_order, nat, c.dmax, tpiba, ei);
    GBCP_LAUNCH_CHECK(c);
  }

  // V_ion + V_H on the sphere, E_loc and E_H partials, then V(r)
  const int nb_g = std::max(1, std::min(4 * 152, (c.nhg + kET - 1) / kET));
  const int nb_r = std::max(1, (int)std::min<size_t>(4 * 152, (nnr1 + kET - 1) / kET));
  if (!ensure(c, c.en_red, sizeof(double) * (2 * (size_t)nb_g + 2 * (size_t)nb_r + 8))) return 6;
  double* part_g = static_cast<double*>(c.en_red.p);
  double* part_r = part_g + 2 * nb_g;
  double* sums = part_r + 2 * nb_r;
  GBCP_CUDA_TRY(c, cudaMemsetAsync(gb, 0, sizeof(cx<double>) * ngrid, c.stream));
  {
    ProfScope ps_(c, "k_pot_g");
    k_pot_g<<<nb_g, kET, 0, c.stream>>>(c.nhg, c.dpos, c.dneg, c.dmill, c.dg2, ga, nsp, d_spstart, vps, c.dmax, ei,
                                        gb, part_g);
    GBCP_LAUNCH_CHECK(c);
  }
  if ((rc = dense_fft(c, gb, true))) return rc;

  // xc, V_eff, dE/dV
  const int nb_n = std::max(1, (int)std::min<size_t>(4096, (ngrid + kET - 1) / kET));
  if (c.xc == 1) {
    // PBE: grad rho by three inverse FFTs of i G rho(G); the per-point functional writes
    // h = 2 df/dsigma grad rho over them; div h by three forward FFTs and one inverse
    if (!ensure(c, c.en_g3, sizeof(cx<double>) * 3 * ngrid)) return 6;
    cx<double>* g3 = static_cast<cx<double>*>(c.en_g3.p);
    {
      ProfScope ps_(c, "k_grad_g");
      k_grad_g<<<nb_n, kET, 0, c.stream>>>(ga, g3, n1, n2, n3, k1, k2, tpiba);
      GBCP_LAUNCH_CHECK(c);
    }
    for (int d = 0; d < 3; ++d)
      if ((rc = dense_fft(c, g3 + d * ngrid, true))) return rc;
    {
      ProfScope ps_(c, "k_xc_pbe");
      k_xc_pbe<<<nb_r, kET, 0, c.stream>>>(rho, gb, vext, g3, n1, n2, n3, k1, k2, k3, c.omega / nmesh, veff, dvloc,
                                           part_r);
      GBCP_LAUNCH_CHECK(c);
    }
    for (int d = 0; d < 3; ++d)
      if ((rc = dense_fft(c, g3 + d * ngrid, false))) return rc;
    {
      ProfScope ps_(c, "k_div_g");
      k_div_g<<<nb_n, kET, 0, c.stream>>>(g3, n1, n2, n3, k1, k2, tpiba);
      GBCP_LAUNCH_CHECK(c);
    }
    if ((rc = dense_fft(c, g3, true))) return rc;
    {
      ProfScope ps_(c, "k_sub_div");
      k_sub_div<<<nb_n, kET, 0, c.stream>>>(g3, n1, n2, n3, k1, k2, veff);
      GBCP_LAUNCH_CHECK(c);
    }
  } else {
    ProfScope ps_(c, "k_xc");
    k_xc<<<nb_r, kET, 0, c.stream>>>(rho, gb, vext, n1, n2, n3, k1, k2, k3, c.omega / nmesh, veff, dvloc, part_r);
    GBCP_LAUNCH_CHECK(c);
  }
  {
    ProfScope ps_(c, "k_fold_pairs");
    k_fold_pairs<<<1, kET, 0, c.stream>>>(part_g, nb_g, sums);
    GBCP_LAUNCH_CHECK(c);
    k_fold_pairs<<<1, kET, 0, c.stream>>>(part_r, nb_r, sums + 2);
    GBCP_LAUNCH_CHECK(c);
  }

  // forces
  if (fion && nat > 0) {
    const int ntile = (nat + kAT - 1) / kAT;
    const int nchunk = std::max(1, std::min((c.nhg + kET - 1) / kET, (4 * 152 + ntile - 1) / ntile));
    if (!ensure(c, c.en_fp, sizeof(double) * (size_t)nchunk * 3 * nat)) return 6;
    double* fp = static_cast<double*>(c.en_fp.p);
    ProfScope ps_(c, "k_forces");
    k_forces<<<dim3(nchunk, ntile), kET, 0, c.stream>>>(c.nhg, c.dpos, c.dmill, c.dg2, ga, nat, d_jsp, vps, c.dmax,
                                                        ei, fp);
    GBCP_LAUNCH_CHECK(c);
    k_forces_fold<<<(3 * nat + 127) / 128, 128, 0, c.stream>>>(fp, nchunk, nat, d_order, 2.0 * c.omega * tpiba,
                                                                fion);
    GBCP_LAUNCH_CHECK(c);
  }
  *sums_out = sums;
  return 0;
}

// host read of the four partial sums of vofrho: {E_loc, E_H, E_xc, E_ext} in Ha
static int vofrho_energies(Ctx& c, const double* sums, const double* dscal, double* e4, double* ekin) {
  double h[8];
  GBCP_CUDA_TRY(c, cudaMemcpyAsync(h, sums, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  if (dscal) GBCP_CUDA_TRY(c, cudaMemcpyAsync(h + 4, dscal, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  const double nmesh = (double)c.nr[0] * c.nr[1] * c.nr[2];
  e4[0] = c.omega * h[0];
  e4[1] = c.omega * h[1];
  e4[2] = c.omega / nmesh * h[2];
  e4[3] = c.omega / nmesh * h[3];
  if (ekin) *ekin = h[4];
  for (int k = 0; k < 4; ++k)
    if (!std::isfinite(e4[k])) {
      c.err = "energy: non-finite result";
      return 3;
    }
  if (ekin && !std::isfinite(*ekin)) {
    c.err = "energy: non-finite kinetic energy";
    return 3;
  }
  return 0;
}

int vofrho_host_energies(Ctx& c, int nat, int nsp, const int* isp_host, const double* rho, const double* tau,
                         const double* vps, const double* vext, double* veff, double* energies4, double* fion) {
  double* sums = nullptr;
  int rc = vofrho(c, rho, nat, nsp, isp_host, tau, vps, vext, veff, nullptr, fion, &sums);
  if (rc) return rc;
  return vofrho_energies(c, sums, nullptr, energies4, nullptr);
}

int energy_and_grad(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, int nat, int nsp,
                    const int* isp_host, const double* tau, const double* vps, const double* vext,
                    double* energies_host, cx<double>* c2, int ldc2, double* dvloc, double* fion) {
  const size_t nnr1 = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  int rc;
  // density and E_kin (band loop in the context precision; E_kin summed in its gather)
  if (!ensure(c, c.en_rho, sizeof(double) * nnr1) || !ensure(c, c.rho_sc, 4 * sizeof(double))) return 6;
  double* rho = static_cast<double*>(c.en_rho.p);
  double* dscal = static_cast<double*>(c.rho_sc.p);
  if ((rc = band_rhoofr(c, c0, ldc, nstate, f, rho, dscal))) return rc;
  if (!ensure(c, c.en_veff, sizeof(double) * nnr1)) return 6;
  double* veff = static_cast<double*>(c.en_veff.p);
  double* sums = nullptr;
  if ((rc = vofrho(c, rho, nat, nsp, isp_host, tau, vps, vext, veff, dvloc, fion, &sums))) return rc;

  // C2 = vpsi(c0, 0, f, V_eff)
  if (c2) {
    GBCP_CUDA_TRY(c, cudaMemset2DAsync(c2, sizeof(cx<double>) * (size_t)ldc2, 0, sizeof(cx<double>) * c.ngw, nstate,
                                       c.stream));
    if ((rc = band_vpsi(c, c0, ldc, c2, ldc2, f, veff, nstate))) return rc;
  }

  double e4[4], ekin = 0.0;
  if ((rc = vofrho_energies(c, sums, dscal, e4, &ekin))) return rc;
  energies_host[0] = ekin + e4[0] + e4[1] + e4[2] + e4[3];
  energies_host[1] = ekin;
  for (int k = 0; k < 4; ++k) energies_host[2 + k] = e4[k];
  return 0;
}

}  // namespace gbcp
