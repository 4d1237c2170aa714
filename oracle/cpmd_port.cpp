// C++/OpenMP FP64 restatement of CPMD's Γ-point CPU path: rhoofr, vpsi and the
// Cholesky Gram-Schmidt ortho.
//
// TEST INFRASTRUCTURE AND TIMED CPU BASELINE ONLY.  Nothing in the product (the
// cpmd_gb300 package, its CUDA library, the C ABI) links or calls this file; the
// tests use it as a second checker beside cpmd_oracle.py, and bench.py times it
// as the CPU stand-in for the reference (Fortran + FFTW + BLAS/LAPACK), which
// cannot be built here.  It follows the reference's structure, not the GPU
// design: every OpenMP thread takes whole state pairs, as CPMD's band loop does
// (rhoofr_utils.mod.F90:305-409, vpsi_utils.mod.F90:376-675), and each pair goes
// through a sparse 3D FFT that transforms only the lines the wavefunction sphere
// occupies, the pruning of the reference's sparse FFT (fftnew_utils.mod.F90:
// 71-157; z-lines of the sphere columns, y-lines of the sphere's x range, full
// x-rows, with the density or V(r) applied on each x-row).
//
// Conventions restated (cited in cpmd_oracle.py as well):
//  * Γ pair packing psi = c1 + i c2 at +G, conj(c1) + i conj(c2) at -G
//    (state_utils.mod.F90:182-187);
//  * inverse FFT e^{+iGr} unscaled, forward e^{-iGr} scaled 1/N
//    (fftmain_utils.mod.F90:90-154);
//  * density rho += f1/omega Re(psi)^2 + f2/omega Im(psi)^2 (density_utils.mod.F90:77-80);
//  * kinetic energy tpiba2 sum f hg |c|^2, norm sum f <c|c> with the Γ weights
//    (kin_energy_utils.mod.F90:93-108, dotp_utils.mod.F90:45-52), csumr
//    (rhoofr_utils.mod.F90:607-618);
//  * vpsi decode c2 += -f/2 (tpiba2 hg c + fp/fm), f = 0 counted as 2
//    (vpsi_utils.mod.F90:627-671, 717);
//  * Gram-Schmidt S = 2 Re C^H C - Re c(0) Re c(0)^T, S = U^T U, C <- C U^-1,
//    Im c(G=0) = 0 (rgs_utils.mod.F90:63-74, 127-158; ortho_utils.mod.F90:264-268).
// The 1D FFT is a mixed-radix (2, 3, 4, 5) Stockham autosort transform written
// from the textbook recurrence (Van Loan, Computational Frameworks for the FFT,
// 1992, section 1.7); twiddles come from std::cos/std::sin.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

namespace {

using cd = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------- 1D FFT
struct Fft1 {
  int n = 0;
  std::vector<int> rad;  // radices, product n
  std::vector<int> off;  // twiddle offset of each stage
  std::vector<cd> tw[2];  // [0] sign -1 (forward), [1] sign +1 (inverse)
};

bool plan1(Fft1& p, int n) {
  p.n = n;
  p.rad.clear();
  int m = n;
  while (m % 4 == 0) { p.rad.push_back(4); m /= 4; }
  while (m % 2 == 0) { p.rad.push_back(2); m /= 2; }
  while (m % 3 == 0) { p.rad.push_back(3); m /= 3; }
  while (m % 5 == 0) { p.rad.push_back(5); m /= 5; }
  if (m != 1) return false;
  p.off.clear();
  for (int sg = 0; sg < 2; ++sg) p.tw[sg].clear();
  int len = n;
  for (int r : p.rad) {
    const int mm = len / r;
    p.off.push_back((int)p.tw[0].size());
    for (int q = 0; q < mm; ++q)
      for (int k = 1; k < r; ++k) {
        const double a = 2.0 * kPi * (double)q * k / len;
        p.tw[0].push_back(cd(std::cos(a), -std::sin(a)));
        p.tw[1].push_back(cd(std::cos(a), std::sin(a)));
      }
    len = mm;
  }
  return true;
}

// length-r DFT in place with omega = e^{sign 2 pi i / r}
inline void dft_small(int r, cd* a, double sg) {
  const cd I(0.0, sg);
  if (r == 2) {
    const cd t = a[0] - a[1];
    a[0] += a[1];
    a[1] = t;
  } else if (r == 4) {
    const cd s02 = a[0] + a[2], d02 = a[0] - a[2], s13 = a[1] + a[3], d13 = I * (a[1] - a[3]);
    a[0] = s02 + s13;
    a[1] = d02 + d13;
    a[2] = s02 - s13;
    a[3] = d02 - d13;
  } else if (r == 3) {
    const double s3 = std::sqrt(3.0) * 0.5;
    const cd t = a[1] + a[2], m = a[0] - 0.5 * t, d = I * (s3 * (a[1] - a[2]));
    a[0] += t;
    a[1] = m + d;
    a[2] = m - d;
  } else {  // 5
    const double c1 = std::cos(2.0 * kPi / 5.0), c2 = std::cos(4.0 * kPi / 5.0);
    const double s1 = std::sin(2.0 * kPi / 5.0), s2 = std::sin(4.0 * kPi / 5.0);
    const cd t1 = a[1] + a[4], t2 = a[2] + a[3], t3 = a[1] - a[4], t4 = a[2] - a[3];
    const cd m1 = a[0] + c1 * t1 + c2 * t2, m2 = a[0] + c2 * t1 + c1 * t2;
    const cd n1 = I * (s1 * t3 + s2 * t4), n2 = I * (s2 * t3 - s1 * t4);
    a[0] += t1 + t2;
    a[1] = m1 + n1;
    a[4] = m1 - n1;
    a[2] = m2 + n2;
    a[3] = m2 - n2;
  }
}

// x (length n, contiguous) transformed in place; work has room for n values.
// sign +1: e^{+2 pi i jk/n} (inverse, unscaled); -1: e^{-2 pi i jk/n}.
void fft1(const Fft1& p, cd* x, cd* work, int sign) {
  const double sg = sign > 0 ? 1.0 : -1.0;
  const std::vector<cd>& tw = p.tw[sign > 0 ? 1 : 0];
  cd* src = x;
  cd* dst = work;
  int len = p.n, s = 1;
  for (size_t st = 0; st < p.rad.size(); ++st) {
    const int r = p.rad[st], m = len / r;
    const cd* w = tw.data() + p.off[st];
    cd a[5];
    for (int q = 0; q < m; ++q) {
      const cd* wq = w + (size_t)q * (r - 1);
      for (int j0 = 0; j0 < s; ++j0) {
        for (int k = 0; k < r; ++k) a[k] = src[j0 + (size_t)s * (q + k * m)];
        dft_small(r, a, sg);
        cd* o = dst + j0 + (size_t)s * r * q;
        o[0] = a[0];
        for (int k = 1; k < r; ++k) o[(size_t)s * k] = a[k] * wq[k - 1];
      }
    }
    std::swap(src, dst);
    len = m;
    s *= r;
  }
  if (src != x) std::memcpy(x, src, sizeof(cd) * p.n);
}

inline int fidx(int g, int n) { return g < 0 ? g + n : g; }

// ---------------------------------------------------------------- cell geometry
struct Port {
  int nr[3], kr[3], ngw, geq0, nthreads;
  double omega, tpiba2;
  std::vector<double> hg;
  Fft1 fx, fy, fz;
  // sphere columns (gx, gy) of +G and -G, sorted by gx then gy
  int ncol = 0, gxlo = 0, nslot = 0;
  std::vector<int> col_gx, col_gy;
  std::vector<std::vector<std::pair<int, int>>> col_ent;  // (gz, +-(ig+1))
  std::vector<std::vector<int>> slot_cols;                 // columns of each gx slot
  std::vector<int> pos_plus, pos_minus;                    // (column, gz) of +G / -G as col * nr3 + idx(gz)
};

// per-thread work buffers of one pair's sparse transform
struct Work {
  std::vector<cd> zc;   // ncol x nr3: z-lines of the sphere columns
  std::vector<cd> yb;   // nr3 x nslot x nr2: y-lines of the sphere's x range
  std::vector<cd> line, tmp;
  std::vector<double> rho;  // private density (nr1 nr2 nr3)
};

void alloc_work(const Port& P, Work& w, bool rho) {
  w.zc.assign((size_t)P.ncol * P.nr[2], cd());
  w.yb.assign((size_t)P.nr[2] * P.nslot * P.nr[1], cd());
  const int nmax = std::max({P.nr[0], P.nr[1], P.nr[2]});
  w.line.assign(nmax, cd());
  w.tmp.assign(nmax, cd());
  if (rho) w.rho.assign((size_t)P.nr[0] * P.nr[1] * P.nr[2], 0.0);
}

// inverse sparse transform of the pair (c1, c2) up to the y-lines (yb); the
// x-rows are formed by the caller
void pair_inverse_zy(const Port& P, const cd* c1, const cd* c2, Work& w) {
  const int n2 = P.nr[1], n3 = P.nr[2];
  // z-lines of the sphere columns, pair-packed
  for (int col = 0; col < P.ncol; ++col) {
    cd* zl = w.zc.data() + (size_t)col * n3;
    std::fill(zl, zl + n3, cd());
    for (const auto& e : P.col_ent[col]) {
      const int ig = std::abs(e.second) - 1;
      const cd u = c1[ig], v = c2 ? c2[ig] : cd();
      zl[fidx(e.first, n3)] = e.second > 0 ? u + cd(0, 1) * v : std::conj(u) + cd(0, 1) * std::conj(v);
    }
    fft1(P.fz, zl, w.tmp.data(), +1);
  }
  // y-lines of every z-plane and gx slot
  for (int z = 0; z < n3; ++z)
    for (int s = 0; s < P.nslot; ++s) {
      cd* yl = w.yb.data() + ((size_t)z * P.nslot + s) * n2;
      std::fill(yl, yl + n2, cd());
      for (int col : P.slot_cols[s]) yl[fidx(P.col_gy[col], n2)] = w.zc[(size_t)col * n3 + z];
      fft1(P.fy, yl, w.tmp.data(), +1);
    }
}

// x-row (y, z) of the pair from the y-lines
inline void form_row(const Port& P, const Work& w, int y, int z, cd* row) {
  const int n1 = P.nr[0], n2 = P.nr[1];
  std::fill(row, row + n1, cd());
  for (int s = 0; s < P.nslot; ++s) row[fidx(P.gxlo + s, n1)] = w.yb[((size_t)z * P.nslot + s) * n2 + y];
}

void kin_norm(const Port& P, const cd* c0, int ldc, int nstate, const double* f, double* ekin, double* csumg) {
  double ek = 0.0, cg = 0.0;
#pragma omp parallel for reduction(+ : ek, cg) schedule(static) num_threads(P.nthreads)
  for (int i = 0; i < nstate; ++i) {
    const cd* c = c0 + (size_t)i * ldc;
    double sk = 0.0, sn = 0.0;
    for (int ig = 0; ig < P.ngw; ++ig) {
      const double a2 = std::norm(c[ig]);
      sk += P.hg[ig] * a2;
      sn += (P.geq0 && ig == 0) ? c[ig].real() * c[ig].real() : 2.0 * a2;
    }
    ek += f[i] * sk;
    cg += f[i] * sn;
  }
  *ekin = ek * P.tpiba2;
  *csumg = cg;
}

// ---------------------------------------------------------------- Gram-Schmidt helpers
// S (n x n, row-major) = A^T A over the real view A (K x n, column j at A + j lda)
void syrk_t(const double* A, int lda, int K, int n, double* S, int nthreads) {
  constexpr int T = 32, KB = 256;
  const int nt = (n + T - 1) / T;
  std::vector<std::pair<int, int>> tiles;
  for (int bi = 0; bi < nt; ++bi)
    for (int bj = bi; bj < nt; ++bj) tiles.push_back({bi, bj});
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (int t = 0; t < (int)tiles.size(); ++t) {
    const int i0 = tiles[t].first * T, j0 = tiles[t].second * T;
    const int ni = std::min(T, n - i0), nj = std::min(T, n - j0);
    double acc[T][T] = {};
    for (int k0 = 0; k0 < K; k0 += KB) {
      const int kb = std::min(KB, K - k0);
      for (int i = 0; i < ni; ++i) {
        const double* ai = A + (size_t)(i0 + i) * lda + k0;
        for (int j = 0; j < nj; ++j) {
          const double* aj = A + (size_t)(j0 + j) * lda + k0;
          double s = 0.0;
          for (int k = 0; k < kb; ++k) s += ai[k] * aj[k];
          acc[i][j] += s;
        }
      }
    }
    for (int i = 0; i < ni; ++i)
      for (int j = 0; j < nj; ++j) {
        S[(size_t)(i0 + i) * n + j0 + j] = acc[i][j];
        S[(size_t)(j0 + j) * n + i0 + i] = acc[i][j];
      }
  }
}

}  // namespace

// ============================================================================ C ABI (ctypes)
extern "C" {

// mill: (ngw, 3) centred Miller indices of the half sphere (G = 0 first when geq0)
void* port_create(int nr1, int nr2, int nr3, int kr1, int kr2, int kr3, int ngw, int geq0, double omega,
                  double tpiba2, const int32_t* mill, const double* hg, int nthreads) {
  Port* P = new Port();
  P->nr[0] = nr1; P->nr[1] = nr2; P->nr[2] = nr3;
  P->kr[0] = kr1; P->kr[1] = kr2; P->kr[2] = kr3;
  P->ngw = ngw;
  P->geq0 = geq0;
  P->omega = omega;
  P->tpiba2 = tpiba2;
  P->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
  P->hg.assign(hg, hg + ngw);
  if (!plan1(P->fx, nr1) || !plan1(P->fy, nr2) || !plan1(P->fz, nr3)) {
    delete P;
    return nullptr;
  }
  std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> cols;
  for (int ig = 0; ig < ngw; ++ig) {
    const int gx = mill[3 * ig], gy = mill[3 * ig + 1], gz = mill[3 * ig + 2];
    cols[{gx, gy}].push_back({gz, ig + 1});
    if (!(geq0 && ig == 0)) cols[{-gx, -gy}].push_back({-gz, -(ig + 1)});
  }
  int gxhi = -(1 << 30);
  P->gxlo = 1 << 30;
  for (auto& kv : cols) {
    P->col_gx.push_back(kv.first.first);
    P->col_gy.push_back(kv.first.second);
    P->col_ent.push_back(kv.second);
    P->gxlo = std::min(P->gxlo, kv.first.first);
    gxhi = std::max(gxhi, kv.first.first);
  }
  P->ncol = (int)P->col_gx.size();
  P->nslot = gxhi - P->gxlo + 1;
  P->slot_cols.assign(P->nslot, {});
  for (int c = 0; c < P->ncol; ++c) P->slot_cols[P->col_gx[c] - P->gxlo].push_back(c);
  P->pos_plus.assign(ngw, -1);
  P->pos_minus.assign(ngw, -1);
  for (int c = 0; c < P->ncol; ++c)
    for (auto& e : P->col_ent[c]) {
      const int pos = c * nr3 + fidx(e.first, nr3);
      if (e.second > 0) P->pos_plus[e.second - 1] = pos;
      else P->pos_minus[-e.second - 1] = pos;
    }
  for (int ig = 0; ig < ngw; ++ig)
    if (P->pos_minus[ig] < 0) P->pos_minus[ig] = P->pos_plus[ig];  // G = 0 is its own mirror
  return P;
}

void port_destroy(void* h) { delete static_cast<Port*>(h); }

// one 1D transform of length n (tests of the FFT itself)
int port_fft1(int n, double* x, int sign) {
  Fft1 p;
  if (!plan1(p, n)) return 7;
  std::vector<cd> work(n);
  fft1(p, reinterpret_cast<cd*>(x), work.data(), sign);
  return 0;
}

// rhoofr: rhoe (kr1, kr2, kr3) x fastest, ekin, csumg, csumr (any may be NULL)
int port_rhoofr(void* h, const double* c0d, int ldc, int nstate, const double* f, double* rhoe, double* ekin,
                double* csumg, double* csumr) {
  const Port& P = *static_cast<Port*>(h);
  const cd* c0 = reinterpret_cast<const cd*>(c0d);
  const int n1 = P.nr[0], n2 = P.nr[1], n3 = P.nr[2];
  const size_t nn = (size_t)n1 * n2 * n3;
  const int npairs = (nstate + 1) / 2;
  const int nth = std::max(1, std::min(P.nthreads, npairs));
  std::vector<Work> works(nth);
#pragma omp parallel num_threads(nth)
  {
    Work& w = works[omp_get_thread_num()];
    alloc_work(P, w, true);
    std::vector<cd> row(n1);
#pragma omp for schedule(dynamic)
    for (int ip = 0; ip < npairs; ++ip) {
      const int i1 = 2 * ip, i2 = i1 + 1;
      const bool two = i2 < nstate;
      pair_inverse_zy(P, c0 + (size_t)i1 * ldc, two ? c0 + (size_t)i2 * ldc : nullptr, w);
      const double f1 = f[i1] / P.omega, f2 = two ? f[i2] / P.omega : 0.0;
      for (int z = 0; z < n3; ++z)
        for (int y = 0; y < n2; ++y) {
          form_row(P, w, y, z, row.data());
          fft1(P.fx, row.data(), w.tmp.data(), +1);
          double* rr = w.rho.data() + (size_t)n1 * (y + (size_t)n2 * z);
          for (int x = 0; x < n1; ++x) rr[x] += f1 * row[x].real() * row[x].real() + f2 * row[x].imag() * row[x].imag();
        }
    }
  }
  double rsum = 0.0;
#pragma omp parallel for reduction(+ : rsum) schedule(static) num_threads(P.nthreads)
  for (int z = 0; z < P.kr[2]; ++z)
    for (int y = 0; y < P.kr[1]; ++y)
      for (int x = 0; x < P.kr[0]; ++x) {
        double v = 0.0;
        if (x < n1 && y < n2 && z < n3) {
          const size_t i = x + (size_t)n1 * (y + (size_t)n2 * z);
          for (int t = 0; t < nth; ++t) v += works[t].rho[i];
        }
        rhoe[x + (size_t)P.kr[0] * (y + (size_t)P.kr[1] * z)] = v;
        rsum += v;
      }
  double ek = 0.0, cg = 0.0;
  if (ekin || csumg) kin_norm(P, c0, ldc, nstate, f, &ek, &cg);
  if (ekin) *ekin = ek;
  if (csumg) *csumg = cg;
  if (csumr) *csumr = rsum * P.omega / (double)nn;
  return 0;
}

// vpsi: c2 += -f/2 (tpiba2 hg c0 + FFT[V psi]) for all states; vpot (kr1, kr2, kr3)
int port_vpsi(void* h, const double* c0d, int ldc, double* c2d, int ldc2, const double* f, const double* vpot,
              int nstate) {
  const Port& P = *static_cast<Port*>(h);
  const cd* c0 = reinterpret_cast<const cd*>(c0d);
  cd* c2 = reinterpret_cast<cd*>(c2d);
  const int n1 = P.nr[0], n2 = P.nr[1], n3 = P.nr[2];
  const double scale = 1.0 / ((double)n1 * n2 * n3);
  const int npairs = (nstate + 1) / 2;
  const int nth = std::max(1, std::min(P.nthreads, npairs));
#pragma omp parallel num_threads(nth)
  {
    Work w;
    alloc_work(P, w, false);
    std::vector<cd> row(n1);
#pragma omp for schedule(dynamic)
    for (int ip = 0; ip < npairs; ++ip) {
      const int i1 = 2 * ip, i2 = i1 + 1;
      const bool two = i2 < nstate;
      pair_inverse_zy(P, c0 + (size_t)i1 * ldc, two ? c0 + (size_t)i2 * ldc : nullptr, w);
      // x-rows: inverse, x V(r), forward, keep the sphere's x range
      for (int z = 0; z < n3; ++z)
        for (int y = 0; y < n2; ++y) {
          form_row(P, w, y, z, row.data());
          fft1(P.fx, row.data(), w.tmp.data(), +1);
          const double* vr = vpot + (size_t)P.kr[0] * (y + (size_t)P.kr[1] * z);
          for (int x = 0; x < n1; ++x) row[x] *= vr[x];
          fft1(P.fx, row.data(), w.tmp.data(), -1);
          for (int s = 0; s < P.nslot; ++s)
            w.yb[((size_t)z * P.nslot + s) * n2 + y] = row[fidx(P.gxlo + s, n1)];
        }
      // forward y-lines, keep the sphere columns
      for (int z = 0; z < n3; ++z)
        for (int s = 0; s < P.nslot; ++s) {
          cd* yl = w.yb.data() + ((size_t)z * P.nslot + s) * n2;
          fft1(P.fy, yl, w.tmp.data(), -1);
          for (int col : P.slot_cols[s]) w.zc[(size_t)col * n3 + z] = yl[fidx(P.col_gy[col], n2)];
        }
      // forward z-lines of the columns (scaled 1/N at the last pass)
      for (int col = 0; col < P.ncol; ++col) {
        cd* zl = w.zc.data() + (size_t)col * n3;
        fft1(P.fz, zl, w.tmp.data(), -1);
        for (int z = 0; z < n3; ++z) zl[z] *= scale;
      }
      // decode fp = Q(+G) + Q(-G), fm = Q(+G) - Q(-G) (vpsi_utils.mod.F90:661-671)
      double fi1 = f[i1] * 0.5, fi2 = two ? f[i2] * 0.5 : 0.0;
      if (fi1 == 0.0) fi1 = 1.0;
      if (fi2 == 0.0) fi2 = 1.0;
      const cd* a1 = c0 + (size_t)i1 * ldc;
      cd* o1 = c2 + (size_t)i1 * ldc2;
      for (int ig = 0; ig < P.ngw; ++ig) {
        const cd qp = w.zc[P.pos_plus[ig]], qm = w.zc[P.pos_minus[ig]];
        const double kin = P.tpiba2 * P.hg[ig];
        o1[ig] -= fi1 * (kin * a1[ig] + cd(qp.real() + qm.real(), qp.imag() - qm.imag()));
        if (two) {
          const cd* a2 = c0 + (size_t)i2 * ldc;
          cd* o2 = c2 + (size_t)i2 * ldc2;
          o2[ig] -= fi2 * (kin * a2[ig] + cd(qp.imag() + qm.imag(), qm.real() - qp.real()));
        }
      }
    }
  }
  return 0;
}

// Gram-Schmidt ortho in place (rgs); returns 2 when S is not positive definite
int port_rgs(void* h, double* c0d, int ldc, int nstate) {
  const Port& P = *static_cast<Port*>(h);
  const int n = nstate, K = 2 * P.ngw, lda = 2 * ldc;
  std::vector<double> S((size_t)n * n);
  syrk_t(c0d, lda, K, n, S.data(), P.nthreads);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double v = 2.0 * S[(size_t)i * n + j];
      if (P.geq0) v -= c0d[(size_t)i * lda] * c0d[(size_t)j * lda];
      S[(size_t)i * n + j] = v;
    }
  // S = U^T U (upper U, row-major U[i][j], j >= i)
  std::vector<double> U((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double d = S[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) d -= U[(size_t)k * n + j] * U[(size_t)k * n + j];
    if (!(d > 0.0)) return 2;
    const double ujj = std::sqrt(d);
    U[(size_t)j * n + j] = ujj;
    for (int i = j + 1; i < n; ++i) {
      double v = S[(size_t)j * n + i];
      for (int k = 0; k < j; ++k) v -= U[(size_t)k * n + j] * U[(size_t)k * n + i];
      U[(size_t)j * n + i] = v / ujj;
    }
  }
  // X = U^-1 (upper), column by column: U X = I
  std::vector<double> X((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    X[(size_t)j * n + j] = 1.0 / U[(size_t)j * n + j];
    for (int i = j - 1; i >= 0; --i) {
      double v = 0.0;
      for (int k = i + 1; k <= j; ++k) v += U[(size_t)i * n + k] * X[(size_t)k * n + j];
      X[(size_t)i * n + j] = -v / U[(size_t)i * n + i];
    }
  }
  // C <- C X over row blocks of the real view
  constexpr int RB = 64;
  const int nrb = (K + RB - 1) / RB;
#pragma omp parallel num_threads(P.nthreads)
  {
    std::vector<double> a((size_t)RB * n), o((size_t)RB * n);
#pragma omp for schedule(static)
    for (int b = 0; b < nrb; ++b) {
      const int k0 = b * RB, kb = std::min(RB, K - k0);
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < kb; ++k) a[(size_t)k * n + j] = c0d[(size_t)j * lda + k0 + k];
      std::fill(o.begin(), o.end(), 0.0);
      for (int k = 0; k < kb; ++k) {
        double* ok = o.data() + (size_t)k * n;
        const double* ak = a.data() + (size_t)k * n;
        for (int i = 0; i < n; ++i) {
          const double v = ak[i];
          const double* xi = X.data() + (size_t)i * n;
          for (int j = i; j < n; ++j) ok[j] += v * xi[j];
        }
      }
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < kb; ++k) c0d[(size_t)j * lda + k0 + k] = o[(size_t)k * n + j];
    }
  }
  if (P.geq0)
    for (int j = 0; j < n; ++j) c0d[(size_t)j * lda + 1] = 0.0;  // zclean
  return 0;
}

int port_threads(void* h) { return static_cast<Port*>(h)->nthreads; }

}  // extern "C"
