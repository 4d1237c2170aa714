// C ABI of the GB300 wavefunction hot path (declared in include/cpmd_gb300.h).
//
// The context replaces the reference's FFT set-up (fftprp_utils.mod.F90:
// 116-330 builds the ray maps nzh/indz/msp; fftnew_utils.mod.F90:101-170
// copies them to the device) and the module singletons cp_cufft/cp_curho/
// cp_cuvpsi (per-stream device buffers).  The maps here describe the
// sphere column by column for the pruned 3D FFT of band.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/cpmd_gb300.h"
#include "ctx.h"
#include "fs_plan.h"

namespace gbcp {

std::atomic<long long> g_launches{0};

bool ensure(Ctx& c, Scratch& s, size_t bytes) {
  if (bytes <= s.cap && s.p) return true;
  if (&s == &c.st_c0) c.wfn.valid = false;  // a new buffer holds no cached wavefunction
  if (&s == &c.zbuf) {  // nor a kept Z stage
    c.zk.valid = false;
    c.zk_skip = nullptr;
    c.zk_host = false;
  }
  if (s.p) {
    cudaStreamSynchronize(c.stream);
    cudaFree(s.p);
    s.p = nullptr;
    s.cap = 0;
  }
  if (bytes == 0) bytes = 16;
  if (cudaMalloc(&s.p, bytes) != cudaSuccess) {
    cudaGetLastError();
    s.p = nullptr;
    return false;
  }
  s.cap = bytes;
  return true;
}

static cudaEvent_t pool_event(Ctx& c) {
  if (!c.prof_pool.empty()) {
    cudaEvent_t e = c.prof_pool.back();
    c.prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(Ctx& ctx, const char* name) : c(ctx), on(ctx.prof), s(ctx.stream) {
  if (!on) return;
  r.name = name;
  r.lane = 0;
  r.a = pool_event(c);
  r.b = pool_event(c);
  cudaEventRecord(r.a, s);
}

ProfScope::ProfScope(Ctx& ctx, const char* name, cudaStream_t stream, int lane)
    : c(ctx), on(ctx.prof), s(stream) {
  if (!on) return;
  r.name = name;
  r.lane = lane;
  r.a = pool_event(c);
  r.b = pool_event(c);
  cudaEventRecord(r.a, s);
}

ProfScope::~ProfScope() {
  if (!on) return;
  cudaEventRecord(r.b, s);
  c.prof_live.push_back(r);
}

void prof_fold(Ctx& c) {
  if (c.prof_live.empty()) return;
  cudaStreamSynchronize(c.stream);
  if (c.copy) cudaStreamSynchronize(c.copy);
  if (c.copy_out) cudaStreamSynchronize(c.copy_out);
  if (c.side) cudaStreamSynchronize(c.side);
  for (ProfRec& r : c.prof_live) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    if (c.prof_base) {
      float t0 = 0.f, t1 = 0.f;
      cudaEventElapsedTime(&t0, c.prof_base, r.a);
      cudaEventElapsedTime(&t1, c.prof_base, r.b);
      c.prof_tl.push_back({r.name, r.lane, t0, t1});
    }
    bool found = false;
    for (auto& kv : c.prof_acc) {
      if (kv.first == r.name) {
        kv.second.ms += ms;
        kv.second.n += 1;
        found = true;
        break;
      }
    }
    if (!found) {
      ProfAcc a;
      a.ms = ms;
      a.n = 1;
      c.prof_acc.push_back({r.name, a});
    }
    c.prof_pool.push_back(r.a);
    c.prof_pool.push_back(r.b);
  }
  c.prof_live.clear();
}

static void release(Scratch& s) {
  if (s.p) cudaFree(s.p);
  s.p = nullptr;
  s.cap = 0;
}

// Factor n into radices 8, 5, 4, 3, 2 (largest first).  0 if n has a prime
// factor above 5 (the reference's own FFT tables hold 2,3,5-smooth sizes only,
// gfft_utils.mod.F90:39-84).
static bool make_plan(int n, FftPlan& p) {
  p.n = n;
  p.npass = 0;
  int m = n;
  const int rad[5] = {8, 5, 4, 3, 2};
  while (m > 1) {
    bool found = false;
    for (int r : rad) {
      if (m % r == 0) {
        if (p.npass >= kMaxPasses) return false;
        p.radix[p.npass++] = r;
        m /= r;
        found = true;
        break;
      }
    }
    if (!found) return false;
  }
  if (p.npass == 0) {  // n == 1
    return false;
  }
  return true;
}

template <typename T> static bool upload(Ctx& c, const std::vector<T>& h, const T*& dptr) {
  void* p = nullptr;
  const size_t bytes = std::max<size_t>(sizeof(T) * h.size(), 16);
  if (cudaMalloc(&p, bytes) != cudaSuccess) return false;
  if (!h.empty() && cudaMemcpy(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) return false;
  c.dev_allocs.push_back(p);
  dptr = static_cast<const T*>(p);
  return true;
}

static int build_geometry(Ctx& c, const int32_t* inyh, const double* hg) {
  const int n[3] = {c.nr[0], c.nr[1], c.nr[2]};
  const int ngw = c.ngw;
  struct Pt {
    int gx, gy, gz, ent;
  };
  std::vector<Pt> pts;
  pts.reserve(2 * (size_t)ngw);
  for (int ig = 0; ig < ngw; ++ig) {
    int m[3];
    for (int a = 0; a < 3; ++a) {
      m[a] = inyh[3 * (size_t)ig + a] - (n[a] / 2 + 1);
      if (2 * std::abs(m[a]) >= n[a]) {
        c.err = "inyh: G vector " + std::to_string(ig) + " outside the mesh";
        return 1;
      }
    }
    pts.push_back({m[0], m[1], m[2], ig + 1});
    if (m[0] != 0 || m[1] != 0 || m[2] != 0) pts.push_back({-m[0], -m[1], -m[2], -(ig + 1)});
  }
  // columns keyed by (gx, gy)
  std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> cols;
  for (const Pt& p : pts) cols[{p.gx, p.gy}].push_back({p.gz, p.ent});
  // slots: gx range and per gx the gy range (dense, holes allowed)
  std::map<int, std::pair<int, int>> gyr;
  for (auto& kv : cols) {
    const int gx = kv.first.first, gy = kv.first.second;
    auto it = gyr.find(gx);
    if (it == gyr.end()) gyr[gx] = {gy, gy};
    else it->second = {std::min(it->second.first, gy), std::max(it->second.second, gy)};
  }
  const int gxlo = gyr.begin()->first, gxhi = gyr.rbegin()->first;
  const int nslot = gxhi - gxlo + 1;
  std::vector<int> slot_col0(nslot, 0), slot_gylo(nslot, 0), slot_ncol(nslot, 0);
  std::vector<int> col_start, col_zlo, col_ent, col_slot, col_gy, ent_col;
  std::vector<int> pos_plus(ngw, -1), pos_minus(ngw, -1);
  int ncol = 0;
  for (int s = 0; s < nslot; ++s) {
    const int gx = gxlo + s;
    slot_col0[s] = ncol;
    auto it = gyr.find(gx);
    if (it == gyr.end()) continue;  // empty slot (hole in gx)
    slot_gylo[s] = it->second.first;
    slot_ncol[s] = it->second.second - it->second.first + 1;
    for (int gy = it->second.first; gy <= it->second.second; ++gy) {
      col_start.push_back((int)col_ent.size());
      col_slot.push_back(s);
      col_gy.push_back(gy);
      auto ci = cols.find({gx, gy});
      if (ci == cols.end()) {
        col_zlo.push_back(0);
      } else {
        int zlo = 1 << 30, zhi = -(1 << 30);
        for (auto& e : ci->second) {
          zlo = std::min(zlo, e.first);
          zhi = std::max(zhi, e.first);
        }
        col_zlo.push_back(zlo);
        const int base = (int)col_ent.size();
        col_ent.resize(base + (zhi - zlo + 1), 0);
        ent_col.resize(col_ent.size(), ncol);
        for (auto& e : ci->second) {
          const int pos = base + (e.first - zlo);
          if (col_ent[pos] != 0) {
            c.err = "inyh: duplicate G vector";
            return 1;
          }
          col_ent[pos] = e.second;
          if (e.second > 0) pos_plus[e.second - 1] = pos;
          else pos_minus[-e.second - 1] = pos;
        }
      }
      ++ncol;
    }
  }
  col_start.push_back((int)col_ent.size());
  for (int ig = 0; ig < ngw; ++ig)
    if (pos_minus[ig] < 0) pos_minus[ig] = pos_plus[ig];  // G = 0 is its own mirror
  std::vector<double> hgv(hg, hg + ngw);
  std::vector<float> hg32v(hg, hg + ngw);
  // the four-step Z-stage gather table: one coalesced load per (line, z) instead of
  // col_start -> col_ent -> c0, and hg(|G|) of the entry without a gather of its own
  std::vector<int2> zgat;
  {
    const int N = n[2], N1 = gbcp::fs_n1(N), L = gbcp::fs_lines(N);
    if (N1 > 0) {
      const int N2 = N / N1, nblk = (ncol + L - 1) / L, h = (N + 1) / 2;
      zgat.assign((size_t)nblk * N * L, int2{0, 0});
      for (int b = 0; b < nblk; ++b)
        for (int n1 = 0; n1 < N1; ++n1)
          for (int n2 = 0; n2 < N2; ++n2)
            for (int l = 0; l < L; ++l) {
              const int col = b * L + l;
              if (col >= ncol) continue;
              const int i = n2 + N2 * n1, fz = i < h ? i : i - N;
              const int st = col_start[col], len = col_start[col + 1] - st, off = fz - col_zlo[col];
              if (off < 0 || off >= len) continue;
              const int e = col_ent[st + off];
              const float hge = e != 0 ? hg32v[(e > 0 ? e : -e) - 1] : 0.0f;
              int bits;
              std::memcpy(&bits, &hge, sizeof(bits));
              zgat[(((size_t)b * N1 + n1) * N2 + n2) * L + l] = int2{e, bits};
            }
    }
  }
  GeoDev& g = c.geo;
  g.geq0 = c.geq0;
  g.n1 = n[0];
  g.n2 = n[1];
  g.n3 = n[2];
  g.k1 = c.kr[0];
  g.k2 = c.kr[1];
  g.ngw = ngw;
  g.ncol = ncol;
  g.nslot = nslot;
  g.gxlo = gxlo;
  g.nent = (int)col_ent.size();
  {
    int gymin = 1 << 30, gymax = -(1 << 30);
    for (int cc = 0; cc < ncol; ++cc) {
      gymin = std::min(gymin, col_gy[cc]);
      gymax = std::max(gymax, col_gy[cc]);
    }
    g.prune_x = n[0] % 4 == 0 && gxlo >= -n[0] / 4 && gxlo + nslot - 1 <= n[0] / 4 - 1;
    g.prune_y = n[1] % 4 == 0 && gymin >= -n[1] / 4 && gymax <= n[1] / 4 - 1;
  }
  g.yblk_cols = ncol;
  if (gbcp::fs_lines(n[1]) > 0) {
    const int L = gbcp::fs_lines(n[1]);
    g.yblk_cols = 0;
    for (int sb = 0; sb < nslot; sb += L) {
      const int ce = sb + L < nslot ? slot_col0[sb + L] : ncol;
      g.yblk_cols = std::max(g.yblk_cols, ce - slot_col0[sb]);
    }
  }
  if (!upload(c, col_start, g.col_start) || !upload(c, col_zlo, g.col_zlo) || !upload(c, col_ent, g.col_ent) ||
      !upload(c, col_slot, g.col_slot) || !upload(c, col_gy, g.col_gy) || !upload(c, ent_col, g.ent_col) ||
      !upload(c, slot_col0, g.slot_col0) || !upload(c, slot_gylo, g.slot_gylo) ||
      !upload(c, slot_ncol, g.slot_ncol) || !upload(c, pos_plus, g.pos_plus) || !upload(c, pos_minus, g.pos_minus) ||
      !upload(c, hgv, g.hg) || !upload(c, hg32v, g.hg32) || (!zgat.empty() && !upload(c, zgat, g.zgat))) {
    c.err = "geometry upload failed";
    return 6;
  }
  std::vector<double> kin(ngw);
  for (int ig = 0; ig < ngw; ++ig) kin[ig] = c.tpiba2 * hg[ig];
  const double* dk = nullptr;
  if (!upload(c, kin, dk)) {
    c.err = "geometry upload failed";
    return 6;
  }
  c.kin = const_cast<double*>(dk);
  std::vector<short4> wm(ngw);
  for (int ig = 0; ig < ngw; ++ig)
    wm[ig] = make_short4((short)(inyh[3 * (size_t)ig] - (n[0] / 2 + 1)), (short)(inyh[3 * (size_t)ig + 1] - (n[1] / 2 + 1)),
                         (short)(inyh[3 * (size_t)ig + 2] - (n[2] / 2 + 1)), 0);
  const short4* dwm = nullptr;
  if (!upload(c, wm, dwm)) {
    c.err = "geometry upload failed";
    return 6;
  }
  c.wmill = dwm;
  return 0;
}

static int build_fft(Ctx& c) {
  for (int a = 0; a < 3; ++a) {
    if (!make_plan(c.nr[a], c.plan[a])) {
      c.err = "mesh size " + std::to_string(c.nr[a]) + " is not 2,3,5-smooth";
      return 7;
    }
    const int n = c.nr[a];
    std::vector<cx<double>> t64(n);
    std::vector<cx<float>> t32(n);
    for (int m = 0; m < n; ++m) {
      // FP64 host trigonometry; the quarter points are set exactly
      const double ang = 2.0 * M_PI * (double)m / (double)n;
      t64[m] = mk<double>(std::cos(ang), std::sin(ang));
      if (4 * m == n) t64[m] = mk<double>(0.0, 1.0);
      if (2 * m == n) t64[m] = mk<double>(-1.0, 0.0);
      if (4 * m == 3 * n) t64[m] = mk<double>(0.0, -1.0);
      t32[m] = mk<float>((float)t64[m].x, (float)t64[m].y);
    }
    const cx<double>* d64;
    const cx<float>* d32;
    if (!upload(c, t64, d64) || !upload(c, t32, d32)) {
      c.err = "twiddle upload failed";
      return 6;
    }
    c.tw64[a] = const_cast<cx<double>*>(d64);
    c.tw32[a] = const_cast<cx<float>*>(d32);
    const int n1 = fs_n1(n);
    if (n1 > 0) {
      const int n2 = n / n1;
      std::vector<cx<double>> a64(n), b64(n);
      std::vector<cx<float>> a32(n), b32(n);
      for (int k1 = 0; k1 < n1; ++k1)
        for (int j = 0; j < n2; ++j) {
          const cx<double> w = t64[(k1 * j) % n];
          a64[k1 * n2 + j] = w;
          b64[j * n1 + k1] = w;
          a32[k1 * n2 + j] = mk<float>((float)w.x, (float)w.y);
          b32[j * n1 + k1] = mk<float>((float)w.x, (float)w.y);
        }
      const cx<double>*pa64, *pb64;
      const cx<float>*pa32, *pb32;
      if (!upload(c, a64, pa64) || !upload(c, b64, pb64) || !upload(c, a32, pa32) || !upload(c, b32, pb32)) {
        c.err = "twiddle upload failed";
        return 6;
      }
      c.twA64[a] = const_cast<cx<double>*>(pa64);
      c.twB64[a] = const_cast<cx<double>*>(pb64);
      c.twA32[a] = const_cast<cx<float>*>(pa32);
      c.twB32[a] = const_cast<cx<float>*>(pb32);
    }
  }
  return 0;
}

}  // namespace gbcp

using gbcp::Ctx;
using gbcp::cx;


static int set_err(gbcp_ctx* h, int rc, const char* msg) {
  if (h && msg) h->c.err = msg;
  return rc;
}

extern "C" {

int gbcp_ctx_create(const gbcp_grid_desc* grid, int precision, int max_batch, void* stream, gbcp_ctx** out) {
  if (!grid || !out || !grid->inyh || !grid->hg) return GBCP_ERR_ARG;
  if (grid->nr1 < 2 || grid->nr2 < 2 || grid->nr3 < 2 || grid->kr1 < grid->nr1 || grid->kr2 < grid->nr2 ||
      grid->kr3 < grid->nr3 || grid->ngw < 1 || !(grid->omega > 0) || !(grid->tpiba2 > 0))
    return GBCP_ERR_ARG;
  if (precision != GBCP_PREC_FP64 && precision != GBCP_PREC_MIXED) return GBCP_ERR_ARG;
  gbcp_ctx* h = new gbcp_ctx();
  Ctx& c = h->c;
  c.nr[0] = grid->nr1;
  c.nr[1] = grid->nr2;
  c.nr[2] = grid->nr3;
  c.kr[0] = grid->kr1;
  c.kr[1] = grid->kr2;
  c.kr[2] = grid->kr3;
  c.ngw = grid->ngw;
  c.geq0 = grid->geq0 ? 1 : 0;
  c.omega = grid->omega;
  c.tpiba2 = grid->tpiba2;
  c.precision = precision;
  c.batch = std::min(gbcp::kMaxBatch, max_batch > 0 ? max_batch : gbcp::kMaxBatch);
  if (cudaStreamCreateWithFlags(&c.own, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return GBCP_ERR_CUDA;
  }
  c.stream = stream ? static_cast<cudaStream_t>(stream) : c.own;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c.nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  int rc = gbcp::build_geometry(c, grid->inyh, grid->hg);
  if (!rc) rc = gbcp::build_fft(c);
  if (!rc && cudaMalloc(&c.d_info, 16) != cudaSuccess) rc = GBCP_ERR_NOMEM;
  if (rc) {
    fprintf(stderr, "gbcp_ctx_create: %s\n", c.err.c_str());
    gbcp_ctx_destroy(h);
    return rc;
  }
  *out = h;
  return GBCP_OK;
}

int gbcp_ctx_destroy(gbcp_ctx* h) {
  if (!h) return GBCP_OK;
  Ctx& c = h->c;
  if (c.stream) cudaStreamSynchronize(c.stream);
  for (void* p : c.dev_allocs) cudaFree(p);
  gbcp::Scratch* all[] = {&c.zbuf, &c.ybuf, &c.qbuf, &c.st_c0, &c.st_c2, &c.st_rho, &c.st_vpot, &c.st_f,
                          &c.st_misc, &c.st_misc2, &c.st_vf, &c.red, &c.red2, &c.smat, &c.smat2, &c.smat3, &c.sparts, &c.cscr, &c.cdiag, &c.cwork, &c.xr_part, &c.xr_tk, &c.rt_mats, &c.en_g3, &c.oz_a, &c.oz_b,
                          &c.nl_a, &c.nl_b, &c.nl_c, &c.nl_d, &c.nl_ta, &c.nl_tb, &c.nl_tp, &c.en_rho, &c.en_a, &c.en_b, &c.en_veff,
                          &c.en_red, &c.en_ei, &c.en_fp, &c.en_idx, &c.en_in[0], &c.en_in[1], &c.en_in[2],
                          &c.en_in[3], &c.en_in[4], &c.oz_c, &c.oz_rmax, &c.rho_sc, &c.rho_tk, &c.zk_sum};
  for (auto* s : all) gbcp::release(*s);
  for (cudaStream_t* st : {&c.copy, &c.copy_out, &c.side})
    if (*st) {
      cudaStreamSynchronize(*st);
      cudaStreamDestroy(*st);
    }
  for (cudaEvent_t e : c.pipe_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : c.side_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : c.col_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : c.zk_ev)
    if (e) cudaEventDestroy(e);
  if (c.d_info) cudaFree(c.d_info);
  gbcp::prof_fold(c);
  for (cudaEvent_t e : c.prof_pool) cudaEventDestroy(e);
  if (c.prof_base) cudaEventDestroy(c.prof_base);
  if (c.own) {
    cudaStreamSynchronize(c.own);
    cudaStreamDestroy(c.own);
  }
  delete h;
  return GBCP_OK;
}

int gbcp_set_precision(gbcp_ctx* h, int precision) {
  if (!h || (precision != GBCP_PREC_FP64 && precision != GBCP_PREC_MIXED)) return GBCP_ERR_ARG;
  h->c.precision = precision;
  return GBCP_OK;
}

int gbcp_set_option(gbcp_ctx* h, int key, int value) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (key == GBCP_OPT_GEMM && value >= -1 && value <= 1) {
    c.gemm_mode = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_BATCH && value > 0 && value <= gbcp::kMaxBatch) {
    c.batch = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_FFT && (value == 0 || value == 2)) {
    c.fft_engine = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_ZMIRROR && value >= -1 && value <= 1) {
    c.zmirror = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_ORTHO_COLUMNS && (value == 0 || value == 1)) {
    c.ortho_cols = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_ZKEEP && (value == 0 || value == 1)) {
    c.zkeep = value;
    c.zk.valid = false;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_STAGES && value >= 0) {
    c.stage_first = value & 0xFF;
    c.stage_n = (value >> 8) & 0xFF;
    c.stage_groups = (value >> 16) & 0xFF;
    c.stage_last = (value >> 24) & 0x7F;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_XCHUNKS && value >= 0 && value <= 8) {
    c.xr_chunks = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_XC && (value == 0 || value == 1)) {
    c.xc = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_PLANE && value >= 0 && value <= 3) {
    c.plane = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_SIMT_TILE && (value == 32 || value == 64)) {
    c.simt_tile = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_CHOL && value >= 0 && value <= 3) {
    c.chol_df = value;
    return GBCP_OK;
  }
  if (key == GBCP_OPT_WFN_CACHE && (value == 0 || value == 1)) {
    c.wfn.on = value == 1;
    c.wfn.valid = false;  // setting the option always drops a kept copy
    return GBCP_OK;
  }
  if (key == GBCP_OPT_TEST_TIMEOUT && (value == 0 || value == 1)) {
    c.test_stall = value;
    return GBCP_OK;
  }
  return set_err(h, GBCP_ERR_ARG, "set_option: unknown key or value");
}

int gbcp_set_stream(gbcp_ctx* h, void* stream) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.own;
  if (s == c.stream) return GBCP_OK;
  gbcp::prof_fold(c);
  c.stream = s;
  return GBCP_OK;
}

int gbcp_synchronize(gbcp_ctx* h) {
  if (!h) return GBCP_ERR_ARG;
  cudaError_t e = cudaStreamSynchronize(h->c.stream);
  if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
  return GBCP_OK;
}

int gbcp_last_error(gbcp_ctx* h, char* buf, int len) {
  if (!h || !buf || len <= 0) return GBCP_ERR_ARG;
  snprintf(buf, (size_t)len, "%s", h->c.err.c_str());
  return GBCP_OK;
}

int64_t gbcp_kernel_launches(void) { return (int64_t)gbcp::g_launches.load(); }

int gbcp_profile_enable(gbcp_ctx* h, int enable) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  gbcp::prof_fold(c);
  c.prof_acc.clear();
  c.prof_tl.clear();
  c.prof = enable != 0;
  if (c.prof) {
    if (!c.prof_base && cudaEventCreate(&c.prof_base) != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, "profile event");
    cudaEventRecord(c.prof_base, c.stream);
  }
  return GBCP_OK;
}

int gbcp_profile_timeline(gbcp_ctx* h, int idx, char* name, int name_len, int* lane, double* t0_ms, double* t1_ms) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  gbcp::prof_fold(c);
  if (idx < 0 || idx >= (int)c.prof_tl.size()) return GBCP_ERR_ARG;
  const gbcp::TimelineRec& r = c.prof_tl[(size_t)idx];
  if (name && name_len > 0) snprintf(name, (size_t)name_len, "%s", r.name.c_str());
  if (lane) *lane = r.lane;
  if (t0_ms) *t0_ms = r.t0;
  if (t1_ms) *t1_ms = r.t1;
  return GBCP_OK;
}

int gbcp_profile_read(gbcp_ctx* h, int idx, char* name, int name_len, double* total_ms, int64_t* count) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  gbcp::prof_fold(c);
  if (idx < 0 || idx >= (int)c.prof_acc.size()) return GBCP_ERR_ARG;
  const auto& kv = c.prof_acc[(size_t)idx];
  if (name && name_len > 0) snprintf(name, (size_t)name_len, "%s", kv.first.c_str());
  if (total_ms) *total_ms = kv.second.ms;
  if (count) *count = kv.second.n;
  return GBCP_OK;
}

}  // extern "C"

namespace {

using gbcp::Scratch;

// Stage a host (ngw x n, leading dim ld) complex array into packed device memory.
// ---- the wavefunction cache (see WfnCache) ----
// the reference's key, SUM(ABS(c0(:,1))) (rhoofr_utils.mod.F90:244)
// (the moduli by sqrt(re^2 + im^2), four running sums: std::hypot took ~0.3 ms for
// 43k coefficients, on the host between the calls of every step)
double wfn_key(const double* h, int rows) {
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  int i = 0;
  for (; i + 4 <= rows; i += 4)
    for (int u = 0; u < 4; ++u) {
      const double re = h[2 * (size_t)(i + u)], im = h[2 * (size_t)(i + u) + 1];
      s[u] += std::sqrt(re * re + im * im);
    }
  for (; i < rows; ++i) s[0] += std::sqrt(h[2 * (size_t)i] * h[2 * (size_t)i] + h[2 * (size_t)i + 1] * h[2 * (size_t)i + 1]);
  return (s[0] + s[1]) + (s[2] + s[3]);
}
// every part of the key but the host pass over c0(:,1)
bool wfn_maybe(const Ctx& c, const double* h, int ld, int n) {
  const gbcp::WfnCache& w = c.wfn;
  return w.on && w.valid && w.host == h && w.ldc == ld && w.n == n && w.dev == c.st_c0.p;
}
bool wfn_hit(Ctx& c, const double* h, int ld, int n) { return wfn_maybe(c, h, ld, n) && wfn_key(h, c.ngw) == c.wfn.key; }
void wfn_put(Ctx& c, const double* h, int ld, int n) {
  gbcp::WfnCache& w = c.wfn;
  if (!w.on) return;
  w.valid = true;
  w.host = h;
  w.dev = c.st_c0.p;
  w.ldc = ld;
  w.n = n;
  w.key = wfn_key(h, c.ngw);
}

int stage_in_cx(Ctx& c, Scratch& s, const double* h, int ld, int rows, int n, cx<double>** d) {
  if (&s == &c.st_c0) c.wfn.valid = false;  // the cached copy is overwritten
  const size_t bytes = sizeof(cx<double>) * (size_t)rows * n;
  if (!gbcp::ensure(c, s, bytes)) return GBCP_ERR_NOMEM;
  *d = static_cast<cx<double>*>(s.p);
  if (n > 0) {
    gbcp::ProfScope ps_(c, "h2d_states", c.stream, 1);
    GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(s.p, sizeof(cx<double>) * rows, h, sizeof(cx<double>) * (size_t)ld,
                                       sizeof(cx<double>) * rows, n, cudaMemcpyHostToDevice, c.stream));
  }
  return 0;
}

int stage_out_cx(Ctx& c, const cx<double>* d, double* h, int ld, int rows, int n) {
  if (n > 0) {
    gbcp::ProfScope ps_(c, "d2h_states", c.stream, 2);
    GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(h, sizeof(cx<double>) * (size_t)ld, d, sizeof(cx<double>) * rows,
                                       sizeof(cx<double>) * rows, n, cudaMemcpyDeviceToHost, c.stream));
  }
  return 0;
}

int stage_in(Ctx& c, Scratch& s, const void* h, size_t bytes, void** d) {
  if (!gbcp::ensure(c, s, bytes)) return GBCP_ERR_NOMEM;
  *d = s.p;
  if (bytes) GBCP_CUDA_TRY(c, cudaMemcpyAsync(s.p, h, bytes, cudaMemcpyHostToDevice, c.stream));
  return 0;
}

// Host-memory calls of the band loop overlap their copies with the compute: the
// states go up per band-loop batch on a second stream, and each batch waits only
// for its own columns (and, for vpsi, sends its C2 columns back while the next
// batch computes).  Ordered after earlier work on the context stream.
int pipe_prepare(Ctx& c, int nbatch) {
  if ((!c.copy && cudaStreamCreateWithFlags(&c.copy, cudaStreamNonBlocking) != cudaSuccess) ||
      (!c.copy_out && cudaStreamCreateWithFlags(&c.copy_out, cudaStreamNonBlocking) != cudaSuccess)) {
    c.err = "copy streams";
    return GBCP_ERR_CUDA;
  }
  const size_t need = 2 * (size_t)nbatch + 2;
  while (c.pipe_ev.size() < need) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      c.err = "pipeline events";
      return GBCP_ERR_CUDA;
    }
    c.pipe_ev.push_back(e);
  }
  GBCP_CUDA_TRY(c, cudaEventRecord(c.pipe_ev[0], c.stream));
  GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.copy, c.pipe_ev[0], 0));
  return 0;
}

// upload states [s0, s0 + ns) of a host (ld) array into the packed device array d (rows = ngw)
int pipe_up(Ctx& c, cx<double>* d, const double* h, int ld, int s0, int ns) {
  gbcp::ProfScope ps_(c, "h2d_states", c.copy, 1);
  GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(d + (size_t)s0 * c.ngw, sizeof(cx<double>) * c.ngw,
                                     h + 2 * (size_t)s0 * ld, sizeof(cx<double>) * (size_t)ld,
                                     sizeof(cx<double>) * c.ngw, ns, cudaMemcpyHostToDevice, c.copy));
  return 0;
}

// pairs per staging chunk of a host-memory call: about four chunks, so that the whole
// stage chain of one chunk overlaps the copies of the next; host-memory calls launch the
// band loop chunk by chunk (their launch batch is the chunk)
// Staging chunks of a host-memory band-loop call, as pair ranges, each at most one
// launch batch.  vpsi: a small first chunk (its upload is the only one the
// transforms wait for), two large middle ones, and a small last one (its
// transforms and its C2 download are the tail nothing overlaps); with c0 already
// on the device, three chunks from large to small.  rhoofr: a small first chunk
// and three equal ones.  GBCP_OPT_STAGES fixes the plan for both.  Returns the
// number of chunks.
enum StageKind { STAGE_VPSI = 0, STAGE_RHOOFR = 1, STAGE_VPSI_CACHED = 2 };
int stage_plan(Ctx& c, int nstate, int kind) {
  const int npairs = (nstate + 1) / 2;
  std::vector<int>& b = c.stage_bounds;
  b.assign(1, 0);
  if (npairs <= 0) return 0;
  // rhoofr, whose transforms wait for c0 to land: a small first chunk, then three
  // equal ones (measured on the 128-state cell: 0.81 ms against 0.87 for the plan
  // below); vpsi with c0 already on the device, where only C2 moves: 3/8, 3/8 and
  // 1/4 of the pairs (1.07 ms against 1.11)
  const bool fixed = c.stage_n > 0;
  const int nfix = fixed ? c.stage_n : (kind == STAGE_RHOOFR ? 4 : kind == STAGE_VPSI_CACHED ? 3 : 0);
  if (nfix > 0) {
    // a fixed plan: the first chunk, then equal chunks of at most one launch batch
    const int f0 = fixed ? c.stage_first : kind == STAGE_RHOOFR ? npairs / 16 : (3 * npairs + 7) / 8;
    const int first = std::max(1, std::min({f0 > 0 ? f0 : npairs, npairs, c.batch}));
    b.push_back(first);
    // a fixed last chunk (GBCP_OPT_STAGES), the rest in equal chunks between
    const int l0 = fixed ? c.stage_last : kind == STAGE_VPSI_CACHED ? npairs / 4 : 0;
    const int lastc = std::min({l0, c.batch, std::max(0, npairs - first - 1)});
    const int rest = npairs - first - lastc;
    if (rest > 0) {
      const int k = std::max(std::max(1, nfix - 1 - (lastc > 0 ? 1 : 0)), (rest + c.batch - 1) / c.batch);
      for (int q = 1; q <= k; ++q) {
        const int e = first + (int)((long long)rest * q / k);
        if (e > b.back()) b.push_back(e);
      }
    }
    if (lastc > 0) b.push_back(npairs);
    return (int)b.size() - 1;
  }
  const int first = std::max(1, std::min(c.batch, npairs / 16));
  const int last = (npairs - first >= 3) ? std::max(1, std::min(c.batch, npairs / 6)) : 0;
  int p = first;
  b.push_back(p);
  const int mid = npairs - first - last;
  if (mid > 0) {
    const int per = std::min(c.batch, std::max(1, (mid + 1) / 2));
    for (int q = p + per; q < first + mid; q += per) b.push_back(q);
    b.push_back(first + mid);
  }
  if (last > 0) b.push_back(npairs);
  return (int)b.size() - 1;
}
int stage_max(const Ctx& c) {
  int m = 1;
  for (size_t q = 0; q + 1 < c.stage_bounds.size(); ++q) m = std::max(m, c.stage_bounds[q + 1] - c.stage_bounds[q]);
  return m;
}

int finish(Ctx& c, int rc) {
  if (rc) {
    if (c.err.empty()) c.err = "error";
    return rc;
  }
  cudaError_t e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) {
    c.err = cudaGetErrorString(e);
    return GBCP_ERR_CUDA;
  }
  return GBCP_OK;
}

bool bad_mem(int mem) { return mem != GBCP_MEM_HOST && mem != GBCP_MEM_DEVICE; }

}  // namespace

extern "C" {

// |csumr - csumg| allowed by rhoofr's charge check: the reference's delta = 1e-6
// (rhoofr_utils.mod.F90:625) in FP64; in the mixed mode, where rho comes from
// FP32 transforms, 1e-6 of the charge (the FP32 density agrees to ~1e-7 of it).
static double charge_tolerance(const gbcp::Ctx& c, double csumg) {
  return c.precision == GBCP_PREC_FP64 ? 1e-6 : 1e-6 * std::max(1.0, std::fabs(csumg));
}

int gbcp_rhoofr(gbcp_ctx* h, const double* c0, int ldc, int nstate, const double* f, double* rhoe, double* ekin,
                double* csumg, double* csumr, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate < 0 || (nstate > 0 && (!c0 || !f || ldc < c.ngw)) || !rhoe)
    return set_err(h, GBCP_ERR_ARG, "rhoofr: bad argument");
  c.err.clear();
  const size_t nnr1 = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  const cx<double>* dc0 = reinterpret_cast<const cx<double>*>(c0);
  const double* df = f;
  double* drho = rhoe;
  int dld = ldc;
  int rc = 0, saved_batch = 0;
  if (mem == GBCP_MEM_HOST) {
    void* tf;
    if ((rc = stage_in(c, c.st_f, f, sizeof(double) * nstate, &tf))) return rc;
    if (!gbcp::ensure(c, c.st_rho, sizeof(double) * nnr1) ||
        !gbcp::ensure(c, c.st_c0, sizeof(cx<double>) * (size_t)c.ngw * std::max(nstate, 1)))
      return GBCP_ERR_NOMEM;
    cx<double>* t = static_cast<cx<double>*>(c.st_c0.p);
    const int nb = stage_plan(c, nstate, STAGE_RHOOFR);
    if ((rc = pipe_prepare(c, nb + 2))) return rc;
    // events [nb + 1, nb + 2]: the two slabs of rho final; nb + 3: their downloads done.
    // The first slab 70 % of the planes: its download overlaps the rest, and each
    // launch stays a few full waves
    c.rho_slabs = 2;
    c.rho_zsplit = c.nr[2] * 7 / 10;
    c.rho_ev = c.pipe_ev.data() + nb + 1;
    const bool resident = wfn_hit(c, c0, ldc, nstate);
    for (int b = 0; b < nb; ++b) {
      const int s0 = 2 * c.stage_bounds[b], ns = std::min(2 * c.stage_bounds[b + 1], nstate) - s0;
      if (!resident && (rc = pipe_up(c, t, c0, ldc, s0, ns))) return rc;
      GBCP_CUDA_TRY(c, cudaEventRecord(c.pipe_ev[1 + b], c.copy));
    }
    c.batch_ready = c.pipe_ev.data() + 1;  // launch batches stay c.batch pairs (see rhoofr_t)
    dc0 = t;
    df = static_cast<double*>(tf);
    drho = static_cast<double*>(c.st_rho.p);
    dld = c.ngw;
  }
  // E_kin and csumg are summed inside the band loop's gather, csumr from the
  // density, all on the device; the host reads the three at the end
  const bool scalars = ekin || csumg || csumr;
  double* dsc = nullptr;
  if (scalars) {
    if (!gbcp::ensure(c, c.rho_sc, 4 * sizeof(double))) return GBCP_ERR_NOMEM;
    dsc = static_cast<double*>(c.rho_sc.p);
  }
  rc = gbcp::band_rhoofr(c, dc0, dld, nstate, df, drho, dsc);
  c.batch_ready = nullptr;
  const cudaEvent_t* slab_ev = c.rho_ev;
  c.rho_ev = nullptr;
  c.rho_slabs = 0;
  // the cache key (a host pass over c0's first column) once the GPU has its work
  if (mem == GBCP_MEM_HOST) wfn_put(c, c0, ldc, nstate);
  if (saved_batch) c.batch = saved_batch;
  if (!rc && mem == GBCP_MEM_HOST) {
    // rho back in two slabs of z planes on the download stream, each once final (the
    // second with the padding planes), beside the density scalars
    const size_t plane = (size_t)c.kr[0] * c.kr[1];
    for (int i = 0; i < 2; ++i) {
      const size_t p0 = i ? plane * (size_t)c.rho_zsplit : 0, p1 = i ? nnr1 : plane * (size_t)c.rho_zsplit;
      GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.copy_out, slab_ev[i], 0));
      gbcp::ProfScope ps_(c, "d2h_rho", c.copy_out, 2);
      GBCP_CUDA_TRY(c, cudaMemcpyAsync(rhoe + p0, drho + p0, sizeof(double) * (p1 - p0), cudaMemcpyDeviceToHost,
                                       c.copy_out));
    }
    GBCP_CUDA_TRY(c, cudaEventRecord(slab_ev[2], c.copy_out));
    GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, slab_ev[2], 0));
  }
  if (!rc && scalars) {
    double hs[3] = {0.0, 0.0, 0.0};
    GBCP_CUDA_TRY(c, cudaMemcpyAsync(hs, dsc, sizeof(hs), cudaMemcpyDeviceToHost, c.stream));
    GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    if (ekin) *ekin = hs[0];
    if (csumg) *csumg = hs[1];
    if (csumr) *csumr = hs[2];
    if (!std::isfinite(hs[0]) || !std::isfinite(hs[1]) || !std::isfinite(hs[2])) {
      c.err = "rhoofr: non-finite kinetic energy, norm or density";
      rc = GBCP_ERR_NONFINITE;
    } else if (std::fabs(hs[2] - hs[1]) > charge_tolerance(c, hs[1])) {
      // the reference stops here: 'TOTAL DENSITY SUMS ARE NOT EQUAL' (rhoofr_utils.mod.F90:625-635)
      char msg[160];
      snprintf(msg, sizeof(msg), "rhoofr: total density sums are not equal (Fourier space %.12f, real space %.12f)",
               hs[1], hs[2]);
      c.err = msg;
      rc = GBCP_ERR_CHARGE;
    }
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_vpsi(gbcp_ctx* h, const double* c0, int ldc, double* c2, int ldc2, const double* f, const double* vpot,
              int nstate, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate < 0 || (nstate > 0 && (!c0 || !c2 || !f || !vpot || ldc < c.ngw || ldc2 < c.ngw)))
    return set_err(h, GBCP_ERR_ARG, "vpsi: bad argument");
  c.err.clear();
  if (nstate == 0) return GBCP_OK;
  const size_t nnr1 = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  const cx<double>* dc0 = reinterpret_cast<const cx<double>*>(c0);
  cx<double>* dc2 = reinterpret_cast<cx<double>*>(c2);
  const double* df = f;
  const double* dv = vpot;
  int l0 = ldc, l2 = ldc2;
  int rc = 0, saved_batch = 0;
  if (mem == GBCP_MEM_HOST) {
    void* tf;
    if ((rc = stage_in(c, c.st_f, f, sizeof(double) * nstate, &tf))) return rc;
    if (!gbcp::ensure(c, c.st_vpot, sizeof(double) * nnr1) ||
        !gbcp::ensure(c, c.st_c0, sizeof(cx<double>) * (size_t)c.ngw * nstate) ||
        !gbcp::ensure(c, c.st_c2, sizeof(cx<double>) * (size_t)c.ngw * nstate))
      return GBCP_ERR_NOMEM;
    void* tv = c.st_vpot.p;
    cx<double>* t0 = static_cast<cx<double>*>(c.st_c0.p);
    cx<double>* t2 = static_cast<cx<double>*>(c.st_c2.p);
    const int nb = stage_plan(c, nstate, wfn_maybe(c, c0, ldc, nstate) ? STAGE_VPSI_CACHED : STAGE_VPSI);
    auto chunk = [&](int b, int* s0, int* ns) {
      *s0 = 2 * c.stage_bounds[b];
      *ns = std::min(2 * c.stage_bounds[b + 1], nstate) - *s0;
    };
    // events: [0] ordering, [1, nb] c0 chunks, [nb+1, 2nb] C2 downloads, [2nb+1, 3nb] C2 uploads,
    // [3nb+1] V(r), last: the final download
    if ((rc = pipe_prepare(c, 2 * nb + 1))) return rc;
    // V(r) goes first, queued before the host reads the cache key, so the copy engine
    // is busy meanwhile; then chunk 0's states, and chunk b's C2 columns behind chunk
    // b+1's states, so that the first transforms start after one chunk and each
    // decode finds its C2
    {
      gbcp::ProfScope ps_(c, "h2d_vpot", c.copy, 1);
      GBCP_CUDA_TRY(c, cudaMemcpyAsync(tv, vpot, sizeof(double) * nnr1, cudaMemcpyHostToDevice, c.copy));
      GBCP_CUDA_TRY(c, cudaEventRecord(c.pipe_ev[3 * nb + 1], c.copy));
    }
    const bool resident = wfn_hit(c, c0, ldc, nstate);  // c0 still on the device from rhoofr
    c.zk_resident = resident;
    for (int b = 0; b <= nb; ++b) {
      int s0, ns;
      if (b < nb) {
        chunk(b, &s0, &ns);
        if (!resident && (rc = pipe_up(c, t0, c0, ldc, s0, ns))) return rc;
        GBCP_CUDA_TRY(c, cudaEventRecord(c.pipe_ev[1 + b], c.copy));
      }
      if (b > 0) {
        chunk(b - 1, &s0, &ns);
        if ((rc = pipe_up(c, t2, c2, ldc2, s0, ns))) return rc;
        GBCP_CUDA_TRY(c, cudaEventRecord(c.pipe_ev[2 * nb + b], c.copy));
      }
    }
    c.batch_ready = c.pipe_ev.data() + 1;
    c.batch_c2_ready = c.pipe_ev.data() + 2 * nb + 1;
    c.vpot_ready = c.pipe_ev[3 * nb + 1];
    saved_batch = c.batch;
    c.batch = stage_max(c);
    // C2 columns of batch b go back as soon as its decode is queued
    c.batch_done = [&c, c2, ldc2, nstate, t2, nb](int b) -> int {
      const int s0 = 2 * c.stage_bounds[b], ns = std::min(2 * c.stage_bounds[b + 1], nstate) - s0;
      cudaEvent_t e = c.pipe_ev[1 + nb + b];
      GBCP_CUDA_TRY(c, cudaEventRecord(e, c.stream));
      GBCP_CUDA_TRY(c, cudaStreamWaitEvent(c.copy_out, e, 0));
      gbcp::ProfScope ps_(c, "d2h_c2", c.copy_out, 2);
      GBCP_CUDA_TRY(c, cudaMemcpy2DAsync(c2 + 2 * (size_t)s0 * ldc2, sizeof(cx<double>) * (size_t)ldc2,
                                         t2 + (size_t)s0 * c.ngw, sizeof(cx<double>) * c.ngw,
                                         sizeof(cx<double>) * c.ngw, ns, cudaMemcpyDeviceToHost, c.copy_out));
      return 0;
    };
    dc0 = t0;
    dc2 = t2;
    df = static_cast<double*>(tf);
    dv = static_cast<double*>(tv);
    l0 = l2 = c.ngw;
  }
  rc = gbcp::band_vpsi(c, dc0, l0, dc2, l2, df, dv, nstate);
  c.zk_resident = false;
  c.batch_ready = nullptr;
  c.batch_c2_ready = nullptr;
  c.vpot_ready = nullptr;
  c.batch_done = nullptr;
  if (saved_batch) c.batch = saved_batch;
  if (mem == GBCP_MEM_HOST) {
    // the context stream (and so finish) waits for the last C2 copies
    cudaEvent_t e = c.pipe_ev[c.pipe_ev.size() - 1];
    cudaEventRecord(e, c.copy_out);
    cudaStreamWaitEvent(c.stream, e, 0);
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_ortho(gbcp_ctx* h, double* c0, int ldc, int nstate, int method, double* scond, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate < 0 || (nstate > 0 && (!c0 || ldc < c.ngw)) ||
      (method != GBCP_ORTHO_GS && method != GBCP_ORTHO_LOWDIN))
    return set_err(h, GBCP_ERR_ARG, "ortho: bad argument");
  c.err.clear();
  if (nstate == 0) return GBCP_OK;
  cx<double>* dc0 = reinterpret_cast<cx<double>*>(c0);
  int l0 = ldc;
  int rc = 0;
  if (mem == GBCP_MEM_HOST && method == GBCP_ORTHO_GS) {
    // copies overlapped with the work where the tensor-core engine runs the step; c0 is
    // rewritten in st_c0 and on the host, so the cached copy ends here
    // on a likely cache hit the read-only part (overlap, Cholesky) starts on the cached
    // copy while the host checks the key, which is confirmed before C U^-1 rewrites it
    const bool maybe = wfn_maybe(c, c0, ldc, nstate);
    const double key = c.wfn.key;
    c.wfn.valid = false;
    const std::function<bool()> confirm = [&c, c0, key]() { return wfn_key(c0, c.ngw) == key; };
    rc = gbcp::ortho_gs_host(c, c0, ldc, nstate, scond, maybe ? 1 : 0, maybe ? &confirm : nullptr);
    if (rc == 8) rc = gbcp::ortho_gs_host(c, c0, ldc, nstate, scond, 0, nullptr);
    if (rc != 7) return finish(c, rc);
    rc = 0;
    c.err.clear();
  }
  if (mem == GBCP_MEM_HOST) {
    if ((rc = stage_in_cx(c, c.st_c0, c0, ldc, c.ngw, nstate, &dc0))) return rc;
    l0 = c.ngw;
  }
  rc = method == GBCP_ORTHO_GS ? gbcp::ortho_gs(c, dc0, l0, nstate, scond)
                               : gbcp::ortho_lowdin(c, dc0, l0, nstate, scond);
  if (!rc && mem == GBCP_MEM_HOST) rc = stage_out_cx(c, dc0, c0, ldc, c.ngw, nstate);
  return finish(c, rc);
}

int gbcp_rortog(gbcp_ctx* h, const double* c0, int ldc0, double* cm, int ldcm, int nstate, int tnon, double epsog,
                int maxit, double* gam, int* iters, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (iters) *iters = 0;
  if (bad_mem(mem) || nstate < 0 || maxit < 0 || !(epsog >= 0.0) ||
      (nstate > 0 && (!c0 || !cm || ldc0 < c.ngw || ldcm < c.ngw || (const double*)cm == c0)))
    return set_err(h, GBCP_ERR_ARG, "rortog: bad argument");
  c.err.clear();
  if (nstate == 0) return GBCP_OK;
  const cx<double>* d0 = reinterpret_cast<const cx<double>*>(c0);
  cx<double>* dm = reinterpret_cast<cx<double>*>(cm);
  int l0 = ldc0, lm = ldcm;
  double* dg = gam;
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    cx<double>* t;
    if ((rc = stage_in_cx(c, c.st_c0, c0, ldc0, c.ngw, nstate, &t))) return rc;
    d0 = t;
    if ((rc = stage_in_cx(c, c.st_c2, cm, ldcm, c.ngw, nstate, &dm))) return rc;
    l0 = lm = c.ngw;
    if (gam) {
      if (!gbcp::ensure(c, c.st_misc, sizeof(double) * (size_t)nstate * nstate)) return GBCP_ERR_NOMEM;
      dg = static_cast<double*>(c.st_misc.p);
    }
  }
  rc = gbcp::rortho(c, d0, l0, dm, lm, nstate, tnon, epsog, maxit, dg, iters);
  if (!rc && mem == GBCP_MEM_HOST) {
    rc = stage_out_cx(c, dm, cm, ldcm, c.ngw, nstate);
    if (!rc && gam) {
      cudaError_t e =
          cudaMemcpyAsync(gam, dg, sizeof(double) * (size_t)nstate * nstate, cudaMemcpyDeviceToHost, c.stream);
      if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  return finish(c, rc);
}

int gbcp_ovlap(gbcp_ctx* h, const double* c0, int ldc, int nstate, double* smat, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate <= 0 || !c0 || !smat || ldc < c.ngw) return set_err(h, GBCP_ERR_ARG, "ovlap: bad argument");
  c.err.clear();
  const cx<double>* dc0 = reinterpret_cast<const cx<double>*>(c0);
  int l0 = ldc;
  double* dS = smat;
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    cx<double>* t;
    if ((rc = stage_in_cx(c, c.st_c0, c0, ldc, c.ngw, nstate, &t))) return rc;
    dc0 = t;
    l0 = c.ngw;
    if (!gbcp::ensure(c, c.st_misc, sizeof(double) * (size_t)nstate * nstate)) return GBCP_ERR_NOMEM;
    dS = static_cast<double*>(c.st_misc.p);
  }
  rc = gbcp::ovlap_gamma(c, dc0, l0, nstate, dS);
  if (!rc && mem == GBCP_MEM_HOST) {
    cudaError_t e =
        cudaMemcpyAsync(smat, dS, sizeof(double) * (size_t)nstate * nstate, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

static int fft_entry(gbcp_ctx* h, double* f, int mem, bool inv) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || !f) return set_err(h, GBCP_ERR_ARG, "fft: bad argument");
  c.err.clear();
  const size_t n = (size_t)c.kr[0] * c.kr[1] * c.nr[2];
  cx<double>* d = reinterpret_cast<cx<double>*>(f);
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    void* t;
    if ((rc = stage_in(c, c.st_misc2, f, sizeof(cx<double>) * n, &t))) return rc;
    d = static_cast<cx<double>*>(t);
  }
  rc = gbcp::dense_fft(c, d, inv);
  if (!rc && mem == GBCP_MEM_HOST) {
    cudaError_t e = cudaMemcpyAsync(f, d, sizeof(cx<double>) * n, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_invfftn(gbcp_ctx* h, double* f, int mem) { return fft_entry(h, f, mem, true); }
int gbcp_fwfftn(gbcp_ctx* h, double* f, int mem) { return fft_entry(h, f, mem, false); }

// Elements of the caller's fnl (kdim 1) or dfnl (kdim 3) a species block spans from
// its base: fnl(ia, iv, i) at ia + lda (iv + ldp i), dfnl(ia, iv, k, i) at
// ia + lda (iv + ldp (k + 3 i)); lda = 0 / ldp = 0 stand for nat / ngh.
static size_t fnl_span(int nat, int ngh, int nstate, int& lda, int& ldp, int kdim) {
  lda = lda > 0 ? lda : nat;
  ldp = ldp > 0 ? ldp : ngh;
  if (lda < nat || ldp < ngh) return 0;
  return (size_t)(nat - 1) + (size_t)lda * ((size_t)(ngh - 1) + (size_t)ldp * ((size_t)kdim * nstate - 1)) + 1;
}

int gbcp_rnlsm1(gbcp_ctx* h, const double* c0, int ldc, int nstate, int nat, int ngh, const int32_t* nghtol,
                const double* twnl, const double* eigr, double* fnl, int ld_atoms, int ld_proj, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate <= 0 || nat <= 0 || ngh <= 0 || !c0 || !nghtol || !twnl || !eigr || !fnl ||
      ldc < c.ngw)
    return set_err(h, GBCP_ERR_ARG, "rnlsm1: bad argument");
  const size_t nfnl = fnl_span(nat, ngh, nstate, ld_atoms, ld_proj, 1);
  if (!nfnl) return set_err(h, GBCP_ERR_ARG, "rnlsm1: fnl leading dimensions below nat / ngh");
  c.err.clear();
  const cx<double>* dc0 = reinterpret_cast<const cx<double>*>(c0);
  const double* dtw = twnl;
  const cx<double>* de = reinterpret_cast<const cx<double>*>(eigr);
  double* dfnl = fnl;
  int l0 = ldc;
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    cx<double>* t0;
    void *t1, *t2, *t3;
    if ((rc = stage_in_cx(c, c.st_c0, c0, ldc, c.ngw, nstate, &t0))) return rc;
    if ((rc = stage_in(c, c.nl_b, twnl, sizeof(double) * (size_t)c.ngw * ngh, &t1))) return rc;
    if ((rc = stage_in(c, c.nl_c, eigr, sizeof(cx<double>) * (size_t)c.ngw * nat, &t2))) return rc;
    // the span holds other species' entries too: staged in and out whole, so they come back unchanged
    if ((rc = stage_in(c, c.nl_d, fnl, sizeof(double) * nfnl, &t3))) return rc;
    dc0 = t0;
    dtw = static_cast<double*>(t1);
    de = static_cast<cx<double>*>(t2);
    dfnl = static_cast<double*>(t3);
    l0 = c.ngw;
  }
  rc = gbcp::nl_rnlsm1(c, dc0, l0, nstate, nat, ngh, nghtol, dtw, de, dfnl, ld_atoms, ld_proj);
  if (!rc && mem == GBCP_MEM_HOST) {
    cudaError_t e = cudaMemcpyAsync(fnl, dfnl, sizeof(double) * nfnl, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_rnlsm2(gbcp_ctx* h, const double* c0, int ldc, int nstate, int nat, int ngh, const int32_t* nghtol,
                const double* twnl, const double* eigr, double* dfnl, int ld_atoms, int ld_proj, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate <= 0 || nat <= 0 || ngh <= 0 || !c0 || !nghtol || !twnl || !eigr || !dfnl ||
      ldc < c.ngw)
    return set_err(h, GBCP_ERR_ARG, "rnlsm2: bad argument");
  const size_t nd = fnl_span(nat, ngh, nstate, ld_atoms, ld_proj, 3);
  if (!nd) return set_err(h, GBCP_ERR_ARG, "rnlsm2: dfnl leading dimensions below nat / ngh");
  c.err.clear();
  const cx<double>* dc0 = reinterpret_cast<const cx<double>*>(c0);
  const double* dtw = twnl;
  const cx<double>* de = reinterpret_cast<const cx<double>*>(eigr);
  double* dd = dfnl;
  int l0 = ldc;
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    cx<double>* t0;
    void *t1, *t2, *t3;
    if ((rc = stage_in_cx(c, c.st_c0, c0, ldc, c.ngw, nstate, &t0))) return rc;
    if ((rc = stage_in(c, c.nl_b, twnl, sizeof(double) * (size_t)c.ngw * ngh, &t1))) return rc;
    if ((rc = stage_in(c, c.nl_c, eigr, sizeof(cx<double>) * (size_t)c.ngw * nat, &t2))) return rc;
    if ((rc = stage_in(c, c.nl_d, dfnl, sizeof(double) * nd, &t3))) return rc;
    dc0 = t0;
    dtw = static_cast<double*>(t1);
    de = static_cast<cx<double>*>(t2);
    dd = static_cast<double*>(t3);
    l0 = c.ngw;
  }
  rc = gbcp::nl_rnlsm2(c, dc0, l0, nstate, nat, ngh, nghtol, dtw, de, dd, ld_atoms, ld_proj);
  if (!rc && mem == GBCP_MEM_HOST) {
    cudaError_t e = cudaMemcpyAsync(dfnl, dd, sizeof(double) * nd, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_rnlfor(gbcp_ctx* h, int nstate, const double* f, int nat, int ngh, const double* wsg, const double* fnl,
                const double* dfnl, int ld_atoms, int ld_proj, double* fion, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate <= 0 || nat <= 0 || ngh <= 0 || !f || !wsg || !fnl || !dfnl || !fion)
    return set_err(h, GBCP_ERR_ARG, "rnlfor: bad argument");
  const size_t nf = fnl_span(nat, ngh, nstate, ld_atoms, ld_proj, 1);
  const size_t nd = fnl_span(nat, ngh, nstate, ld_atoms, ld_proj, 3);
  if (!nf || !nd) return set_err(h, GBCP_ERR_ARG, "rnlfor: fnl leading dimensions below nat / ngh");
  c.err.clear();
  const double *df = f, *dw = wsg, *dfn = fnl, *ddf = dfnl;
  double* dfi = fion;
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    void *t1, *t2, *t3, *t4, *t5;
    if ((rc = stage_in(c, c.st_f, f, sizeof(double) * nstate, &t1))) return rc;
    if ((rc = stage_in(c, c.st_misc, wsg, sizeof(double) * ngh, &t2))) return rc;
    if ((rc = stage_in(c, c.nl_b, fnl, sizeof(double) * nf, &t3))) return rc;
    if ((rc = stage_in(c, c.nl_d, dfnl, sizeof(double) * nd, &t4))) return rc;
    if ((rc = stage_in(c, c.st_misc2, fion, sizeof(double) * 3 * nat, &t5))) return rc;
    df = static_cast<double*>(t1);
    dw = static_cast<double*>(t2);
    dfn = static_cast<double*>(t3);
    ddf = static_cast<double*>(t4);
    dfi = static_cast<double*>(t5);
  }
  rc = gbcp::nl_rnlfor(c, nstate, df, nat, ngh, dw, dfn, ddf, dfi, ld_atoms, ld_proj);
  if (!rc && mem == GBCP_MEM_HOST) {
    cudaError_t e = cudaMemcpyAsync(fion, dfi, sizeof(double) * 3 * nat, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_fnonloc(gbcp_ctx* h, double* c2, int ldc2, int nstate, const double* f, int nat, int ngh,
                 const int32_t* nghtol, const double* twnl, const double* eigr, const double* fnl, int ld_atoms,
                 int ld_proj, const double* wsg, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate <= 0 || nat <= 0 || ngh <= 0 || !c2 || !f || !nghtol || !twnl || !eigr || !fnl ||
      !wsg || ldc2 < c.ngw)
    return set_err(h, GBCP_ERR_ARG, "fnonloc: bad argument");
  const size_t nf = fnl_span(nat, ngh, nstate, ld_atoms, ld_proj, 1);
  if (!nf) return set_err(h, GBCP_ERR_ARG, "fnonloc: fnl leading dimensions below nat / ngh");
  c.err.clear();
  cx<double>* dc2 = reinterpret_cast<cx<double>*>(c2);
  const double* df = f;
  const double* dtw = twnl;
  const cx<double>* de = reinterpret_cast<const cx<double>*>(eigr);
  const double* dfnl = fnl;
  const double* dw = wsg;
  int l2 = ldc2;
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    void *t1, *t2, *t3, *t4, *t5;
    if ((rc = stage_in_cx(c, c.st_c2, c2, ldc2, c.ngw, nstate, &dc2))) return rc;
    if ((rc = stage_in(c, c.st_f, f, sizeof(double) * nstate, &t1))) return rc;
    if ((rc = stage_in(c, c.nl_b, twnl, sizeof(double) * (size_t)c.ngw * ngh, &t2))) return rc;
    if ((rc = stage_in(c, c.nl_c, eigr, sizeof(cx<double>) * (size_t)c.ngw * nat, &t3))) return rc;
    if ((rc = stage_in(c, c.nl_d, fnl, sizeof(double) * nf, &t4))) return rc;
    if ((rc = stage_in(c, c.st_misc, wsg, sizeof(double) * ngh, &t5))) return rc;
    df = static_cast<double*>(t1);
    dtw = static_cast<double*>(t2);
    de = static_cast<cx<double>*>(t3);
    dfnl = static_cast<double*>(t4);
    dw = static_cast<double*>(t5);
    l2 = c.ngw;
  }
  rc = gbcp::nl_fnonloc(c, dc2, l2, nstate, df, nat, ngh, nghtol, dtw, de, dfnl, dw, ld_atoms, ld_proj);
  if (!rc && mem == GBCP_MEM_HOST) rc = stage_out_cx(c, dc2, c2, ldc2, c.ngw, nstate);
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_set_dens_sphere(gbcp_ctx* h, int nhg, const int32_t* inyh, const double* hg) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (nhg < c.ngw || !inyh || !hg) return set_err(h, GBCP_ERR_ARG, "set_dens_sphere: bad argument");
  c.err.clear();
  const int n[3] = {c.nr[0], c.nr[1], c.nr[2]};
  std::vector<int> pos(nhg), neg(nhg);
  std::vector<short4> mill(nhg);
  std::vector<double> g2(nhg);
  int dmax = 0;
  for (int ig = 0; ig < nhg; ++ig) {
    int m[3], p[3], q[3];
    for (int a = 0; a < 3; ++a) {
      m[a] = inyh[3 * (size_t)ig + a] - (n[a] / 2 + 1);
      if (2 * std::abs(m[a]) >= n[a] || std::abs(m[a]) > 32767)
        return set_err(h, GBCP_ERR_ARG, "set_dens_sphere: G vector outside the mesh");
      dmax = std::max(dmax, std::abs(m[a]));
      p[a] = ((m[a] % n[a]) + n[a]) % n[a];
      q[a] = ((-m[a] % n[a]) + n[a]) % n[a];
    }
    pos[ig] = p[0] + c.kr[0] * (p[1] + c.kr[1] * p[2]);
    neg[ig] = q[0] + c.kr[0] * (q[1] + c.kr[1] * q[2]);
    mill[ig] = make_short4((short)m[0], (short)m[1], (short)m[2], 0);
    g2[ig] = hg[ig] * c.tpiba2;
  }
  const int *dp, *dn;
  const short4* dm;
  const double* dg;
  if (!gbcp::upload(c, pos, dp) || !gbcp::upload(c, neg, dn) || !gbcp::upload(c, mill, dm) ||
      !gbcp::upload(c, g2, dg))
    return set_err(h, GBCP_ERR_NOMEM, "set_dens_sphere: upload failed");
  c.dpos = dp;
  c.dneg = dn;
  c.dmill = dm;
  c.dg2 = dg;
  c.dmax = dmax;
  c.nhg = nhg;
  return GBCP_OK;
}

int gbcp_vofrho(gbcp_ctx* h, const double* rhoe, int nat, int nsp, const int32_t* isp, const double* tau,
                const double* vps, const double* vext, double* veff, double* energies, double* fion, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nat < 0 || nsp <= 0 || !rhoe || !veff || !energies || (nat > 0 && (!isp || !tau || !vps)))
    return set_err(h, GBCP_ERR_ARG, "vofrho: bad argument");
  if (c.nhg <= 0) return set_err(h, GBCP_ERR_ARG, "vofrho: call gbcp_set_dens_sphere first");
  c.err.clear();
  const size_t nnr1 = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  const double *drho = rhoe, *dtau = tau, *dvps = vps, *dvext = vext;
  double *dve = veff, *dfi = fion;
  int rc = 0;
  static const double zero3[3] = {0.0, 0.0, 0.0};
  static const int32_t zero_sp[1] = {0};
  const int nat_eff = nat > 0 ? nat : 1;  // no atoms: one atom of zero form factor
  const int32_t* isp_h = nat > 0 ? isp : zero_sp;
  if (mem == GBCP_MEM_HOST) {
    void *tr, *tt, *tv, *te;
    if ((rc = stage_in(c, c.en_in[2], rhoe, sizeof(double) * nnr1, &tr))) return rc;
    if ((rc = stage_in(c, c.en_in[0], nat > 0 ? tau : zero3, sizeof(double) * 3 * nat_eff, &tt))) return rc;
    drho = static_cast<double*>(tr);
    dtau = static_cast<double*>(tt);
    if (nat > 0) {
      if ((rc = stage_in(c, c.en_in[1], vps, sizeof(double) * (size_t)c.nhg * nsp, &tv))) return rc;
      dvps = static_cast<double*>(tv);
    }
    if (vext) {
      if ((rc = stage_in(c, c.en_in[3], vext, sizeof(double) * nnr1, &te))) return rc;
      dvext = static_cast<double*>(te);
    }
    if (!gbcp::ensure(c, c.st_vpot, sizeof(double) * nnr1)) return GBCP_ERR_NOMEM;
    dve = static_cast<double*>(c.st_vpot.p);
    if (fion) {
      if (!gbcp::ensure(c, c.en_in[4], sizeof(double) * 3 * nat_eff)) return GBCP_ERR_NOMEM;
      dfi = static_cast<double*>(c.en_in[4].p);
    }
  }
  if (nat == 0) {
    if (mem == GBCP_MEM_DEVICE) {
      if (!gbcp::ensure(c, c.en_in[0], sizeof(double) * 3)) return GBCP_ERR_NOMEM;
      GBCP_CUDA_TRY(c, cudaMemsetAsync(c.en_in[0].p, 0, sizeof(double) * 3, c.stream));
      dtau = static_cast<double*>(c.en_in[0].p);
    }
    if (!gbcp::ensure(c, c.en_in[1], sizeof(double) * (size_t)c.nhg)) return GBCP_ERR_NOMEM;
    GBCP_CUDA_TRY(c, cudaMemsetAsync(c.en_in[1].p, 0, sizeof(double) * (size_t)c.nhg, c.stream));
    dvps = static_cast<double*>(c.en_in[1].p);
    nsp = 1;
  }
  double* fion_dev = (fion && nat > 0) ? dfi : nullptr;
  rc = gbcp::vofrho_host_energies(c, nat_eff, nsp, isp_h, drho, dtau, dvps, dvext, dve, energies, fion_dev);
  if (!rc && mem == GBCP_MEM_HOST) {
    GBCP_CUDA_TRY(c, cudaMemcpyAsync(veff, dve, sizeof(double) * nnr1, cudaMemcpyDeviceToHost, c.stream));
    if (fion && nat > 0)
      GBCP_CUDA_TRY(c, cudaMemcpyAsync(fion, dfi, sizeof(double) * 3 * nat, cudaMemcpyDeviceToHost, c.stream));
  }
  return finish(c, rc);
}

int gbcp_ovlap2(gbcp_ctx* h, const double* c1, int ldc1, const double* c2, int ldc2, int nstate, double* amat,
                int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate <= 0 || !c1 || !c2 || !amat || ldc1 < c.ngw || ldc2 < c.ngw)
    return set_err(h, GBCP_ERR_ARG, "ovlap2: bad argument");
  c.err.clear();
  const cx<double>* d1 = reinterpret_cast<const cx<double>*>(c1);
  const cx<double>* d2 = reinterpret_cast<const cx<double>*>(c2);
  int l1 = ldc1, l2 = ldc2;
  double* dA = amat;
  int rc = 0;
  if (mem == GBCP_MEM_HOST) {
    cx<double>*t1, *t2;
    if ((rc = stage_in_cx(c, c.st_c0, c1, ldc1, c.ngw, nstate, &t1))) return rc;
    if ((rc = stage_in_cx(c, c.st_c2, c2, ldc2, c.ngw, nstate, &t2))) return rc;
    d1 = t1;
    d2 = t2;
    l1 = l2 = c.ngw;
    if (!gbcp::ensure(c, c.st_misc, sizeof(double) * (size_t)nstate * nstate)) return GBCP_ERR_NOMEM;
    dA = static_cast<double*>(c.st_misc.p);
  }
  GBCP_CUDA_TRY(c, cudaMemsetAsync(c.d_info, 0, 16, c.stream));
  // xovlap writes row-major A[i][j] = <X_i|Y_j>; with X = c2, Y = c1 that is the
  // column-major a(i, j) = <c1_i|c2_j> of the reference
  rc = gbcp::xovlap(c, d2, l2, d1, l1, nstate, dA);
  if (!rc && gbcp::use_tc_gemm(c)) {
    int st = 0;
    GBCP_CUDA_TRY(c, cudaMemcpyAsync(&st, c.d_info, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    GBCP_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    if (st == -2) rc = set_err(h, GBCP_ERR_TIMEOUT, "ovlap2: tensor-core pipeline wait expired");
  }
  if (!rc && mem == GBCP_MEM_HOST) {
    cudaError_t e =
        cudaMemcpyAsync(amat, dA, sizeof(double) * (size_t)nstate * nstate, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return set_err(h, GBCP_ERR_CUDA, cudaGetErrorString(e));
  }
  if (mem == GBCP_MEM_HOST || rc) return finish(c, rc);
  return GBCP_OK;
}

int gbcp_energy(gbcp_ctx* h, const double* c0, int ldc, int nstate, const double* f, int nat, int nsp,
                const int32_t* isp, const double* tau, const double* vps, const double* vext, double* energies,
                double* c2, int ldc2, double* dvloc, double* fion, int mem) {
  if (!h) return GBCP_ERR_ARG;
  Ctx& c = h->c;
  if (bad_mem(mem) || nstate <= 0 || nat < 0 || nsp <= 0 || !c0 || !f || !energies || ldc < c.ngw ||
      (nat > 0 && (!isp || !tau || !vps)) || (c2 && ldc2 < c.ngw))
    return set_err(h, GBCP_ERR_ARG, "energy: bad argument");
  if (c.nhg <= 0) return set_err(h, GBCP_ERR_ARG, "energy: call gbcp_set_dens_sphere first");
  c.err.clear();
  const size_t nnr1 = (size_t)c.kr[0] * c.kr[1] * c.kr[2];
  const cx<double>* dc0 = reinterpret_cast<const cx<double>*>(c0);
  cx<double>* dc2 = reinterpret_cast<cx<double>*>(c2);
  const double *df = f, *dtau = tau, *dvps = vps, *dvext = vext;
  double *ddv = dvloc, *dfi = fion;
  int l0 = ldc, l2 = ldc2;
  int rc = 0;
  static const double zero3[3] = {0.0, 0.0, 0.0};
  static const int32_t zero_sp[1] = {0};
  const int nat_eff = nat > 0 ? nat : 1;  // no atoms: one atom of zero form factor
  const int32_t* isp_h = nat > 0 ? isp : zero_sp;
  if (mem == GBCP_MEM_HOST) {
    cx<double>* t0;
    void *tf, *tt, *tv, *te;
    if ((rc = stage_in_cx(c, c.st_c0, c0, ldc, c.ngw, nstate, &t0))) return rc;
    if ((rc = stage_in(c, c.st_f, f, sizeof(double) * nstate, &tf))) return rc;
    if ((rc = stage_in(c, c.en_in[0], nat > 0 ? tau : zero3, sizeof(double) * 3 * nat_eff, &tt))) return rc;
    dc0 = t0;
    df = static_cast<double*>(tf);
    dtau = static_cast<double*>(tt);
    if (nat > 0) {
      if ((rc = stage_in(c, c.en_in[1], vps, sizeof(double) * (size_t)c.nhg * nsp, &tv))) return rc;
      dvps = static_cast<double*>(tv);
    }
    if (vext) {
      if ((rc = stage_in(c, c.en_in[2], vext, sizeof(double) * nnr1, &te))) return rc;
      dvext = static_cast<double*>(te);
    }
    if (c2) {
      if (!gbcp::ensure(c, c.st_c2, sizeof(cx<double>) * (size_t)c.ngw * nstate)) return GBCP_ERR_NOMEM;
      dc2 = static_cast<cx<double>*>(c.st_c2.p);
      l2 = c.ngw;
    }
    if (dvloc) {
      if (!gbcp::ensure(c, c.en_in[3], sizeof(double) * nnr1)) return GBCP_ERR_NOMEM;
      ddv = static_cast<double*>(c.en_in[3].p);
    }
    if (fion) {
      if (!gbcp::ensure(c, c.en_in[4], sizeof(double) * 3 * nat_eff)) return GBCP_ERR_NOMEM;
      dfi = static_cast<double*>(c.en_in[4].p);
    }
    l0 = c.ngw;
  }
  if (nat == 0) {
    // a single dummy atom at the origin with a zero form factor
    if (mem == GBCP_MEM_DEVICE) {
      if (!gbcp::ensure(c, c.en_in[0], sizeof(double) * 3)) return GBCP_ERR_NOMEM;
      GBCP_CUDA_TRY(c, cudaMemsetAsync(c.en_in[0].p, 0, sizeof(double) * 3, c.stream));
      dtau = static_cast<double*>(c.en_in[0].p);
    }
    if (!gbcp::ensure(c, c.en_in[1], sizeof(double) * (size_t)c.nhg)) return GBCP_ERR_NOMEM;
    GBCP_CUDA_TRY(c, cudaMemsetAsync(c.en_in[1].p, 0, sizeof(double) * (size_t)c.nhg, c.stream));
    dvps = static_cast<double*>(c.en_in[1].p);
    nsp = 1;
  }
  double* fion_dev = (fion && nat > 0) ? dfi : nullptr;
  rc = gbcp::energy_and_grad(c, dc0, l0, nstate, df, nat_eff, nsp, isp_h, dtau, dvps, dvext, energies, dc2, l2, ddv,
                             fion_dev);
  if (!rc && mem == GBCP_MEM_HOST) {
    if (c2) rc = stage_out_cx(c, dc2, c2, ldc2, c.ngw, nstate);
    if (!rc && dvloc) GBCP_CUDA_TRY(c, cudaMemcpyAsync(dvloc, ddv, sizeof(double) * nnr1, cudaMemcpyDeviceToHost, c.stream));
    if (!rc && fion && nat > 0)
      GBCP_CUDA_TRY(c, cudaMemcpyAsync(fion, dfi, sizeof(double) * 3 * nat, cudaMemcpyDeviceToHost, c.stream));
  }
  return finish(c, rc);
}

}  // extern "C"
