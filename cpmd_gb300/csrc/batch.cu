// Many independent Γ-point cells per step in ONE CUDA-graph launch, with a
// per-size-class autotuner.
//
// The reference has no batched form: every cell is its own CPMD run, and its
// GPU path pushes each state pair through cuFFT with host round trips
// (rhoofr_utils.mod.F90:305-409, vpsi_utils.mod.F90:285-430).  Here a batch
// owns one context per cell (geometry, plans, workspaces); a step queues, for
// every cell, rhoofr + E_kin + int V rho (FP64 reductions into device memory),
// vpsi and Gram-Schmidt ortho without any host synchronisation, spread over
// worker streams (fork/join events) so that small cells run side by side.
// The first step with a given set of buffers runs eagerly (allocating the
// workspaces) and is then captured into a CUDA graph without being executed
// again; later steps replay it with a single cudaGraphLaunch, which also copies
// energies and status words back to pinned host memory.
//
// Autotuner: cells with equal mesh, sphere and state count form a size class.
// For the first cell of each class it times (CUDA events, copies of that cell's
// states) every band-loop configuration -- FFT kernels (four-step register
// codelets or run-time planned Stockham) x state pairs per launch x plane-fused
// y/x stages -- and then the ortho GEMMs (FP64 SIMT with 64 x 64 or 32 x 32
// output tiles, or the tcgen05 split GEMM with its K-split and C M partitions)
// x the Cholesky (blocked FP64 or double-float), and applies the fastest to the
// whole class.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/cpmd_gb300.h"
#include "ctx.h"
#include "fs_plan.h"

using gbcp::Ctx;
using gbcp::cx;

struct gbcp_batch {
  std::vector<gbcp_ctx*> cells;
  std::vector<int> klass;                 // size class of each cell (after tuning / first step)
  int precision = 0;
  cudaStream_t s0 = nullptr;
  std::vector<cudaStream_t> ws;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  double* d_out = nullptr;                // 2 per cell: E_kin, int V rho
  int* d_status = nullptr;                // per cell: ortho status word
  double* h_out = nullptr;                // pinned mirrors
  int* h_status = nullptr;
  std::vector<int> assign;                // worker stream of each cell
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  std::vector<uintptr_t> key;             // buffers + flags the graph was captured for
  long long kernels_per_graph = 0;
  std::string err, report;
};

namespace {

int status_code(int s) {
  if (s == 0) return GBCP_OK;
  if (s == -1) return GBCP_ERR_NONFINITE;
  if (s == -2) return GBCP_ERR_TIMEOUT;
  return GBCP_ERR_NOT_SPD;
}

int fail(gbcp_batch* b, int rc, const std::string& msg) {
  b->err = msg;
  return rc;
}

// complex64 (ld lda) <-> complex128 (ld ngw) for ortho on complex64 storage; the
// conversions are integer operations on the bit patterns (exact one way, round
// to nearest the other)
__global__ void k_c64_to_c128(const cx<float>* __restrict__ a, int lda, cx<double>* __restrict__ b, int ngw, int n) {
  const size_t tot = (size_t)ngw * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const size_t s = e / ngw, g = e - s * ngw;
    const cx<float> v = a[s * lda + g];
    b[e] = gbcp::mk<double>(gbcp::f2d_int(v.x), gbcp::f2d_int(v.y));
  }
}
__global__ void k_c128_to_c64(const cx<double>* __restrict__ b, int ngw, int n, cx<float>* __restrict__ a, int lda) {
  const size_t tot = (size_t)ngw * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const size_t s = e / ngw, g = e - s * ngw;
    const cx<double> v = b[e];
    a[s * lda + g] = gbcp::mk<float>(gbcp::d2f_int(v.x), gbcp::d2f_int(v.y));
  }
}

// all work of one cell, queued on c.stream; no host synchronisation
int queue_cell(Ctx& c, const gbcp_cell_io& io, int flags, double* dout, int* dstatus) {
  cx<double>* c0 = reinterpret_cast<cx<double>*>(io.c0);
  int rc = 0;
  c.psi32 = (flags & GBCP_STEP_PSI_C64) ? 1 : 0;
  if (flags & GBCP_STEP_RHOOFR) {
    // E_kin summed in the band loop's gather, as in gbcp_rhoofr (the scalars stay on the device)
    if (!gbcp::ensure(c, c.rho_sc, 4 * sizeof(double))) return 6;
    double* sc = static_cast<double*>(c.rho_sc.p);
    if ((rc = gbcp::band_rhoofr(c, c0, io.ldc, io.nstate, io.f, io.rhoe, sc))) return rc;
    GBCP_CUDA_TRY(c, cudaMemcpyAsync(dout, sc, sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    if ((rc = gbcp::vrho_async(c, io.rhoe, io.vpot, dout + 1))) return rc;
  }
  if (flags & GBCP_STEP_VPSI) {
    if ((rc = gbcp::band_vpsi(c, c0, io.ldc, reinterpret_cast<cx<double>*>(io.c2), io.ldc2, io.f, io.vpot,
                              io.nstate)))
      return rc;
  }
  if (flags & GBCP_STEP_ORTHO) {
    if (c.psi32) {
      // FP64 Gram-Schmidt on a widened copy, rounded back into the complex64 states
      if (!gbcp::ensure(c, c.st_c0, sizeof(cx<double>) * (size_t)c.ngw * io.nstate)) return 6;
      cx<double>* w = static_cast<cx<double>*>(c.st_c0.p);
      const int nb = std::max(1, std::min(1024, (int)(((size_t)c.ngw * io.nstate + 255) / 256)));
      k_c64_to_c128<<<nb, 256, 0, c.stream>>>(reinterpret_cast<const cx<float>*>(io.c0), io.ldc, w, c.ngw, io.nstate);
      GBCP_LAUNCH_CHECK(c);
      if ((rc = gbcp::ortho_gs_queue(c, w, c.ngw, io.nstate))) return rc;
      k_c128_to_c64<<<nb, 256, 0, c.stream>>>(w, c.ngw, io.nstate, reinterpret_cast<cx<float>*>(io.c0), io.ldc);
      GBCP_LAUNCH_CHECK(c);
    } else if ((rc = gbcp::ortho_gs_queue(c, c0, io.ldc, io.nstate))) {
      return rc;
    }
    GBCP_CUDA_TRY(c, cudaMemcpyAsync(dstatus, c.d_info, sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
  } else {
    GBCP_CUDA_TRY(c, cudaMemsetAsync(dstatus, 0, sizeof(int), c.stream));
  }
  return 0;
}

// fork -> every cell on its worker stream -> join -> results to the host (pinned)
int queue_all(gbcp_batch* b, const gbcp_cell_io* io, int flags) {
  const int n = (int)b->cells.size();
  if (cudaEventRecord(b->fork, b->s0) != cudaSuccess) return fail(b, GBCP_ERR_CUDA, "batch: fork event");
  for (cudaStream_t w : b->ws)
    if (cudaStreamWaitEvent(w, b->fork, 0) != cudaSuccess) return fail(b, GBCP_ERR_CUDA, "batch: fork wait");
  for (int i = 0; i < n; ++i) {
    Ctx& c = b->cells[i]->c;
    c.stream = b->ws[b->assign[i]];
    const int rc = queue_cell(c, io[i], flags, b->d_out + 2 * i, b->d_status + i);
    if (rc) return fail(b, rc, "batch cell " + std::to_string(i) + ": " + c.err);
  }
  for (size_t w = 0; w < b->ws.size(); ++w) {
    if (cudaEventRecord(b->join[w], b->ws[w]) != cudaSuccess ||
        cudaStreamWaitEvent(b->s0, b->join[w], 0) != cudaSuccess)
      return fail(b, GBCP_ERR_CUDA, "batch: join");
  }
  if (cudaMemcpyAsync(b->h_out, b->d_out, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, b->s0) != cudaSuccess ||
      cudaMemcpyAsync(b->h_status, b->d_status, sizeof(int) * n, cudaMemcpyDeviceToHost, b->s0) != cudaSuccess)
    return fail(b, GBCP_ERR_CUDA, "batch: result copy");
  return 0;
}

// longest-first assignment of cells to worker streams by estimated cost
void assign_streams(gbcp_batch* b, const gbcp_cell_io* io) {
  const int n = (int)b->cells.size();
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) {
    const Ctx& c = b->cells[i]->c;
    const double N = (double)c.nr[0] * c.nr[1] * c.nr[2];
    cost[i] = (io[i].nstate + 1) / 2 * N * std::log2(N) + (double)io[i].nstate * io[i].nstate * c.ngw;
  }
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int a, int c) { return cost[a] > cost[c]; });
  std::vector<double> load(b->ws.size(), 0.0);
  b->assign.assign(n, 0);
  for (int i : order) {
    const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    b->assign[i] = w;
    load[w] += cost[i];
  }
}

void drop_graph(gbcp_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->key.clear();
}

std::vector<uintptr_t> make_key(const gbcp_batch* b, const gbcp_cell_io* io, int flags) {
  std::vector<uintptr_t> k;
  k.push_back((uintptr_t)flags);
  for (size_t i = 0; i < b->cells.size(); ++i) {
    const gbcp_cell_io& x = io[i];
    for (uintptr_t v : {(uintptr_t)x.c0, (uintptr_t)x.ldc, (uintptr_t)x.nstate, (uintptr_t)x.f, (uintptr_t)x.vpot,
                        (uintptr_t)x.rhoe, (uintptr_t)x.c2, (uintptr_t)x.ldc2})
      k.push_back(v);
    const Ctx& c = b->cells[i]->c;
    k.push_back((uintptr_t)(c.batch * 16 + c.fft_engine * 4 + (c.gemm_mode + 1)));
  }
  return k;
}

bool same_class(const Ctx& a, int na, const Ctx& c, int nc) {
  return a.nr[0] == c.nr[0] && a.nr[1] == c.nr[1] && a.nr[2] == c.nr[2] && a.ngw == c.ngw && na == nc &&
         a.omega == c.omega && a.tpiba2 == c.tpiba2;
}

int check_io(gbcp_batch* b, const gbcp_cell_io* io, int flags) {
  if (!io || (flags & 7) == 0 || flags > 15) return fail(b, GBCP_ERR_ARG, "batch: bad flags or io");
  if ((flags & GBCP_STEP_PSI_C64) && b->precision != GBCP_PREC_MIXED)
    return fail(b, GBCP_ERR_ARG, "batch: complex64 states need the MIXED precision");
  for (size_t i = 0; i < b->cells.size(); ++i) {
    const Ctx& c = b->cells[i]->c;
    const gbcp_cell_io& x = io[i];
    if (!x.c0 || x.nstate <= 0 || x.ldc < c.ngw || !x.f) return fail(b, GBCP_ERR_ARG, "batch: bad cell io");
    if ((flags & GBCP_STEP_RHOOFR) && (!x.rhoe || !x.vpot)) return fail(b, GBCP_ERR_ARG, "batch: rhoe/vpot");
    if ((flags & GBCP_STEP_VPSI) && (!x.c2 || !x.vpot || x.ldc2 < c.ngw))
      return fail(b, GBCP_ERR_ARG, "batch: c2/vpot");
  }
  return 0;
}

// time `reps` runs of one cell's queued step on s0 (after one untimed run)
int time_cell(gbcp_batch* b, Ctx& c, const gbcp_cell_io& io, int flags, double* dout, int* dst, float* ms) {
  c.stream = b->s0;
  int rc = queue_cell(c, io, flags, dout, dst);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->s0);
  const int reps = 3;
  for (int r = 0; r < reps && !rc; ++r) rc = queue_cell(c, io, flags, dout, dst);
  cudaEventRecord(e1, b->s0);
  cudaError_t e = cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) {
    c.err = cudaGetErrorString(e);
    return GBCP_ERR_CUDA;
  }
  *ms = t / reps;
  return 0;
}

}  // namespace

extern "C" {

int gbcp_batch_create(int ncells, const gbcp_grid_desc* grids, int precision, int nstreams, gbcp_batch** out) {
  if (ncells <= 0 || !grids || !out) return GBCP_ERR_ARG;
  if (nstreams <= 0) nstreams = 8;
  nstreams = std::min(nstreams, 64);
  gbcp_batch* b = new gbcp_batch();
  b->precision = precision;
  auto bail = [&](int rc) {
    gbcp_batch_destroy(b);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking) != cudaSuccess) return bail(GBCP_ERR_CUDA);
  b->ws.resize(nstreams, nullptr);
  b->join.resize(nstreams, nullptr);
  for (int w = 0; w < nstreams; ++w)
    if (cudaStreamCreateWithFlags(&b->ws[w], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join[w], cudaEventDisableTiming) != cudaSuccess)
      return bail(GBCP_ERR_CUDA);
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) return bail(GBCP_ERR_CUDA);
  for (int i = 0; i < ncells; ++i) {
    gbcp_ctx* h = nullptr;
    const int rc = gbcp_ctx_create(&grids[i], precision, 0, nullptr, &h);
    if (rc) return bail(rc);
    // the plain Z-stage gather: half as many CTAs with twice the shared memory each
    // (the mirror pairing) co-reside worse with the other cells' kernels (64-cell
    // batch: 332 000 against 355 000 state-applies/s)
    h->c.zmirror = 0;
    b->cells.push_back(h);
  }
  if (cudaMalloc(&b->d_out, sizeof(double) * 2 * ncells) != cudaSuccess ||
      cudaMalloc(&b->d_status, sizeof(int) * ncells) != cudaSuccess ||
      cudaMallocHost(&b->h_out, sizeof(double) * 2 * ncells) != cudaSuccess ||
      cudaMallocHost(&b->h_status, sizeof(int) * ncells) != cudaSuccess)
    return bail(GBCP_ERR_NOMEM);
  *out = b;
  return GBCP_OK;
}

int gbcp_batch_destroy(gbcp_batch* b) {
  if (!b) return GBCP_ERR_ARG;
  if (b->s0) cudaStreamSynchronize(b->s0);
  drop_graph(b);
  for (gbcp_ctx* h : b->cells) {
    // the context's stream is one of the batch's worker streams; give it back its own
    h->c.stream = h->c.own;
    gbcp_ctx_destroy(h);
  }
  for (cudaStream_t w : b->ws)
    if (w) cudaStreamDestroy(w);
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->s0) cudaStreamDestroy(b->s0);
  if (b->d_out) cudaFree(b->d_out);
  if (b->d_status) cudaFree(b->d_status);
  if (b->h_out) cudaFreeHost(b->h_out);
  if (b->h_status) cudaFreeHost(b->h_status);
  delete b;
  return GBCP_OK;
}

int gbcp_batch_tune(gbcp_batch* b, const gbcp_cell_io* io, int flags, char* report, int report_len) {
  if (!b) return GBCP_ERR_ARG;
  int rc = check_io(b, io, flags);
  if (rc) return rc;
  drop_graph(b);
  const int n = (int)b->cells.size();
  b->klass.assign(n, -1);
  std::vector<int> heads;
  for (int i = 0; i < n; ++i) {
    for (size_t k = 0; k < heads.size(); ++k)
      if (same_class(b->cells[heads[k]]->c, io[heads[k]].nstate, b->cells[i]->c, io[i].nstate)) {
        b->klass[i] = (int)k;
        break;
      }
    if (b->klass[i] < 0) {
      b->klass[i] = (int)heads.size();
      heads.push_back(i);
    }
  }
  b->report.clear();
  for (size_t k = 0; k < heads.size(); ++k) {
    const int i0 = heads[k];
    Ctx& c = b->cells[i0]->c;
    const gbcp_cell_io& x = io[i0];
    // private copies of the head cell's states and output so tuning leaves the caller's data alone
    const size_t esz = (flags & GBCP_STEP_PSI_C64) ? sizeof(cx<float>) : sizeof(cx<double>);
    const size_t wbytes = esz * (size_t)x.ldc * x.nstate;
    const size_t w2bytes = x.c2 ? esz * (size_t)x.ldc2 * x.nstate : 0;
    void *t0 = nullptr, *t2 = nullptr;
    if (cudaMalloc(&t0, wbytes) != cudaSuccess || (w2bytes && cudaMalloc(&t2, w2bytes) != cudaSuccess)) {
      if (t0) cudaFree(t0);
      return fail(b, GBCP_ERR_NOMEM, "batch tune: scratch");
    }
    cudaMemcpyAsync(t0, x.c0, wbytes, cudaMemcpyDeviceToDevice, b->s0);
    if (w2bytes) cudaMemcpyAsync(t2, x.c2, w2bytes, cudaMemcpyDeviceToDevice, b->s0);
    gbcp_cell_io xt = x;
    xt.c0 = static_cast<double*>(t0);
    xt.c2 = static_cast<double*>(t2);
    const int npairs = (x.nstate + 1) / 2;
    std::vector<int> engines;
    if (gbcp::fs_n1(c.nr[0]) > 0 && gbcp::fs_n1(c.nr[1]) > 0 && gbcp::fs_n1(c.nr[2]) > 0) engines.push_back(0);
    engines.push_back(2);
    std::vector<int> batches;
    for (int bt : {2, 4, 8, 16, 32, 64})
      if (bt < npairs && bt <= gbcp::kMaxBatch) batches.push_back(bt);
    if (npairs <= gbcp::kMaxBatch) batches.push_back(npairs);
    float best = 1e30f, t = 0.f;
    int best_e = c.fft_engine, best_b = c.batch, best_g = c.gemm_mode, best_p = c.plane;
    int best_ks = c.oz_ksplit, best_rg = c.oz_rgrid, best_ts = c.simt_tile, best_ch = c.chol_df;
    const int band_flags = flags & (GBCP_STEP_RHOOFR | GBCP_STEP_VPSI | GBCP_STEP_PSI_C64);
    // plane-fused y/x stages (FP32, four-step meshes whose plane fits): none, vpsi,
    // rhoofr or both
    std::vector<int> planes{0};
    if (c.precision == GBCP_PREC_MIXED) planes = {0, 1, 2, 3};
    char line[400];
    if (band_flags & (GBCP_STEP_RHOOFR | GBCP_STEP_VPSI)) {
      for (int e : engines)
        for (int bt : batches)
          for (int pl : planes) {
            if (e != 0 && pl != 0) continue;  // the plane kernels are four-step kernels
            c.fft_engine = e;
            c.batch = bt;
            c.plane = pl;
            if ((rc = time_cell(b, c, xt, band_flags, b->d_out + 2 * i0, b->d_status + i0, &t))) break;
            if (t < best) {
              best = t;
              best_e = e;
              best_b = bt;
              best_p = pl;
            }
          }
      c.fft_engine = best_e;
      c.batch = best_b;
      c.plane = best_p;
    }
    float best_o = 0.f;
    if (!rc && (flags & GBCP_STEP_ORTHO)) {
      best_o = 1e30f;
      // GEMM engine, and for the split GEMM its partition: K splits of the overlap
      // tiles and persistent CTAs of C U^-1 (many cells share the SMs in a batch)
      // (FP64 SIMT: output tile 64 or 32), and the Cholesky (blocked FP64 or, in the
      // mixed precision, double-float)
      struct Part {
        int g, ks, rg, ts;
      };
      std::vector<Part> parts{{0, 0, 0, 64}, {0, 0, 0, 32}};
      for (int ks : {0, 1, 2, 4, 8})
        for (int rg : {0, 16, 38, 76}) parts.push_back({1, ks, rg, 64});
      std::vector<int> chols{0};
      if (c.precision == GBCP_PREC_MIXED) chols.push_back(1);
      for (const Part& q : parts)
        for (int ch : chols) {
          c.gemm_mode = q.g;
          c.oz_ksplit = q.ks;
          c.oz_rgrid = q.rg;
          c.simt_tile = q.ts;
          c.chol_df = ch;
          if ((rc = time_cell(b, c, xt, GBCP_STEP_ORTHO | (flags & GBCP_STEP_PSI_C64), b->d_out + 2 * i0,
                              b->d_status + i0, &t)))
            break;
          if (t < best_o) {
            best_o = t;
            best_g = q.g;
            best_ks = q.ks;
            best_rg = q.rg;
            best_ts = q.ts;
            best_ch = ch;
          }
        }
      c.gemm_mode = best_g;
      c.oz_ksplit = best_ks;
      c.oz_rgrid = best_rg;
      c.simt_tile = best_ts;
      c.chol_df = best_ch;
    }
    cudaStreamSynchronize(b->s0);
    cudaFree(t0);
    if (t2) cudaFree(t2);
    if (rc) return fail(b, rc, "batch tune: " + c.err);
    static const char* plane_name[4] = {"three-stage", "plane vpsi", "plane rhoofr", "plane rhoofr+vpsi"};
    char gemm[96];
    const char* chol = best_ch ? "double-float" : "fp64 blocked";
    if (best_g == 1)
      std::snprintf(gemm, sizeof(gemm), "tcgen05 (K splits %s%d, C M CTAs %s%d), Cholesky %s", best_ks ? "" : "auto ",
                    best_ks, best_rg ? "" : "auto ", best_rg, chol);
    else
      std::snprintf(gemm, sizeof(gemm), "fp64-simt (tile %dx%d), Cholesky %s", best_ts, best_ts, chol);
    std::snprintf(line, sizeof(line), "mesh %dx%dx%d ngw %d nstate %d (%d cells): fft %s %s, %d pairs/launch, ortho %s; "
                                      "band %.3f ms, ortho %.3f ms\n",
                  c.nr[0], c.nr[1], c.nr[2], c.ngw, x.nstate,
                  (int)std::count(b->klass.begin(), b->klass.end(), (int)k), best_e == 0 ? "four-step" : "stockham",
                  plane_name[best_p & 3], best_b, gemm, band_flags ? best : 0.f, best_o);
    b->report += line;
    for (int i = 0; i < n; ++i)
      if (b->klass[i] == (int)k) {
        Ctx& ci = b->cells[i]->c;
        ci.fft_engine = best_e;
        ci.batch = best_b;
        ci.plane = best_p;
        ci.gemm_mode = best_g;
        ci.oz_ksplit = best_ks;
        ci.oz_rgrid = best_rg;
        ci.simt_tile = best_ts;
        ci.chol_df = best_ch;
      }
  }
  if (report && report_len > 0) {
    std::strncpy(report, b->report.c_str(), report_len - 1);
    report[report_len - 1] = 0;
  }
  return GBCP_OK;
}

int gbcp_batch_step(gbcp_batch* b, const gbcp_cell_io* io, int flags, double* energies, int32_t* status) {
  if (!b) return GBCP_ERR_ARG;
  int rc = check_io(b, io, flags);
  if (rc) return rc;
  const int n = (int)b->cells.size();
  std::vector<uintptr_t> key = make_key(b, io, flags);
  bool eager = false;
  if (!b->exec || key != b->key) {
    drop_graph(b);
    assign_streams(b, io);
    // this step runs eagerly (and allocates every workspace the captured
    // sequence will use); the capture below records it for later steps
    // without executing anything
    if ((rc = queue_all(b, io, flags))) return rc;
    if (cudaStreamSynchronize(b->s0) != cudaSuccess) return fail(b, GBCP_ERR_CUDA, "batch: eager run failed");
    eager = true;
    const long long l0 = gbcp::g_launches.load();
    if (cudaStreamBeginCapture(b->s0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return fail(b, GBCP_ERR_CUDA, "batch: begin capture");
    rc = queue_all(b, io, flags);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->s0, &g);
    if (rc || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return rc ? rc : fail(b, GBCP_ERR_CUDA, std::string("batch: capture failed: ") + cudaGetErrorString(ec));
    }
    b->kernels_per_graph = gbcp::g_launches.load() - l0;
    gbcp::g_launches.fetch_sub(b->kernels_per_graph);  // counted when the graph is launched
    if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
      cudaGraphDestroy(g);
      return fail(b, GBCP_ERR_CUDA, "batch: graph instantiation failed");
    }
    b->graph = g;
    b->key = key;
  }
  if (!eager) {
    if (cudaGraphLaunch(b->exec, b->s0) != cudaSuccess) return fail(b, GBCP_ERR_CUDA, "batch: graph launch failed");
    gbcp::count_launch((int)b->kernels_per_graph);
    const cudaError_t e = cudaStreamSynchronize(b->s0);
    if (e != cudaSuccess) return fail(b, GBCP_ERR_CUDA, cudaGetErrorString(e));
  }
  int worst = GBCP_OK;
  for (int i = 0; i < n; ++i) {
    const int s = status_code(b->h_status[i]);
    if (status) status[i] = s;
    if (s != GBCP_OK && worst == GBCP_OK) worst = s;
    if (energies) {
      energies[2 * i] = (flags & GBCP_STEP_RHOOFR) ? b->h_out[2 * i] : 0.0;
      energies[2 * i + 1] = (flags & GBCP_STEP_RHOOFR) ? b->h_out[2 * i + 1] : 0.0;
    }
  }
  if (worst != GBCP_OK) b->err = "batch: at least one cell's ortho failed (see status)";
  return worst;
}

int gbcp_batch_graph_kernels(gbcp_batch* b, int64_t* kernels) {
  if (!b || !kernels) return GBCP_ERR_ARG;
  *kernels = b->exec ? b->kernels_per_graph : 0;
  return GBCP_OK;
}

int gbcp_batch_last_error(gbcp_batch* b, char* buf, int len) {
  if (!b || !buf || len <= 0) return GBCP_ERR_ARG;
  std::strncpy(buf, b->err.c_str(), len - 1);
  buf[len - 1] = 0;
  return GBCP_OK;
}

}  // extern "C"
