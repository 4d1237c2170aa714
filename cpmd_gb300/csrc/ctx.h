// Internal context of the GB300 wavefunction hot path (not part of the ABI).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <functional>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "common.cuh"
#include "fft_core.cuh"

namespace gbcp {

// Programmatic dependent launch for chains of small dependent kernels: the
// kernel may be scheduled while its predecessor on the stream still runs and
// must call pdl_entry() before its first global-memory access (that waits for
// the predecessor grid to finish and its writes to be visible), so only the
// launch latency overlaps.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}


extern std::atomic<long long> g_launches;
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Sphere geometry as seen by the pruned 3D FFT.
//
// Columns are the (gx, gy) pairs touched by the full wavefunction sphere
// (+G and -G of every half-sphere vector), sorted by gx then gy; each column
// holds the contiguous gz range [col_zlo, col_zlo + len) and its entries
// col_ent = +(ig+1) for +G, -(ig+1) for -G, 0 for a hole.  A "slot" is one gx
// value; its columns are consecutive and cover gy in [slot_gylo, +slot_ncol).
struct GeoDev {
  int n1, n2, n3;       // mesh
  int k1, k2;           // leading dims of real-space arrays
  int ngw;
  int ncol, nslot, gxlo, nent;
  int yblk_cols;         // most sphere columns of one y-stage block of slots (four-step plan of n2)
  // the sphere's frequencies along x / y lie within [-n/4, n/4): the inverse step A
  // of a radix-8 four-step transform skips the zero half of its inputs
  int prune_x, prune_y;
  const int* col_start;  // ncol+1
  const int* col_zlo;    // ncol
  const int* col_ent;    // nent
  const int* col_slot;   // ncol
  const int* col_gy;     // ncol
  const int* ent_col;    // nent
  const int* slot_col0;  // nslot
  const int* slot_gylo;  // nslot
  const int* slot_ncol;  // nslot
  const int* pos_plus;   // ngw: entry position of +G
  const int* pos_minus;  // ngw: entry position of -G
  const double* hg;      // ngw
  const float* hg32;     // ngw, hg rounded to FP32 (the FP32 kernels' kinetic sums)
  // four-step Z-stage gather (z length with a four-step plan): for column block b,
  // n1, n2 and line l, {col_ent of column b L + l at frequency n2 + N2 n1 (0 for a
  // hole or no column), hg of that +G entry as FP32 bits}; index ((b N1 + n1) N2 + n2) L + l
  const int2* zgat;
  int geq0;              // entry 0 is G = 0
};

// largest number of state pairs one band-loop launch covers
constexpr int kMaxBatch = 64;

// Launch shape of one FFT stage: lines per CTA.
struct StageTune {
  int zl = 0, yl = 0, xl = 0;  // 0 = derive from target element count
};

struct Scratch {
  void* p = nullptr;
  size_t cap = 0;
};

// Per-kernel event timers (the analogue of the reference's tiset/tihalt
// timers, timer.mod.F90:39-130): when enabled, every launch is bracketed by
// two events on the context stream; totals are folded on read.
struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
  int lane;  // 0 context stream, 1 upload stream, 2 download stream
};
struct TimelineRec {
  std::string name;
  int lane;
  double t0, t1;  // ms after the profile was enabled
};
struct ProfAcc {
  double ms = 0.0;
  long long n = 0;
};

// Device copy of a host wavefunction array kept between host-memory calls (the
// reference's cp_cuwfn_put / cp_cuwfn_get cache, rhoofr_utils.mod.F90:240-245,
// vpsi_utils.mod.F90:278-281): rhoofr's upload of c0 into st_c0 is reused by the
// following vpsi and ortho calls on the same array, recognised by its address,
// leading dimension, state count and SUM(ABS(c0(:,1))), the reference's key.
struct WfnCache {
  bool on = false;       // GBCP_OPT_WFN_CACHE
  bool valid = false;    // st_c0 holds the array below
  const void* host = nullptr;
  const void* dev = nullptr;  // st_c0.p when it was filled (a reallocation drops the copy)
  int ldc = 0, n = 0;
  double key = 0.0;
};

struct Ctx {
  // grid
  int nr[3], kr[3], ngw, geq0;
  double omega, tpiba2;
  int precision;
  int batch;           // pairs per batch
  int gemm_mode = -1;  // overlap GEMM: -1 by precision (mixed -> tensor cores), 0 FP64 SIMT, 1 tensor cores
  int nsm = 0;         // SMs of the device
  int xr_chunks = 0;   // density x-stage pair chunks: 0 = chosen per launch
  // staging chunks of host-memory band-loop calls (0 = automatic): pairs in the
  // first chunk, number of chunks, density x-stage groups of rhoofr, pairs in the last chunk
  int stage_first = 0, stage_n = 0, stage_groups = 0, stage_last = 0;
  int zmirror = -1;    // Z-stage gather over column/mirror pairs: -1 by size, 0 off, 1 on
  int zkeep = 1;       // vpsi reuses the Z stage of the rhoofr before it on the same device states: 0 off, 1 on
  int xc = 0;          // energy functional: 0 LDA (Slater + Perdew-Zunger), 1 PBE
  int fft_engine = 0;  // band-loop FFTs: 0 four-step where a plan exists, else Stockham; 2 Stockham always
  int plane = 1;       // FP32 band loop, y and x stages fused per z-plane where the plane fits: bit 0 vpsi, bit 1 rhoofr
  int psi32 = 0;       // batch steps: c0 / c2 stored as complex64 (FP32 band loop only)
  int test_stall = 0;  // test hook: the next tensor-core overlap issues no loads and times out (one call)
  int ortho_cols = 1;  // host-memory Gram-Schmidt: C U^-1 and its download by column blocks as U^-1 finishes them
  int chol_df = 1;     // double-float Cholesky (one CTA to 64 states, diagonal blocks above): 0 never, 1 mixed, 2 both, 3 one CTA to 128
  int oz_ksplit = 0;   // split GEMM partition: K splits per overlap tile (0 = fill the SMs)
  int oz_rgrid = 0;    // split GEMM partition: persistent CTAs of C M (0 = one per SM)
  int simt_tile = 64;  // FP64 SIMT overlap / C M GEMMs: output tile 64 or 32
  const char* rmul_name = nullptr;  // profiler name of the next split C M products (Loewdin's n x n ones)
  WfnCache wfn;        // host wavefunction kept on the device between host-memory calls
  // The Z stage of a device-memory rhoofr over one launch batch, kept for a vpsi on
  // the same states: zbuf then holds their inverse z-transforms.  The host keeps
  // what identifies the call; the device compares a checksum of the states taken
  // by rhoofr (zk_sum[0]) with one taken by vpsi (zk_sum[1]), and vpsi's Z-stage
  // kernels return at once when they are equal (zk_skip = zk_sum during that vpsi).
  struct ZKeep {
    bool valid = false;
    const void* c0 = nullptr;
    int ldc = 0, nstate = 0, precision = -1, psi32 = 0;
    const void* zb = nullptr;
    size_t zcap = 0;
    bool host = false;  // a host-staged rhoofr: zbuf holds its pairs, c0 its staging copy
  } zk;
  // vpsi with host staging: c0 is the staging copy rhoofr uploaded (the wavefunction
  // cache's hit, set by the caller) and, if zk matches, zk_host skips the Z stage
  bool zk_resident = false;
  bool zk_host = false;
  Scratch zk_sum;
  const unsigned long long* zk_skip = nullptr;
  cudaEvent_t zk_ev[2] = {nullptr, nullptr};  // rhoofr's checksum on the side stream: fork, join
  cudaStream_t stream = nullptr;  // stream all work is queued on
  cudaStream_t own = nullptr;     // the context's own stream
  // geometry
  GeoDev geo{};
  std::vector<void*> dev_allocs;  // geometry arrays
  // fft plans and twiddles per axis
  FftPlan plan[3];
  cx<double>* tw64[3] = {nullptr, nullptr, nullptr};
  cx<float>* tw32[3] = {nullptr, nullptr, nullptr};
  // four-step tables per axis (sizes with a four-step plan): twA[k1*N2+n2] =
  // e^{2 pi i n2 k1/N}, twB[j*N1+k1] = e^{2 pi i k1 j/N}
  cx<double>* twA64[3] = {nullptr, nullptr, nullptr};
  cx<double>* twB64[3] = {nullptr, nullptr, nullptr};
  cx<float>* twA32[3] = {nullptr, nullptr, nullptr};
  cx<float>* twB32[3] = {nullptr, nullptr, nullptr};
  StageTune tune;
  // workspaces
  Scratch zbuf, ybuf, qbuf;
  Scratch st_c0, st_c2, st_rho, st_vpot, st_f, st_misc, st_misc2, st_vf;
  Scratch red, red2;  // reductions
  Scratch rho_sc;     // rhoofr's {E_kin, csumg, csumr} on the device
  Scratch rho_tk;     // ticket counter of the last-CTA fold of those scalars
  Scratch smat, smat2, smat3, sparts, cscr, cdiag, cwork;
  Scratch xr_part, xr_tk;  // density x-stage: partial tiles and ticket counters of the pair chunks
  Scratch rt_mats;         // rortho: the n x n matrices of the constraint iteration
  Scratch oz_a, oz_b;  // bf16 digit planes of the split-precision ortho GEMMs
  Scratch oz_c, oz_rmax;  // C M: planes and row maxima of C, sliced on the side stream while S and the Cholesky run
  Scratch nl_a, nl_b, nl_c, nl_d;
  Scratch nl_ta, nl_tb, nl_tp;  // projector GEMM slices (A, B) and split-K partials
  int* d_info = nullptr;
  double* kin = nullptr;  // tpiba2 * hg (ngw), the kinetic factor of vpsi
  const short4* wmill = nullptr;  // Miller indices of the wavefunction sphere (ngw)
  // density sphere of the energy functional (gbcp_set_dens_sphere)
  int nhg = 0, dmax = 0;           // half-sphere size, largest |Miller index|
  const int* dpos = nullptr;       // offset of +G in the (kr1, kr2, nr3) complex grid
  const int* dneg = nullptr;       // offset of -G
  const short4* dmill = nullptr;   // Miller indices (x, y, z, 0)
  const double* dg2 = nullptr;     // |G|^2 in bohr^-2
  Scratch en_rho, en_a, en_b, en_veff, en_red, en_ei, en_fp, en_idx, en_in[5];
  Scratch en_g3;  // PBE: gradient / flux grids (3 complex FFT grids)
  std::string err;
  // host-staged pipelining (abi.cu): the Z stage of staging chunk q waits for batch_ready[q];
  // vpsi calls batch_done(q) once the decode of chunk q is queued
  cudaStream_t copy = nullptr, copy_out = nullptr;  // uploads, downloads (separate copy engines)
  cudaStream_t side = nullptr;                      // ortho: C M row slicing beside S and the Cholesky
  std::vector<cudaEvent_t> side_ev;
  std::vector<cudaEvent_t> col_ev;  // host Gram-Schmidt: column block k of U^-1 forked to the side stream
  std::vector<cudaEvent_t> pipe_ev;
  const cudaEvent_t* batch_ready = nullptr;
  const cudaEvent_t* batch_c2_ready = nullptr;  // vpsi: the decode of chunk q waits for its C2 columns
  cudaEvent_t vpot_ready = nullptr;             // vpsi: the first x-stage waits for V(r)
  // rhoofr with host staging: the last density x-stage in two slabs of z planes,
  // [0, rho_zsplit) and [rho_zsplit, n3); rho_ev[i] recorded once slab i is final
  int rho_slabs = 0;
  int rho_zsplit = 0;
  const cudaEvent_t* rho_ev = nullptr;
  bool rho_ev_set = false;  // the slab events were recorded by the call's last x-stage
  std::function<int(int)> batch_done;
  std::vector<int> stage_bounds;  // staging chunks as pair ranges [b[q], b[q+1]); each is one launch batch
  // profiling
  bool prof = false;
  cudaEvent_t prof_base = nullptr;  // recorded on the context stream when profiling is enabled
  std::vector<TimelineRec> prof_tl;
  std::vector<ProfRec> prof_live;
  std::vector<cudaEvent_t> prof_pool;
  std::vector<std::pair<std::string, ProfAcc>> prof_acc;
};

// RAII launch timer; a no-op unless profiling is enabled on the context.
struct ProfScope {
  Ctx& c;
  ProfRec r{};
  bool on;
  cudaStream_t s;
  ProfScope(Ctx& ctx, const char* name);
  // work queued on another stream (the host-staging copies): lane 1 uploads, 2 downloads
  ProfScope(Ctx& ctx, const char* name, cudaStream_t stream, int lane);
  ~ProfScope();
};
void prof_fold(Ctx& c);

// Raise a kernel's dynamic shared-memory limit, once per kernel and size
// (cudaFuncSetAttribute costs host time that would otherwise be paid on
// every launch and starve the GPU of work).  Done for every size: the default
// 48 KB cap covers static plus dynamic shared memory, so a dynamic request
// just under 48 KB still fails next to a few hundred bytes of static arrays.
template <typename KernelT> inline void allow_smem(KernelT k, size_t bytes) {
  if (bytes == 0) return;
  static std::mutex mu;
  static std::unordered_map<const void*, size_t> done;
  const void* key = reinterpret_cast<const void*>(k);
  std::lock_guard<std::mutex> lock(mu);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  done[key] = bytes;
}

// grow-only scratch allocation; returns false on cudaMalloc failure
bool ensure(Ctx& c, Scratch& s, size_t bytes);

// ---- band loop (band.cu) ----
// scalars (device, may be null): {E_kin, csumg, csumr} of rhoofr (kin_energy_utils.mod.F90:93-108,
// rhoofr_utils.mod.F90:607-635), queued on the stream without a host synchronisation
int band_rhoofr(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho,
                double* scalars = nullptr);
int band_vpsi(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f, const double* vpot,
              int nstate);
int dense_fft(Ctx& c, cx<double>* grid, bool inv);
// capture-safe reductions (no host synchronisation), result in device memory:
// vrho_async -> dev_out[0] = Omega/N sum_r V rho
int vrho_async(Ctx& c, const double* rho, const double* vpot, double* dev_out);

// ---- linear algebra (linalg.cu) ----
int ovlap_gamma(Ctx& c, const cx<double>* c0, int ldc, int nstate, double* S);
int ovlap_tc(Ctx& c, const cx<double>* c0, int ldc, int nstate, double* S, unsigned long long* scond_bits,
             int* status);
// Cout may be A itself: A is sliced into digit planes before the GEMM reads them.
// zero_row1: row 1 of the result (Im c(G=0) of the real view) is written as 0.
// accumulate: Cout += A M (Cout must not alias A then).
int rmul_tc(Ctx& c, const double* A, int lda, int rows, int n, const double* M, int upper, double* Cout, int ldo,
            int zero_row1, int* status, int accumulate = 0);
// A (row-major n x n) = <X_i | Y_j> in the Γ metric, 2 Re(X^H Y) - Re X(0) Re Y(0)^T, over the
// real views X, Y (K = 2 ngw rows, leading dimensions ldx, ldy), FP64-accurate on the
// tensor cores; queued without a host synchronisation.
int xovlap_tc(Ctx& c, const double* X, int ldx, const double* Y, int ldy, int n, double* A, int* status);
// Range-pipelined forms for host-memory calls (ozaki.cu): S over K ranges kb[0..R]
// (multiples of 32 rows of the real view; range r starts once ready[r] completes) and
// C M over row ranges rb[0..R] (multiples of 128; done[r] recorded after range r).
int ovlap_tc_ranges(Ctx& c, const double* Ar, int lda, int n, const int* kb, int R, const cudaEvent_t* ready,
                    double* S, unsigned long long* scond_bits, int* status);
int rmul_tc_ranges(Ctx& c, const double* A, int lda, int rows, int n, const double* M, int upper, double* Cout,
                   int ldo, int zero_row1, int* status, const int* rb, int R, const cudaEvent_t* done,
                   const cudaEvent_t* sliced = nullptr);
// The digit planes and row maxima C M needs from A (rows x n, n <= 256), range by
// range on the side stream into oz_c / oz_rmax: range r starts once ready[r] (or, with
// ready null, the work queued so far on the context stream) is done, and sliced[r]
// (R events, from side_ev) is recorded when its planes are written.  rmul_tc_ranges
// with these events skips its own slicing.  Returns 7 when n > 256.
int slice_rows_side(Ctx& c, const double* A, int lda, int rows, int n, const int* rb, int R,
                    const cudaEvent_t* ready, const cudaEvent_t** sliced);
// Gram-Schmidt of host-memory c0 with the copies overlapped (tensor-core engine);
// returns 7 when the engine or size does not allow it (the caller stages instead).
// resident != 0: st_c0 already holds h (the wavefunction cache), no uploads
// resident: the states are already in st_c0 (the wavefunction cache).  confirm
// (may be null): called once the read-only part of a resident call is queued; false
// drops that work and returns 8, for a restart with an upload.
int ortho_gs_host(Ctx& c, double* h, int ldh, int n, double* scond_host, int resident = 0,
                  const std::function<bool()>* confirm = nullptr);
// ---- CP-dynamics constraint (rortho.cu) ----
// A (row-major n x n) = <X_i|Y_j>; tensor cores in the mixed mode, FP64 SIMT otherwise.
int xovlap(Ctx& c, const cx<double>* X, int ldx, const cx<double>* Y, int ldy, int n, double* A);
// Lagrange multipliers of the orthonormality constraint and cm += c0 gam; gam_out
// (device, n x n, may be NULL); returns 8 (not converged) past maxit with cm unchanged.
int rortho(Ctx& c, const cx<double>* c0, int ldc0, cx<double>* cm, int ldcm, int n, int tnon, double epsog, int maxit,
           double* gam_out, int* iters);
// mesh length as seen by the band-loop dispatch (-1 forces the Stockham kernels)
inline int band_len(const Ctx& c, int n) { return c.fft_engine == 2 ? -1 : n; }
inline bool use_tc_gemm(const Ctx& c) { return c.gemm_mode == 1 || (c.gemm_mode < 0 && c.precision == 1); }
int chol_inverse(Ctx& c, double* S, double* X, int n);
// the blocked chain with U^-1 finished column block by column block; column(k) is
// called with the context stream set to the side stream, once column block k is queued
int chol_inverse_columns(Ctx& c, double* S, double* X, int n, const std::function<int(int)>& column);
// C U^-1 of column block k (32 columns) from the row planes cut by slice_rows_side, on
// the context stream: the block's digit planes of M, then the tcgen05 split GEMM
int rmul_tc_column_block(Ctx& c, int rows, int n, const double* M, double* Cout, int ldo, int zero_row1,
                         int* status, int k);
int ortho_gs(Ctx& c, cx<double>* c0, int ldc, int nstate, double* scond_host);
// Gram-Schmidt queued on the stream; the status word c.d_info tells the outcome (no synchronisation)
int ortho_gs_queue(Ctx& c, cx<double>* c0, int ldc, int nstate);
int ortho_lowdin(Ctx& c, cx<double>* c0, int ldc, int nstate, double* scond_host);

// ---- energy functional and its adjoint (energy.cu) ----
// density -> potential (vofrho): V_eff (padded layout, device), energies4 (host) = {E_loc, E_H,
// E_xc, E_ext}, the local-potential forces fion (device, may be null, overwritten)
int vofrho_host_energies(Ctx& c, int nat, int nsp, const int* isp_host, const double* rho, const double* tau,
                         const double* vps, const double* vext, double* veff, double* energies4, double* fion);
int energy_and_grad(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, int nat, int nsp,
                    const int* isp_host, const double* tau, const double* vps, const double* vext,
                    double* energies_host, cx<double>* c2, int ldc2, double* dvloc, double* fion);

// ---- projectors (nonlocal.cu) ----
// fnl(ia, iv, i) at ia + lda (iv + ldp i), dfnl(ia, iv, k, i) at ia + lda (iv + ldp (k + 3 i));
// lda = 0 / ldp = 0 mean nat / ngh (a dense species block)
int nl_rnlsm1(Ctx& c, const cx<double>* c0, int ldc, int nstate, int nat, int ngh, const int* nghtol_host,
              const double* twnl, const cx<double>* eigr, double* fnl, int lda = 0, int ldp = 0);
int nl_rnlsm2(Ctx& c, const cx<double>* c0, int ldc, int nstate, int nat, int ngh, const int* nghtol_host,
              const double* twnl, const cx<double>* eigr, double* dfnl, int lda = 0, int ldp = 0);
int nl_rnlfor(Ctx& c, int nstate, const double* f, int nat, int ngh, const double* wsg, const double* fnl,
              const double* dfnl, double* fion, int lda = 0, int ldp = 0);
int nl_fnonloc(Ctx& c, cx<double>* c2, int ldc2, int nstate, const double* f, int nat, int ngh,
               const int* nghtol_host, const double* twnl, const cx<double>* eigr, const double* fnl,
               const double* wsg, int lda = 0, int ldp = 0);

}  // namespace gbcp

#define GBCP_CUDA_TRY(ctx, expr)                                                   \
  do {                                                                           \
    cudaError_t e_ = (expr);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      (ctx).err = std::string(#expr) + ": " + cudaGetErrorString(e_);           \
      return 5;                                                                  \
    }                                                                            \
  } while (0)

#define GBCP_LAUNCH_CHECK(ctx)                                                    \
  do {                                                                           \
    ::gbcp::count_launch();                                                      \
    cudaError_t e_ = cudaGetLastError();                                         \
    if (e_ != cudaSuccess) {                                                     \
      (ctx).err = std::string("launch: ") + cudaGetErrorString(e_) + " at " + __FILE__ + ":" + std::to_string(__LINE__); \
      return 5;                                                                  \
    }                                                                            \
  } while (0)

// GBCP_LAUNCH_PDL: launch_pdl with the error handling of GBCP_LAUNCH_CHECK.
#define GBCP_LAUNCH_PDL(ctx, kernel, grid, block, smem, ...)                      \
  do {                                                                           \
    ::gbcp::count_launch();                                                      \
    cudaError_t e_ = ::gbcp::launch_pdl(kernel, grid, block, smem, (ctx).stream, __VA_ARGS__); \
    if (e_ == cudaSuccess) e_ = cudaGetLastError();                              \
    if (e_ != cudaSuccess) {                                                     \
      (ctx).err = std::string("launch: ") + cudaGetErrorString(e_) + " at " + __FILE__ + ":" + std::to_string(__LINE__); \
      return 5;                                                                  \
    }                                                                            \
  } while (0)

// The opaque handle of the C ABI.
struct gbcp_ctx {
  gbcp::Ctx c;
};
