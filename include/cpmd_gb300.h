/*
 * cpmd_gb300.h -- C ABI of the GB300-native CPMD wavefunction hot path.
 *
 * Every entry point replaces one CPMD Fortran routine of the Γ-point,
 * norm-conserving band loop; a Fortran caller binds them with
 * ISO_C_BINDING exactly like src/cuuser_interfaces.mod.F90:41-201 binds
 * CuUser_C_* (pointers as TYPE(C_PTR) by value, integers by value).
 *
 * Conventions
 *  - Complex arrays are interleaved (re, im) FP64, i.e. COMPLEX(real_8),
 *    column-major with an explicit leading dimension (in complex elements).
 *  - Real-space arrays (rhoe, vpot) use the reference's padded layout
 *    (kr1, kr2, kr3) with x fastest (fpar%kr1, kr2s, kr3s; kr = nr + mod(nr+1,2)),
 *    loadpa_utils.mod.F90:509-525, loadpa_utils.mod.F90:432.
 *  - `mem` says where ALL array arguments of a call live:
 *    GBCP_MEM_HOST   -> the call stages through device buffers owned by the
 *                       context and synchronises before returning;
 *    GBCP_MEM_DEVICE -> pointers are device pointers; work is queued on the
 *                       context's stream; the call synchronises only when it
 *                       returns host scalars (non-NULL scalar outputs).
 *  - Every call returns a status (GBCP_OK = 0).  The reference aborts through
 *    stopgm (error_handling.mod.F90:11-53); here the caller decides.
 *  - A context is not thread-safe; use one per host thread / stream.
 */
#ifndef CPMD_GB300_H
#define CPMD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbcp_ctx gbcp_ctx;

enum gbcp_status {
  GBCP_OK = 0,
  GBCP_ERR_ARG = 1,        /* bad argument (NULL, size, layout) */
  GBCP_ERR_NOT_SPD = 2,    /* overlap matrix not positive definite (rgs_utils.mod.F90:127-155) */
  GBCP_ERR_NONFINITE = 3,  /* NaN/Inf detected in an input or a reduction */
  GBCP_ERR_TIMEOUT = 4,    /* a bounded device-side wait expired */
  GBCP_ERR_CUDA = 5,       /* CUDA runtime error */
  GBCP_ERR_NOMEM = 6,      /* device allocation failed */
  GBCP_ERR_UNSUPPORTED = 7,/* mesh size / option not supported */
  GBCP_ERR_NOT_CONVERGED = 8, /* iterative Loewdin step or rortog iteration did not converge */
  GBCP_ERR_IO = 9,         /* RESTART file cannot be opened, written, or is malformed */
  GBCP_ERR_CHARGE = 10     /* rhoofr: density sums in real and Fourier space differ
                              (rhoofr_utils.mod.F90:625-635, where the reference stops) */
};

enum gbcp_precision {
  GBCP_PREC_FP64 = 0,  /* plain FP64 drop-in */
  GBCP_PREC_MIXED = 1  /* FP32 FFT and V*psi, FP64 reductions and accumulation */
};

enum gbcp_mem { GBCP_MEM_HOST = 0, GBCP_MEM_DEVICE = 1 };

enum gbcp_ortho_method {
  GBCP_ORTHO_GS = 0,     /* rgs: Cholesky Gram-Schmidt (ortho_utils.mod.F90:256) */
  GBCP_ORTHO_LOWDIN = 1  /* lowdin (ortho_utils.mod.F90:193) */
};

/* Grid and basis description: the module globals the reference hot path reads
 * (system.mod: spar%nr*s, fpar%kr*, ncpw%ngw, parm%omega, parm%tpiba2, geq0;
 * cppt: inyh, hg). */
typedef struct gbcp_grid_desc {
  int32_t nr1, nr2, nr3;  /* FFT mesh */
  int32_t kr1, kr2, kr3;  /* leading dimensions of real-space arrays */
  int32_t ngw;            /* wavefunction half-sphere size */
  int32_t geq0;           /* 1 if entry 0 is G = 0 */
  double omega;           /* cell volume (bohr^3) */
  double tpiba2;          /* (2 pi / alat)^2 */
  const int32_t* inyh;    /* (3, ngw) Fortran order: Miller index + nr/2 + 1 (cppt::inyh) */
  const double* hg;       /* (ngw) |G|^2 in tpiba2 units (cppt::hg) */
} gbcp_grid_desc;

/* Context creation: builds the sphere/column maps, FFT plans and twiddles
 * once (the reference's fft_init/setfftn, fftprp_utils.mod.F90:65-95,
 * fftnew_utils.mod.F90:101-170).  `stream` is a cudaStream_t or NULL (the
 * context then creates its own).  `max_batch` is the number of state pairs
 * transformed per launch (0 = default). */
int gbcp_ctx_create(const gbcp_grid_desc* grid, int precision, int max_batch, void* stream, gbcp_ctx** out);
int gbcp_ctx_destroy(gbcp_ctx* ctx);
int gbcp_set_precision(gbcp_ctx* ctx, int precision);

/* Options (the reference's &CPMD GPU keywords, control_utils.mod.F90:2856-2894,
 * become per-context settings):
 *   GBCP_OPT_GEMM   overlap GEMM engine: -1 = by precision (MIXED -> tensor
 *                   cores), 0 = FP64 SIMT, 1 = tcgen05 split-precision
 *                   (FP64-level: per product term below 2^-52 of the scale
 *                   of its row and column maxima, the overlap rounded once,
 *                   C M within 2^-54 of that scale more);
 *   GBCP_OPT_BATCH  state pairs per band-loop launch (1..64);
 *   GBCP_OPT_FFT    band-loop FFT kernels: 0 = four-step register codelets
 *                   where the mesh has a plan, else Stockham; 2 = Stockham;
 *   GBCP_OPT_XCHUNKS pair chunks of the density x-stage (four-step kernels):
 *                   0 = chosen per launch from the SM count, 1..8 = fixed;
 *   GBCP_OPT_XC     exchange-correlation functional of gbcp_energy: 0 = LDA
 *                   (Slater + Perdew-Zunger, the default), 1 = PBE (gradient-
 *                   corrected, the reference's vofrhob/gcener route);
 *   GBCP_OPT_PLANE  FP32 band loop: the y and x stages of each z-plane in one
 *                   kernel, the plane held in shared memory (no y-stage buffer
 *                   in HBM), where the x and y lengths are equal and the plane
 *                   fits; bit 0 for vpsi, bit 1 for rhoofr (default 1: vpsi only,
 *                   the faster split on the 120^3 cell); 0 = three-stage kernels;
 *   GBCP_OPT_WFN_CACHE  1 = keep the device copy of a host-memory c0 that
 *                   gbcp_rhoofr uploads, and let the following gbcp_vpsi and
 *                   gbcp_ortho (Gram-Schmidt) on the same array use it instead
 *                   of uploading again -- the reference's cp_cuwfn cache
 *                   (rhoofr_utils.mod.F90:240-245, vpsi_utils.mod.F90:278-281),
 *                   recognised like there by the array (address, leading
 *                   dimension, states) and SUM(ABS(c0(:,1))); gbcp_ortho ends
 *                   it (it rewrites c0).  A caller that changes c0 on the host
 *                   in a way that keeps that key must drop the copy by setting
 *                   the option again (any value).  0 (the default) = off;
 *   GBCP_OPT_CHOL   Cholesky factor and inverse of the ortho overlap matrix:
 *                   0 = blocked FP64 over many CTAs; 1 (the default) = in the
 *                   MIXED precision, double-float arithmetic (FP32 pairs, about
 *                   2^-46 relative per operation) for the whole job in one CTA
 *                   up to 64 states and for the 32 x 32 diagonal blocks of the
 *                   blocked chain above, where FP64 pivot chains are slow on
 *                   GB300; a pivot at or below 2^-40 of its row's original
 *                   diagonal then reports GBCP_ERR_NOT_SPD (the FP64 chain:
 *                   2^-46); 2 = that in both precisions; 3 = as 2, with the
 *                   one-CTA kernel up to 128 states;
 *   GBCP_OPT_SIMT_TILE  output tile of the FP64 SIMT overlap and C M GEMMs:
 *                   64 (the default) or 32 (less padding for small state
 *                   counts; the batch autotuner chooses per size class);
 *   GBCP_OPT_STAGES  staging of host-memory rhoofr / vpsi calls, whose copies
 *                   overlap the transforms chunk by chunk: 0 (the default) =
 *                   automatic; otherwise (pairs in the first chunk) + 256 x
 *                   (number of chunks) + 65536 x (density x-stage groups of
 *                   rhoofr) + 16777216 x (pairs in the last chunk, 0 = equal
 *                   to the others);
 *   GBCP_OPT_ZMIRROR  Z-stage gather of the four-step band loop: -1 (the
 *                   default) = over pairs of mirror columns (each coefficient
 *                   loaded once) where the sphere has at least 48 column
 *                   blocks, 0 = off, 1 = on; a batch turns it off;
 *   GBCP_OPT_ZKEEP  1 (the default) = a device-memory gbcp_vpsi that follows a
 *                   device-memory gbcp_rhoofr on the same c0 (pointer, leading
 *                   dimension and state count, both calls one launch batch)
 *                   reuses rhoofr's inverse z-transforms of the states when a
 *                   position-keyed 64-bit checksum of all of c0, taken on the
 *                   device by both calls, is unchanged (the reference reuses its
 *                   device copy of c0 on a match of SUM(ABS(c0(:,1))),
 *                   vpsi_utils.mod.F90:278-281); 0 = off;
 *   GBCP_OPT_ORTHO_COLUMNS  host-memory Gram-Schmidt of 65 to 256 states on the
 *                   tensor cores: 1 (the default) = C U^-1 and its download go
 *                   column block by column block (32 states) as the Cholesky
 *                   chain finishes each block of U^-1, so the copy starts after
 *                   the first diagonal block; 0 = by G-row ranges after the whole
 *                   chain (the same states bit for bit);
 *   GBCP_OPT_TEST_TIMEOUT  test hook of the failure path: 1 = the next overlap
 *                   on the tensor cores issues no operand loads, so its first
 *                   bounded wait (no copy in flight towards it) runs out after
 *                   about a millisecond; the call returns GBCP_ERR_TIMEOUT with
 *                   c0 untouched and the hook clears itself. */
enum gbcp_option { GBCP_OPT_GEMM = 1, GBCP_OPT_BATCH = 2, GBCP_OPT_FFT = 3, GBCP_OPT_XCHUNKS = 4, GBCP_OPT_XC = 5,
                   GBCP_OPT_WFN_CACHE = 6, GBCP_OPT_PLANE = 7, GBCP_OPT_CHOL = 8,
                   GBCP_OPT_SIMT_TILE = 9, GBCP_OPT_STAGES = 10, GBCP_OPT_ZMIRROR = 11,
                   GBCP_OPT_ZKEEP = 12, GBCP_OPT_ORTHO_COLUMNS = 13,
                   GBCP_OPT_TEST_TIMEOUT = 90 };
int gbcp_set_option(gbcp_ctx* ctx, int key, int value);
/* Queue later work on `stream` (a cudaStream_t; NULL = the context's own
 * stream; the CUDA legacy default stream is cudaStreamLegacy).  Device-pointer calls are ordered only with respect to this stream,
 * as the reference's GPU path orders work on its thread's stream
 * (thread_view, vpsi_utils.mod.F90:295). */
int gbcp_set_stream(gbcp_ctx* ctx, void* stream);
int gbcp_synchronize(gbcp_ctx* ctx);
/* Last error message of this context (NUL-terminated, truncated to len). */
int gbcp_last_error(gbcp_ctx* ctx, char* buf, int len);
/* Number of kernels this library has launched in this process (all contexts). */
int64_t gbcp_kernel_launches(void);

/* Per-kernel timers, the counterpart of the reference's tiset/tihalt wall-clock
 * table (timer.mod.F90:39-130) and NVTX ranges (cpmd_global.h:93-98).
 * enable != 0 clears the table and brackets every later launch with CUDA
 * events on the context stream; gbcp_profile_read synchronises, then returns
 * entry `idx` (name, total milliseconds, launch count) or GBCP_ERR_ARG past
 * the last entry. */
int gbcp_profile_enable(gbcp_ctx* ctx, int enable);
int gbcp_profile_read(gbcp_ctx* ctx, int idx, char* name, int name_len, double* total_ms, int64_t* count);
/* Timeline of the same records since the last enable: entry `idx` (name, lane:
 * 0 context stream, 1 host->device staging copies, 2 device->host copies, and
 * start / end in milliseconds after the enable), in the order they were queued;
 * GBCP_ERR_ARG past the last entry. */
int gbcp_profile_timeline(gbcp_ctx* ctx, int idx, char* name, int name_len, int* lane, double* t0_ms, double* t1_ms);

/* rhoofr(c0, rhoe, psi, nstate)            rhoofr_utils.mod.F90:122-644
 * rhoe(kr1,kr2,kr3) = sum_i f_i/omega psi_i(r)^2 (zero in the padding);
 * ekin = tpiba2 sum_i f_i sum_G hg |c|^2 (kin_energy_utils.mod.F90:93-108);
 * csumg = sum_i f_i <c_i|c_i>; csumr = sum_r rhoe * omega / (nr1 nr2 nr3)
 * (rhoofr_utils.mod.F90:607-635).  Scalar outputs (host) may be NULL; when
 * any is given the call synchronises once and applies the reference's charge
 * check: |csumr - csumg| above 1e-6 (FP64) or 1e-6 csumg (mixed) returns
 * GBCP_ERR_CHARGE with all outputs written.  In the mixed mode E_kin and csumg
 * square the FP32-rounded coefficients (relative error 2^-24 per term,
 * unbiased) and sum them in double-float. */
int gbcp_rhoofr(gbcp_ctx* ctx, const double* c0, int ldc, int nstate, const double* f, double* rhoe,
                double* ekin, double* csumg, double* csumr, int mem);

/* vpsi(c0, c2, f, vpot, psi, nstate, ...)  vpsi_utils.mod.F90:120-732 (Γ branch 661-671)
 * c2 += -f/2 (tpiba2 hg c0 + FFT[V psi]) per state (add_wfn, l.717). */
int gbcp_vpsi(gbcp_ctx* ctx, const double* c0, int ldc, double* c2, int ldc2, const double* f,
              const double* vpot, int nstate, int mem);

/* ortho(nstate, c0, cscr)                  ortho_utils.mod.F90:124-272
 * In-place orthonormalisation in the Γ metric, then zclean.  `scond` (may be
 * NULL) receives max|S - I| of the input overlap (csmat_utils.mod.F90:82-89). */
int gbcp_ortho(gbcp_ctx* ctx, double* c0, int ldc, int nstate, int method, double* scond, int mem);

/* Overlap matrix only: S = 2 Re(C^H C) - Re c(0) Re c(0)^T, full n x n
 * column-major (ovlap_utils.mod.F90:150-165, symmetric branch). */
int gbcp_ovlap(gbcp_ctx* ctx, const double* c0, int ldc, int nstate, double* smat, int mem);

/* Orthonormality constraint of Car-Parrinello dynamics: rortog -> rortho
 * (rortog_utils.mod.F90:43-87, 315-498) with rotate (rotate_utils.mod.F90:63-101).
 * c0 (orthonormal) and cm (the propagated wavefunctions): ngw x nstate complex,
 * leading dimensions ldc0, ldcm, distinct arrays.  Iterates the Lagrange
 * multipliers until max|gam' - gam| <= epsog/2, at most maxit iterations (the
 * reference's defaults: 1e-6 and 30), symmetrises them, writes gam
 * (nstate x nstate, column-major; may be NULL) and updates cm += c0 gam.
 * tnon != 0: c0 is not exactly orthonormal (the del = (I - <c0|c0>)/2 term).
 * *iters (may be NULL): iterations done.  GBCP_ERR_NOT_CONVERGED past maxit,
 * cm unchanged (the reference stops). */
int gbcp_rortog(gbcp_ctx* ctx, const double* c0, int ldc0, double* cm, int ldcm, int nstate, int tnon, double epsog,
                int maxit, double* gam, int* iters, int mem);

/* Allocation-free overlap matrix.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc (an application whose device memory
 * is all owned by its own pool allocator, or a time-stepping loop that must
 * not stall the device with an allocation's implicit synchronisation).  Same
 * S as gbcp_ovlap, from device pointers only, queued on `stream` (a
 * cudaStream_t; NULL = the legacy default stream); needs no context.
 * It calls no cudaMalloc/cudaFree: its split-K partial sums live in a fixed
 * 8 MiB device array inside the library (held by every GPU that loads the
 * library until the process exits), so nstate <= 1024 (GBCP_ERR_ARG above).
 * The first call in each CUDA context (normally: once per device, with that
 * device current) looks up the array's device address in that context
 * (cudaGetSymbolAddress) and remembers it under the context's unique id, so a
 * new context after cudaDeviceReset, or a caller's own driver-API context, gets
 * its own lookup; make that first call before any stream capture.  An error
 * already pending in the calling thread is returned as GBCP_ERR_CUDA without
 * launching.  All calls share the array: calls whose work overlaps on the GPU
 * race.  c0: device, complex, leading dimension ldc >= ngw;
 * smat: device, nstate x nstate. */
int gbcp_ovlap_noalloc(const double* c0, int ldc, int ngw, int nstate, int geq0, double* smat, void* stream);

/* invfftn / fwfftn                          fftmain_utils.mod.F90:373-431
 * Dense in-place 3D FFT of a complex grid laid out (kr1, kr2, nr3), x fastest,
 * G stored at FFT index (g mod nr).  inv: e^{+iGr}, unscaled;
 * fw: e^{-iGr}, scaled 1/(nr1 nr2 nr3). */
int gbcp_invfftn(gbcp_ctx* ctx, double* f, int mem);
int gbcp_fwfftn(gbcp_ctx* ctx, double* f, int mem);

/* rnlsm(c0, nstate, ...) -> rnlsm1         rnlsm1_utils.mod.F90:42-193
 * One species of nat atoms with ngh projectors of angular momentum nghtol[iv]:
 * fnl(ia, iv, i) = 2 Re sum_G conj((-i)^l twnl(G,iv) eigr(G,ia)) c(G),
 * with the G = 0 term halved.  twnl(ngw, ngh) real, eigr(ngw, nat) complex.
 * fnl layout: element (ia, iv, i) at fnl[ia + ld_atoms (iv + ld_proj i)], so a
 * species block of the reference's global fnl(imagp, ions1%nat, maxsys%nhxs,
 * nstate) is written in place with fnl = C_LOC(fnl(1, isa0+1, 1, 1)),
 * ld_atoms = ions1%nat, ld_proj = maxsys%nhxs (rnlsm1_utils.mod.F90:156-165);
 * only the block's own entries are written.  ld_atoms = 0 / ld_proj = 0 mean
 * nat / ngh (a dense (nat, ngh, nstate) array). */
int gbcp_rnlsm1(gbcp_ctx* ctx, const double* c0, int ldc, int nstate, int nat, int ngh, const int32_t* nghtol,
                const double* twnl, const double* eigr, double* fnl, int ld_atoms, int ld_proj, int mem);

/* rnlsm2(c0, nstate, ikpt, ikind)          rnlsm2_utils.mod.F90:41-299 (Γ branch l.190-240)
 * dfnl(ia, iv, k, i) = d fnl / d R_k
 *   = 2 tpiba Re sum_G conj((-i)^(l+1) twnl(G,iv) eigr(G,ia) G_k) c(G), G = 0 halved,
 * G_k the Miller index along k (cubic cell).  Same operands as gbcp_rnlsm1;
 * dfnl layout: element (ia, iv, k, i) at dfnl[ia + ld_atoms (iv + ld_proj (k + 3 i))],
 * the reference's dfnl(imagp, ions1%nat, maxsys%nhxs, 3, nstate) seen from
 * dfnl(1, isa0+1, 1, 1, 1); 0 / 0 mean a dense (nat, ngh, 3, nstate) array. */
int gbcp_rnlsm2(gbcp_ctx* ctx, const double* c0, int ldc, int nstate, int nat, int ngh, const int32_t* nghtol,
                const double* twnl, const double* eigr, double* dfnl, int ld_atoms, int ld_proj, int mem);

/* rnlfor(fion, f, wk, nstate, nkpoint)      rnlfor_utils.mod.F90:41-368 (KB branch l.283-330)
 * fion(3, nat) -= sum_i sum_iv 2 wsg(iv) f_i fnl(ia,iv,i) dfnl(ia,iv,k,i) for |f_i| > 1e-12
 * (accumulated, like the reference; Γ point, one species); fnl and dfnl in the
 * layouts of gbcp_rnlsm1 / gbcp_rnlsm2 with the same ld_atoms, ld_proj. */
int gbcp_rnlfor(gbcp_ctx* ctx, int nstate, const double* f, int nat, int ngh, const double* wsg, const double* fnl,
                const double* dfnl, int ld_atoms, int ld_proj, double* fion, int mem);

/* fnonloc(c2, f, nstate, ...)               fnonloc_utils.mod.F90:306-354 (BHS/KB branch)
 * c2(G,i) += sum_iv twnl(G,iv) (-i)^l (-f_i wsg(iv)) sum_ia eigr(G,ia) fnl(ia,iv,i),
 * f_i < 1e-5 counted as 1; fnl in the layout of gbcp_rnlsm1 (the reference reads
 * fnl(1, isa0+1, iv, i), fnonloc_utils.mod.F90:322-324). */
int gbcp_fnonloc(gbcp_ctx* ctx, double* c2, int ldc2, int nstate, const double* f, int nat, int ngh,
                 const int32_t* nghtol, const double* twnl, const double* eigr, const double* fnl, int ld_atoms,
                 int ld_proj, const double* wsg, int mem);

/* Density sphere of the energy functional (cppt: nhg, inyh(3,nhg), hg(nhg);
 * the first ngw entries are the wavefunction sphere of gbcp_grid_desc).
 * Host arrays; copied once (the reference's loadpa/rggen set-up). */
int gbcp_set_dens_sphere(gbcp_ctx* ctx, int nhg, const int32_t* inyh, const double* hg);

/* Energy of the local-potential Kohn-Sham functional and its adjoint
 * (the proposed gbcp_energy_and_grad; the reference computes the same terms
 * in vofrhoa_utils.mod.F90:41-144, ppener_utils.mod.F90:23-108,
 * potfor_utils.mod.F90:38-110, cp_lda_*; cubic cell):
 *   E = E_kin + E_loc + E_H + E_xc + E_ext,
 *   V_ion(G) = sum_a vps(G, isp[a]) e^{-iG.R_a}, E_loc = Omega sum_G conj(rho(G)) V_ion(G),
 *   E_H = Omega sum_{G!=0,half} 4 pi |rho(G)|^2 / G^2, E_xc = LDA (Slater + Perdew-Zunger),
 *   E_ext = Omega/N sum_r vext rho (vext may be NULL).
 * Inputs: c0 (ngw, nstate), f (nstate), tau (3, nat) bohr, vps (nhg, nsp)
 * form factors per unit volume, isp (nat) species 0..nsp-1 (HOST array in
 * both memory modes), vext (kr1, kr2, kr3) or NULL.  nat = 0 means no ions.
 * Outputs (any of c2 / dvloc / fion may be NULL):
 *   energies[6] (host) = {E, E_kin, E_loc, E_H, E_xc, E_ext} in Ha;
 *   c2 (ngw, nstate) overwritten with the CP force -(f/2)(G^2 c + 2 [V_eff psi](G)),
 *     i.e. the reference's vpsi applied to V_eff = V_ion + V_H + v_xc + vext;
 *     dE = -4 Re sum_G w_G conj(dc) c2 with w = 1/2 at G = 0, 1 elsewhere
 *     (states with f = 0 follow vpsi's convention and are not gradients);
 *   dvloc (kr1, kr2, kr3) = dE/dV(r) = rho(r) Omega / (nr1 nr2 nr3);
 *   fion (3, nat) overwritten with -dE/dR.
 * The band loop runs in the context precision; everything else is FP64. */
int gbcp_energy(gbcp_ctx* ctx, const double* c0, int ldc, int nstate, const double* f, int nat, int nsp,
                const int32_t* isp, const double* tau, const double* vps, const double* vext, double* energies,
                double* c2, int ldc2, double* dvloc, double* fion, int mem);

/* Density -> potential, the reference's vofrho for a local pseudopotential
 * (rscpot_utils.mod.F90:132 -> vofrhoa_utils.mod.F90:41-144 with the xc step of
 * vofrhob_utils.mod.F90:80-471; cubic cell): from rhoe (kr1, kr2, kr3) to
 *   veff (kr1, kr2, kr3) = V_ion + V_H + v_xc (+ vext), the V(r) that vpsi and the
 *   caller's own fnonloc / force sequence then use (forces_driver.mod.F90:224);
 *   energies[4] (host) = {E_loc, E_H, E_xc, E_ext} in Ha, as in gbcp_energy;
 *   fion (3, nat) overwritten with the local-potential forces (may be NULL).
 * The other arguments are those of gbcp_energy; GBCP_OPT_XC selects LDA or PBE. */
int gbcp_vofrho(gbcp_ctx* ctx, const double* rhoe, int nat, int nsp, const int32_t* isp, const double* tau,
                const double* vps, const double* vext, double* veff, double* energies, double* fion, int mem);

/* General overlap, the reference's ovlap with c1 != c2 (ovlap_utils.mod.F90:157-166,
 * dgemm('T','N') over the real views plus the dger G = 0 correction):
 *   a(i, j) = <c1_i|c2_j> = 2 Re sum_G conj(c1_i) c2_j - Re c1_i(0) Re c2_j(0),
 * a (nstate x nstate) column-major; used for the Lagrange multipliers of CP
 * dynamics (forces_driver.mod.F90:262).  FP64 SIMT, or the FP64-accurate split
 * GEMM on the tensor cores when GBCP_OPT_GEMM selects it. */
int gbcp_ovlap2(gbcp_ctx* ctx, const double* c1, int ldc1, const double* c2, int ldc2, int nstate, double* amat,
                int mem);

/* ---- Batches of independent cells (no counterpart in the reference, where
 * every cell is a separate run).  A batch owns one context per cell; a step
 * runs, for every cell, any of rhoofr (+ E_kin and int V rho in FP64),
 * vpsi and Gram-Schmidt ortho, captured once into a CUDA graph and replayed
 * with one graph launch per step.  All cell arrays are DEVICE pointers. */
typedef struct gbcp_batch gbcp_batch;
typedef struct gbcp_cell_io {
  double* c0;          /* (ldc, nstate) complex; orthonormalised in place by GBCP_STEP_ORTHO */
  int32_t ldc;
  int32_t nstate;
  const double* f;     /* (nstate) */
  const double* vpot;  /* (kr1, kr2, kr3) */
  double* rhoe;        /* (kr1, kr2, kr3) output of GBCP_STEP_RHOOFR */
  double* c2;          /* (ldc2, nstate) complex, accumulated by GBCP_STEP_VPSI */
  int32_t ldc2;
} gbcp_cell_io;
/* GBCP_STEP_PSI_C64 (MIXED batches): c0 and c2 of every cell hold complex64
 * (pairs of float, ldc / ldc2 in complex elements) instead of complex128.  The
 * band loop reads and accumulates them directly (half the coefficient traffic);
 * ortho widens c0 to FP64, runs the FP64-accurate Gram-Schmidt and rounds the
 * result back, so its orthonormality is that of complex64 (~1e-7); E_kin and
 * int V rho stay FP64 sums. */
enum gbcp_step_flags { GBCP_STEP_RHOOFR = 1, GBCP_STEP_VPSI = 2, GBCP_STEP_ORTHO = 4, GBCP_STEP_PSI_C64 = 8 };
/* `nstreams` worker streams run cells side by side (0 = 8). */
int gbcp_batch_create(int ncells, const gbcp_grid_desc* grids, int precision, int nstreams, gbcp_batch** out);
int gbcp_batch_destroy(gbcp_batch* batch);
/* Autotuner: per size class (equal mesh, sphere and nstate) times every
 * band-loop configuration (four-step or Stockham FFT kernels x pairs per
 * launch) and both ortho GEMM engines on private copies of the class's first
 * cell, and keeps the fastest.  `report` (may be NULL) gets one line per class. */
int gbcp_batch_tune(gbcp_batch* batch, const gbcp_cell_io* io, int flags, char* report, int report_len);
/* One step over all cells.  energies (host, may be NULL): 2 per cell, E_kin and
 * Omega/N sum V rho of the input states; status (host, may be NULL): per-cell
 * GBCP status of ortho.  Returns the first non-OK cell status. */
int gbcp_batch_step(gbcp_batch* batch, const gbcp_cell_io* io, int flags, double* energies, int32_t* status);
/* Kernels in the captured step graph (0 before the first step). */
int gbcp_batch_graph_kernels(gbcp_batch* batch, int64_t* kernels);
int gbcp_batch_last_error(gbcp_batch* batch, char* buf, int len);

/* ---- RESTART wavefunction file (Gamma point) --------------------------------
 * The reference's restart file (zhwwf/wv30, wv30_utils.mod.F90:99-233,235-1300;
 * zhrwf/rv30, rv30_utils.mod.F90:104-2242): Fortran unformatted records with
 * 4-byte length markers, sections 1..99 each opened by a record (irecord, fpos)
 * giving the number of records that follow.  Written: 1 header, 2 cell,
 * 3 species counts, 4 tau0, 5 taum, 6 taui (5 and 6 only when given), 7 cutoff /
 * electrons / mesh, 8 states and plane-wave counts, 9 the states C0 in the
 * w_wfnio layout (wfnio_utils.mod.F90:52-233: type 1, then per state the
 * coefficients in the global G order, compress.F90: icompr 1 = FP64 as is,
 * 2 = 32-bit fixed point on the scale max|c|), 10 the velocities cm when given
 * (wr30wfn_utils.mod.F90:569-693, 'NIL': scale max|component|), 23 occupation
 * numbers and 24 the Fermi energy and eigenvalues when given, the others empty.
 * Read: sections 1..10, 23 and 24 of a sequential or STREAM file (icompr 1, 2, 4
 * or 8; the C0 format with a negative section-9 record count, either format of
 * section 10), skipping 11..22 by their record counts; the file may end after
 * section 9.
 * The coefficient order is the reference's global G order, which is the order
 * of the basis (inyh/hg) a context is created with. */
typedef struct gbcp_restart {
  int32_t ibrav, indpg;   /* section 2 (parm%ibrav, symmi%indpg) */
  double celldm[6];       /* section 2 (cell_com%celldm) */
  int32_t nsp, nat;       /* section 3: species and atoms */
  int32_t* na;            /* (nsp) atoms per species */
  double* tau0;           /* (3, nat) section 4, species-major like tau0(:,ia,is) */
  double* taum;           /* (3, nat) section 5 (velocities); write: NULL = empty section */
  double* taui;           /* (3, nat) section 6 (initial positions); write: NULL = empty */
  double ecut, cdual;     /* section 7: cutoff (Ry), dual */
  int32_t dual, nel;      /* section 7: dual flag, number of electrons */
  int32_t nr1s, nr2s, nr3s;
  int32_t nstate, nkpts;  /* section 8: crge%n, k points (0 = Gamma) */
  int32_t ngwks, ngwls, nhgs, nhgls;
  double* c0;             /* (ldc, nstate) complex; read: (ldc, nstate_cap), rows beyond the
                             file's plane waves zeroed, states beyond nstate_read untouched */
  int32_t ldc;            /* leading dimension of c0 (complex elements) */
  int32_t ngw;            /* write: rows of c0 stored (the file's plane waves); read: rows of c0 filled */
  int32_t nstate_cap;     /* read: states c0 can hold */
  int32_t icompr;         /* write: 1 or 2; read: the file's */
  double scale;           /* read: the file's compression scale */
  int32_t nstate_read;    /* read: states stored into c0 */
  int32_t nstate_file;    /* read: states in the file's section 9 */
  int32_t sections;       /* read: bit (k-1) set when section k (1..24) held data */
  double* f;              /* (nstate) section 23 occupation numbers (crge%f); write: NULL = empty */
  double* eigv;           /* (nstate) section 24 eigenvalues; write: NULL = empty */
  double amu;             /* section 24 Fermi energy (ener_com%amu) */
  double* cm;             /* (ldc, nstate) section 10 wavefunction velocities, laid out like c0;
                             write: NULL = empty section; read: NULL = skipped */
  int32_t ncm_read;       /* read: velocity states stored into cm */
  int32_t pad_;
} gbcp_restart;
/* Write `path` (overwritten). */
int gbcp_restart_write(const char* path, const gbcp_restart* r);
/* Read `path`: every scalar field of sections 2, 3, 7, 8, 9, 10 and 24 is filled; array
 * fields that are NULL are skipped (call once with NULL arrays to learn nsp,
 * nat, nstate, ngwks, then allocate).  Inputs: the array pointers, ldc, ngw and
 * nstate_cap; min(nstate_cap, states in the file) states are stored. */
int gbcp_restart_read(const char* path, gbcp_restart* r);

#ifdef __cplusplus
}
#endif

#endif /* CPMD_GB300_H */
