"""GPU parity of the CUDA hot path against the FP64 oracle, through the C ABI.

Tolerances: the FP64 drop-in must match the oracle to 1e-10 relative
(max-norm of the difference over max-norm of the oracle) on rho, H psi (c2)
and the orthonormalised coefficients.  The mixed mode (FP32 FFT and V*psi,
FP64 accumulation) is checked to 2e-5 relative on rho and c2 and to 1e-6
Ha/atom on the energy E_kin + int V rho.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 2e-5


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def dev(x):
    import torch
    if x.dtype == np.complex128 and x.ndim == 2:
        return torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host_wfn(t):
    return np.asfortranarray(t.cpu().numpy().T)


@pytest.fixture(scope="module")
def c0cell():
    return make_cell("c0")


@pytest.fixture(scope="module")
def c0ref(c0cell):
    b = c0cell.basis
    rho, ekin, csumg, csumr = O.rhoofr(c0cell.c0, c0cell.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    c2 = O.vpsi(c0cell.c0, np.zeros_like(c0cell.c0), c0cell.f, c0cell.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    return dict(rho=rho, ekin=ekin, csumg=csumg, csumr=csumr, c2=c2)


def ctx_for(basis, precision="fp64", batch=0):
    from cpmd_gb300 import Context
    return Context(basis, precision=precision, batch=batch)


# ------------------------------------------------------------------ rhoofr
@pytest.mark.parametrize("mode", ["host", "device"])
def test_rhoofr_fp64_parity(gpu_lib, c0cell, c0ref, mode):
    b = c0cell.basis
    ctx = ctx_for(b)
    if mode == "host":
        rho, ekin, csumg, csumr = ctx.rhoofr(c0cell.c0, c0cell.f)
    else:
        rho_t, ekin, csumg, csumr = ctx.rhoofr(dev(c0cell.c0), dev(c0cell.f))
        rho = rho_t.cpu().numpy()
    assert rel(rho, c0ref["rho"]) < TOL64
    assert abs(ekin - c0ref["ekin"]) < TOL64 * abs(c0ref["ekin"])
    assert abs(csumg - c0ref["csumg"]) < TOL64 * abs(c0ref["csumg"])
    assert abs(csumr - c0ref["csumr"]) < TOL64 * abs(c0ref["csumr"])
    assert abs(csumr - csumg) <= 1e-6  # rhoofr_utils.mod.F90:625
    n1, n2, n3 = b.nr
    assert np.all(rho[n3:] == 0) and np.all(rho[:, n2:] == 0) and np.all(rho[:, :, n1:] == 0)


@pytest.mark.parametrize("nstate,batch", [(1, 0), (5, 0), (7, 2), (16, 3)])
def test_rhoofr_odd_states_and_batches(gpu_lib, nstate, batch):
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=11 + nstate)
    b = cl.basis
    f = cl.f.copy()
    if nstate > 2:
        f[1] = 0.0  # a pair with one empty state still counts the other
    ref = O.rhoofr(cl.c0, f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    ctx = ctx_for(b, batch=batch)
    rho, ekin, csumg, csumr = ctx.rhoofr(cl.c0, f)
    assert rel(rho, ref[0]) < TOL64
    assert abs(ekin - ref[1]) < TOL64 * abs(ref[1])


def test_rhoofr_leading_dimension(gpu_lib):
    cl = make_small_cell(10.26, 32, 20.0, 4, seed=21)
    b = cl.basis
    big = np.zeros((b.ngw + 9, 4), complex, order="F")
    big[: b.ngw] = cl.c0
    ctx = ctx_for(b)
    rho1, *_ = ctx.rhoofr(big[: b.ngw], cl.f)
    rho2, *_ = ctx.rhoofr(cl.c0, cl.f)
    assert np.array_equal(rho1, rho2)


@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("mixed", TOL32)])
def test_rhoofr_pair_chunks_deterministic(gpu_lib, c0cell, c0ref, precision, tol):
    """The density x-stage splits a launch's pairs into chunks whose partial tiles
    the last CTA of each tile adds in chunk order: every chunk count matches the
    oracle, and repeated calls are bit-identical."""
    b = c0cell.basis
    for chunks in (1, 3, 8, 0):
        ctx = ctx_for(b, precision=precision)
        ctx.set_option("xchunks", chunks)
        rho1, *_ = ctx.rhoofr(c0cell.c0, c0cell.f)
        rho2, *_ = ctx.rhoofr(c0cell.c0, c0cell.f)
        assert np.array_equal(rho1, rho2), chunks
        assert rel(rho1, c0ref["rho"]) < tol, chunks


def test_rhoofr_zero_states(gpu_lib, c0cell):
    ctx = ctx_for(c0cell.basis)
    rho, ekin, csumg, csumr = ctx.rhoofr(np.zeros((c0cell.basis.ngw, 0), complex, order="F"), np.zeros(0))
    assert np.all(rho == 0) and ekin == 0 and csumr == 0


# ------------------------------------------------------------------ vpsi
@pytest.mark.parametrize("mode", ["host", "device"])
def test_vpsi_fp64_parity(gpu_lib, c0cell, c0ref, mode):
    ctx = ctx_for(c0cell.basis)
    if mode == "host":
        c2 = np.zeros_like(c0cell.c0)
        ctx.vpsi(c0cell.c0, c2, c0cell.f, c0cell.vpot)
    else:
        c2t = dev(np.zeros_like(c0cell.c0))
        ctx.vpsi(dev(c0cell.c0), c2t, dev(c0cell.f), dev(c0cell.vpot))
        c2 = host_wfn(c2t)
    assert rel(c2, c0ref["c2"]) < TOL64


@pytest.mark.parametrize("nstate", [1, 3, 6])
def test_vpsi_accumulates_and_odd_states(gpu_lib, nstate):
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=30 + nstate)
    b = cl.basis
    f = cl.f.copy()
    f[-1] = 0.0  # vpsi counts an empty state with fi = 1 (vpsi_utils.mod.F90:627-632)
    rng = np.random.default_rng(5)
    c2in = np.asfortranarray(rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    ref = O.vpsi(cl.c0, c2in, f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    ctx = ctx_for(b, batch=2)
    c2 = c2in.copy(order="F")
    ctx.vpsi(cl.c0, c2, f, cl.vpot)
    assert rel(c2, ref) < TOL64


@pytest.mark.parametrize("nr,ecut,alat", [(20, 8.0, 10.26), (24, 10.0, 10.26), (36, 20.0, 10.26), (40, 25.0, 10.26),
                                          (48, 30.0, 10.26), (60, 40.0, 10.26), (64, 40.0, 10.26),
                                          (72, 50.0, 10.26), (80, 50.0, 10.26), (96, 60.0, 10.26),
                                          (144, 50.0, 30.78), (240, 70.0, 41.04)])
@pytest.mark.parametrize("precision,plane", [("fp64", 0), ("mixed", 0), ("mixed", 3)])
def test_band_loop_all_mesh_plans(gpu_lib, nr, ecut, alat, precision, plane):
    """Four-step plans (32..240) and the run-time Stockham plan (20, 24) give the oracle's rho and c2;
    in FP32 both with the three-stage kernels and with the plane-fused y/x stages (where they apply)."""
    cl = make_small_cell(alat, nr, ecut, 5 if nr < 144 else 3, seed=nr)
    b = cl.basis
    rho_r, *_ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    c2_r = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    ctx = ctx_for(b, precision)
    ctx.set_option("plane", plane)
    rho, *_ = ctx.rhoofr(cl.c0, cl.f)
    c2 = np.zeros_like(cl.c0)
    ctx.vpsi(cl.c0, c2, cl.f, cl.vpot)
    tol = TOL64 if precision == "fp64" else TOL32
    assert rel(rho, rho_r) < tol
    assert rel(c2, c2_r) < tol


@pytest.mark.parametrize("nr,ecut", [(40, 60.0), (64, 150.0), (80, 240.0)])
@pytest.mark.parametrize("precision,plane", [("fp64", 0), ("mixed", 0), ("mixed", 3)])
def test_radix8_sphere_beyond_quarter_mesh(gpu_lib, nr, ecut, precision, plane):
    """Radix-8 four-step meshes (40 = 8 x 5, 64 = 8 x 8, 80 = 8 x 10) under a
    wavefunction sphere that reaches |G| >= N/4 along x and y (a density cutoff of
    1.2 times the wavefunction cutoff): the inverse step A keeps all eight inputs
    there (the pruned form, which skips positions n1 = 2..5, applies only while the
    sphere lies within [-N/4, N/4)), in the three-stage and plane-fused kernels;
    rho and c2 against the oracle."""
    from cpmd_gb300.cell import make_basis
    from cpmd_gb300.synth import atoms, random_states, vloc_grid
    rng = np.random.default_rng(nr + 11)
    alat = 10.26
    tau, _ = atoms(alat, 1, 0.0, rng)
    b = make_basis(alat, nr, ecut, dual=1.2)
    assert int(np.abs(b.mill[: b.ngw, :2]).max()) >= nr // 4
    c0 = random_states(b, 3, rng)
    vpot = vloc_grid(b, tau)
    f = np.full(3, 2.0)
    rho_r, *_ = O.rhoofr(c0, f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    c2_r = O.vpsi(c0, np.zeros_like(c0), f, vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    ctx = ctx_for(b, precision)
    ctx.set_option("plane", plane)
    rho, *_ = ctx.rhoofr(c0, f)
    c2 = np.zeros_like(c0)
    ctx.vpsi(c0, c2, f, vpot)
    tol = TOL64 if precision == "fp64" else TOL32
    assert rel(rho, rho_r) < tol
    assert rel(c2, c2_r) < tol


@pytest.mark.parametrize("nr,ecut,alat,nstate", [(32, 20.0, 10.26, 5), (72, 50.0, 10.26, 4), (120, 70.0, 20.52, 5),
                                                 (240, 70.0, 41.04, 3)])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("zmirror", [0, 1])
def test_zstage_gather_mirror_pairs(gpu_lib, nr, ecut, alat, nstate, precision, zmirror):
    """The Z-stage gather over column/mirror pairs (GBCP_OPT_ZMIRROR = 1, the default
    from 48 column blocks up) and the plain gather (0) give the oracle's rho, E_kin,
    norm and c2 on small and large meshes, an odd state count included (a single
    state in the last pair)."""
    cl = make_small_cell(alat, nr, ecut, nstate, seed=nr + 7)
    b = cl.basis
    rho_r, ek_r, cg_r, _ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    c2_r = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    ctx = ctx_for(b, precision)
    ctx.set_option("zmirror", zmirror)
    rho, ek, cg, _ = ctx.rhoofr(cl.c0, cl.f)
    c2 = np.zeros_like(cl.c0)
    ctx.vpsi(cl.c0, c2, cl.f, cl.vpot)
    tol = TOL64 if precision == "fp64" else TOL32
    assert rel(rho, rho_r) < tol
    assert rel(c2, c2_r) < tol
    assert abs(ek - ek_r) <= tol * abs(ek_r)
    assert abs(cg - cg_r) <= tol * abs(cg_r)


# ------------------------------------------------------------------ ortho
def perturbed(cl, scale=0.05, seed=3):
    rng = np.random.default_rng(seed)
    c = cl.c0 + scale * (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    c[0] = c[0].real
    return np.asfortranarray(c)


@pytest.mark.parametrize("nstate", [16, 37, 130])
def test_ortho_gs_parity(gpu_lib, nstate):
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=40)
    b = cl.basis
    c = perturbed(cl)
    ref = O.rgs(c, b.geq0)
    ctx = ctx_for(b)
    out = c.copy(order="F")
    sc = ctx.ortho(out, "gs")
    assert rel(out, ref) < TOL64
    assert abs(sc - O.scond(O.overlap(c, b.geq0))) < 1e-12
    assert O.scond(O.overlap(out, b.geq0)) < 1e-12
    assert np.all(out[0].imag == 0.0)


@pytest.mark.parametrize("nstate", [16, 70])
@pytest.mark.parametrize("gemm", [0, 1])
def test_ortho_lowdin_parity(gpu_lib, nstate, gemm):
    """Both GEMM engines (FP64 SIMT; tcgen05 split GEMMs for the overlap, the
    Newton-Schulz products and C S^-1/2) give the oracle's Loewdin states."""
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=41)
    b = cl.basis
    c = perturbed(cl, 0.03)
    ref, sc_ref = O.lowdin(c, b.geq0)
    ctx = ctx_for(b)
    ctx.set_option("gemm", gemm)
    out = dev(c)
    sc = ctx.ortho(out, "lowdin")
    out = host_wfn(out)
    assert rel(out, ref) < TOL64
    assert abs(sc - sc_ref) < 1e-12


def test_ortho_not_spd_is_reported(gpu_lib):
    from cpmd_gb300 import GbcpError
    cl = make_small_cell(10.26, 32, 20.0, 4, seed=42)
    c = cl.c0.copy(order="F")
    c[:, 3] = c[:, 2]
    ctx = ctx_for(cl.basis)
    with pytest.raises(GbcpError) as e:
        ctx.ortho(c, "gs")
    assert e.value.code == 2
    # the context stays usable
    ctx.ortho(cl.c0.copy(order="F"), "gs")


def test_ovlap_matches_oracle(gpu_lib):
    cl = make_small_cell(10.26, 32, 20.0, 20, seed=43)
    c = perturbed(cl, 0.1)
    ctx = ctx_for(cl.basis)
    s = ctx.ovlap(c)
    assert rel(s, O.overlap(c, cl.basis.geq0)) < 1e-13


# ------------------------------------------------------------------ invfftn / fwfftn
@pytest.mark.parametrize("nr", [20, 32, 36])
def test_dense_fft_parity(gpu_lib, nr):
    from cpmd_gb300.cell import make_basis
    b = make_basis(10.26, nr, 8.0)
    k1, k2, _ = b.kr
    rng = np.random.default_rng(nr)
    g = np.zeros((nr, k2, k1), complex)
    g[:, :nr, :nr] = rng.standard_normal((nr, nr, nr)) + 1j * rng.standard_normal((nr, nr, nr))
    ctx = ctx_for(b)
    a = g.copy()
    ctx.invfftn(a)
    assert rel(a[:, :nr, :nr], O.invfftn(g[:, :nr, :nr])) < 1e-12
    assert np.all(a[:, nr:, :] == g[:, nr:, :])  # padding untouched
    ctx.fwfftn(a)
    assert rel(a[:, :nr, :nr], g[:, :nr, :nr]) < 1e-12


# ------------------------------------------------------------------ projectors
def test_rnlsm1_fnonloc_parity(gpu_lib):
    cl = make_small_cell(10.26, 32, 20.0, 9, seed=50, with_proj=True)
    b, p = cl.basis, cl.proj
    f = cl.f.copy()
    f[4] = 0.0
    fnl_ref = O.rnlsm1(cl.c0, p["twnl"], p["eigr"], p["nghtol"], b.geq0)
    ctx = ctx_for(b)
    fnl = ctx.rnlsm(cl.c0, p["twnl"], p["eigr"], p["nghtol"])      # (n, ngh, nat)
    assert rel(np.transpose(fnl, (2, 1, 0)), fnl_ref) < TOL64
    c2in = perturbed(cl, 1.0, seed=9)
    ref = O.fnonloc(c2in, f, fnl_ref, p["twnl"], p["eigr"], p["nghtol"], p["wsg"])
    c2 = c2in.copy(order="F")
    ctx.fnonloc(c2, f, np.ascontiguousarray(np.transpose(fnl_ref, (2, 1, 0))), p["twnl"], p["eigr"], p["nghtol"],
                p["wsg"])
    assert rel(c2, ref) < TOL64


# ------------------------------------------------------------------ mixed precision
def test_mixed_precision_error_bounds(gpu_lib, c0cell, c0ref):
    b = c0cell.basis
    ctx = ctx_for(b, "mixed")
    rho, ekin, csumg, csumr = ctx.rhoofr(c0cell.c0, c0cell.f)
    assert rel(rho, c0ref["rho"]) < TOL32
    c2 = np.zeros_like(c0cell.c0)
    ctx.vpsi(c0cell.c0, c2, c0cell.f, c0cell.vpot)
    assert rel(c2, c0ref["c2"]) < TOL32
    n1, n2, n3 = b.nr
    dv = b.omega / (n1 * n2 * n3)
    e64 = c0ref["ekin"] + dv * float((c0ref["rho"] * c0cell.vpot).sum())
    e32 = ekin + dv * float((rho * c0cell.vpot).sum())
    assert abs(e32 - e64) / c0cell.tau.shape[0] < 1e-6


# ------------------------------------------------------------------ full-size properties (config 1)
def _gamma_dot(a, b):
    return 2.0 * float((a.real * b.real + a.imag * b.imag).sum()) - float((a[0].real * b[0].real).sum())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_full_size_rhoofr_vpsi_consistency(gpu_lib, precision, tol):
    """sum_i <c_i|C2_i> = -(E_kin + int V rho): ties vpsi to rhoofr at 120^3, 128 states."""
    import torch
    cl = make_cell("c1")
    b = cl.basis
    ctx = ctx_for(b, precision, batch=16)
    c0 = dev(cl.c0)
    f = dev(cl.f)
    v = dev(cl.vpot)
    rho, ekin, csumg, csumr = ctx.rhoofr(c0, f)
    # the reference aborts above 1e-6 absolute (rhoofr_utils.mod.F90:625); the
    # FP32 FFT of the mixed mode holds the charge to 1e-7 relative instead
    assert abs(csumr - csumg) <= (1e-6 if precision == "fp64" else 1e-7 * csumg)
    # the mixed mode sums the norm of the FP32-rounded coefficients (the ones its band loop transforms)
    assert abs(csumg - 2.0 * cl.nstate) < (1e-8 if precision == "fp64" else 1e-7 * csumg)
    c2 = torch.zeros_like(c0)
    ctx.vpsi(c0, c2, f, v)
    n1, n2, n3 = b.nr
    epot = b.omega / (n1 * n2 * n3) * float((rho * v).sum())
    lhs = _gamma_dot(cl.c0, host_wfn(c2))
    assert abs(lhs + ekin + epot) < tol * abs(ekin + epot)


def test_full_size_ortho_gs(gpu_lib):
    import torch
    cl = make_cell("c1")
    b = cl.basis
    ctx = ctx_for(b)
    c = dev(perturbed(cl, 0.02))
    ctx.ortho(c, "gs")
    s = ctx.ovlap(c)
    assert float((s - torch.eye(cl.nstate, dtype=torch.float64, device=s.device)).abs().max()) < 1e-12


def test_profile_timeline_host_staging(gpu_lib, c0cell):
    """gbcp_profile_timeline: the staged copies of a host-memory call appear on their
    lanes with the kernels, each record ends after it starts and after the enable."""
    ctx = ctx_for(c0cell.basis, precision="mixed")
    ctx.profile(True)
    ctx.rhoofr(c0cell.c0, c0cell.f)
    tl = ctx.profile_timeline()
    names = {r[0] for r in tl}
    assert "h2d_states" in names and "d2h_rho" in names and "k_zinv" in names
    assert {r[1] for r in tl} >= {0, 1, 2}
    assert all(0.0 <= r[2] <= r[3] for r in tl)
    ups = [r for r in tl if r[0] == "h2d_states"]
    zinv = [r for r in tl if r[0] == "k_zinv"]
    assert min(z[2] for z in zinv) >= min(u[3] for u in ups) - 1e-3  # the first Z stage waits for its states
    ctx.profile(False)
