"""GPU checks of the energy functional and its hand-written adjoint (gbcp_energy).

* FP64 drop-in vs the FP64 oracle: energies, C2 (= CP force), dE/dV and
  forces to 1e-10 relative (max-norm);
* the adjoint vs central finite differences of the GPU energy itself
  (h = 1e-4 bohr for forces on 8 seeded atoms): 1e-6 relative;
* torch.autograd.Function: directional derivatives of E(c0, vext, tau);
* mixed precision vs FP64: |dE| <= 1e-6 Ha/atom, |dF| <= 1e-5 Ha/bohr
  (216-atom, 432-state, 144^3 cell and the small cells).
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def dev(x):
    import torch
    if x.dtype == np.complex128 and x.ndim == 2:
        return torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def setup(cl, two_species=True, vext_amp=0.05, seed=2):
    b = cl.basis
    if two_species:
        vps = np.stack([O.gaussian_vps(b.hg, b.tpiba2, b.omega),
                        O.gaussian_vps(b.hg, b.tpiba2, b.omega, amp=-2.5, width2=0.7)], axis=1)
        isp = (np.arange(len(cl.tau)) % 2).astype(np.int32)
    else:
        vps = O.gaussian_vps(b.hg, b.tpiba2, b.omega)[:, None]
        isp = np.zeros(len(cl.tau), dtype=np.int32)
    vext = None
    if vext_amp:
        rng = np.random.default_rng(seed)
        vext = np.zeros((b.kr[2], b.kr[1], b.kr[0]))
        vext[:b.nr[2], :b.nr[1], :b.nr[0]] = vext_amp * rng.standard_normal(b.nr[::-1])
    return vps, isp, vext


@pytest.fixture(scope="module")
def c0case():
    cl = make_cell("c0")
    vps, isp, vext = setup(cl)
    ref = O.energy(cl.c0, cl.f, cl.basis, cl.tau, vps, isp, vext)
    return cl, vps, isp, vext, ref


def ctx_for(basis, precision="fp64"):
    from cpmd_gb300 import Context
    return Context(basis, precision=precision)


@pytest.mark.parametrize("mode", ["host", "device"])
def test_energy_fp64_parity(gpu_lib, c0case, mode):
    cl, vps, isp, vext, ref = c0case
    terms_ref, c2_ref, dv_ref, f_ref, _ = ref
    ctx = ctx_for(cl.basis)
    if mode == "host":
        terms, c2, dv, fion = ctx.energy(cl.c0, cl.f, cl.tau, vps, isp, vext)
    else:
        terms, c2, dv, fion = ctx.energy(dev(cl.c0), dev(cl.f), dev(cl.tau), dev(np.ascontiguousarray(vps.T)), isp,
                                         dev(vext))
        c2 = np.asfortranarray(c2.cpu().numpy().T)
        dv = dv.cpu().numpy()
        fion = fion.cpu().numpy()
    for k in ("ekin", "eloc", "ehart", "exc", "eext", "etot"):
        assert abs(terms[k] - terms_ref[k]) <= TOL64 * max(abs(terms_ref[k]), 1.0), k
    assert rel(c2, c2_ref) < TOL64
    assert rel(dv, dv_ref) < TOL64
    assert rel(fion, f_ref) < TOL64


def test_energy_no_ions_no_vext(gpu_lib, c0case):
    cl = c0case[0]
    b = cl.basis
    ctx = ctx_for(b)
    terms, c2, dv, fion = ctx.energy(cl.c0, cl.f)
    zero = np.zeros((1, b.nhg))
    t_ref, c2_ref, dv_ref, _, _ = O.energy(cl.c0, cl.f, b, np.zeros((1, 3)), zero.T, np.zeros(1, int), None)
    assert fion is None
    assert abs(terms["eloc"]) == 0.0 and terms["eext"] == 0.0
    for k in ("ekin", "ehart", "exc", "etot"):
        assert abs(terms[k] - t_ref[k]) <= TOL64 * max(abs(t_ref[k]), 1.0), k
    assert rel(c2, c2_ref) < TOL64


def test_energy_fd_small(gpu_lib):
    """Forces, dE/dc* and dE/dV of the FP64 GPU adjoint vs FD of the GPU energy."""
    cl = make_small_cell(10.26, 24, 10.0, 6, seed=3)
    b = cl.basis
    vps, isp, vext = setup(cl)
    ctx = ctx_for(b)
    terms, c2, dv, fion = ctx.energy(cl.c0, cl.f, cl.tau, vps, isp, vext)
    E = lambda c=cl.c0, t=cl.tau, v=vext: ctx.energy(c, cl.f, t, vps, isp, v, grad=False)["etot"]
    h = 1e-4
    fd = np.zeros_like(fion)
    for a in range(len(cl.tau)):
        for d in range(3):
            tp = cl.tau.copy(); tp[a, d] += h
            tm = cl.tau.copy(); tm[a, d] -= h
            fd[a, d] = -(E(t=tp) - E(t=tm)) / (2 * h)
    assert np.abs(fd - fion).max() < 1e-6 * np.abs(fion).max()
    rng = np.random.default_rng(9)
    dc = (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape)) * 1e-2
    dc[0] = dc[0].real
    w = np.ones(b.ngw); w[0] = 0.5
    hc = 1e-3
    fdc = (E(c=np.asfortranarray(cl.c0 + hc * dc)) - E(c=np.asfortranarray(cl.c0 - hc * dc))) / (2 * hc)
    an = -4.0 * np.sum(w[:, None] * (np.conj(dc) * c2).real)
    assert abs(fdc - an) < 1e-6 * abs(an)
    dd = np.zeros_like(vext)
    dd[:b.nr[2], :b.nr[1], :b.nr[0]] = rng.standard_normal(b.nr[::-1])
    fdv = (E(v=vext + hc * dd) - E(v=vext - hc * dd)) / (2 * hc)
    an = float(np.sum(dd * dv))
    assert abs(fdv - an) < 1e-6 * abs(an)


def test_energy_autograd(gpu_lib):
    import torch
    from cpmd_gb300.autograd import energy_fn
    cl = make_small_cell(10.26, 24, 10.0, 6, seed=5)
    b = cl.basis
    vps, isp, vext = setup(cl)
    ctx = ctx_for(b)
    c0 = dev(cl.c0).requires_grad_(True)
    v = dev(vext).requires_grad_(True)
    tau = dev(cl.tau).requires_grad_(True)
    f = dev(cl.f)
    vpsd = dev(np.ascontiguousarray(vps.T))
    e = energy_fn(ctx, c0, v, tau, f, vpsd, isp)
    e.backward()
    rng = np.random.default_rng(1)
    dc = torch.from_numpy(np.ascontiguousarray(
        ((rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape)) * 1e-2).T)).cuda()
    dc[:, 0] = dc[:, 0].real.to(torch.complex128)
    dt = torch.from_numpy(rng.standard_normal(cl.tau.shape) * 1e-2).cuda()
    h = 1e-3
    with torch.no_grad():
        ep = energy_fn(ctx, c0 + h * dc, v, tau + h * dt, f, vpsd, isp).item()
        em = energy_fn(ctx, c0 - h * dc, v, tau - h * dt, f, vpsd, isp).item()
    an = (torch.sum((c0.grad.conj() * dc).real) + torch.sum(tau.grad * dt)).item()
    assert abs((ep - em) / (2 * h) - an) < 1e-6 * abs(an)
    assert torch.allclose(v.grad, torch.from_numpy(O.energy(cl.c0, cl.f, b, cl.tau, vps, isp, vext)[2]).cuda(),
                          rtol=0, atol=1e-10 * float(v.grad.abs().max()))


def test_energy_mixed_vs_fp64_small(gpu_lib, c0case):
    cl, vps, isp, vext, ref = c0case
    terms, c2, dv, fion = ctx_for(cl.basis, "mixed").energy(cl.c0, cl.f, cl.tau, vps, isp, vext)
    nat = len(cl.tau)
    assert abs(terms["etot"] - ref[0]["etot"]) / nat <= 1e-6
    assert np.abs(fion - ref[3]).max() <= 1e-5


@pytest.fixture(scope="module")
def c2cell():
    return make_cell("c2")


def test_energy_c2_mixed_gate_and_fd(gpu_lib, c2cell):
    """216 atoms, 432 states, 50 Ry, 144^3: mixed vs FP64 and FD forces on 8 seeded atoms."""
    cl = c2cell
    b = cl.basis
    vps, isp, _ = setup(cl, two_species=False, vext_amp=0.0)
    ctx64 = ctx_for(b)
    t64, c2_64, dv64, f64 = ctx64.energy(cl.c0, cl.f, cl.tau, vps, isp)
    t32, c2_32, dv32, f32 = ctx_for(b, "mixed").energy(cl.c0, cl.f, cl.tau, vps, isp)
    nat = len(cl.tau)
    assert abs(t32["etot"] - t64["etot"]) / nat <= 1e-6
    assert np.abs(f32 - f64).max() <= 1e-5
    rng = np.random.default_rng(216)
    atoms = rng.choice(nat, size=8, replace=False)
    h = 1e-4
    for a in atoms:
        for d in range(3):
            tp = cl.tau.copy(); tp[a, d] += h
            tm = cl.tau.copy(); tm[a, d] -= h
            ep = ctx64.energy(cl.c0, cl.f, tp, vps, isp, grad=False)["etot"]
            em = ctx64.energy(cl.c0, cl.f, tm, vps, isp, grad=False)["etot"]
            assert abs(-(ep - em) / (2 * h) - f64[a, d]) < 1e-6 * np.abs(f64).max()


# ------------------------------------------------------------------ PBE (gradient-corrected xc)
@pytest.mark.parametrize("mode", ["host", "device"])
def test_energy_pbe_fp64_parity(gpu_lib, c0case, mode):
    """GBCP_OPT_XC = PBE: energies, C2, dE/dV and forces vs the oracle's PBE route
    (grad rho and the divergence term by FFT) to 1e-10 relative."""
    cl, vps, isp, vext, _ = c0case
    terms_ref, c2_ref, dv_ref, f_ref, _ = O.energy(cl.c0, cl.f, cl.basis, cl.tau, vps, isp, vext, xc="pbe")
    ctx = ctx_for(cl.basis)
    ctx.set_option("xc", 1)
    if mode == "host":
        terms, c2, dv, fion = ctx.energy(cl.c0, cl.f, cl.tau, vps, isp, vext)
    else:
        terms, c2, dv, fion = ctx.energy(dev(cl.c0), dev(cl.f), dev(cl.tau), dev(np.ascontiguousarray(vps.T)), isp,
                                         dev(vext))
        c2 = np.asfortranarray(c2.cpu().numpy().T)
        dv = dv.cpu().numpy()
        fion = fion.cpu().numpy()
    for k in ("ekin", "eloc", "ehart", "exc", "eext", "etot"):
        assert abs(terms[k] - terms_ref[k]) <= TOL64 * max(abs(terms_ref[k]), 1.0), k
    assert rel(c2, c2_ref) < TOL64
    assert rel(dv, dv_ref) < TOL64
    assert rel(fion, f_ref) < TOL64
    # the functional differs from LDA by a gradient correction of the expected size
    ctx.set_option("xc", 0)
    lda = ctx.energy(cl.c0, cl.f, cl.tau, vps, isp, vext, grad=False)
    assert 1e-4 < abs(terms_ref["exc"] - lda["exc"]) < 0.2 * abs(lda["exc"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_energy_pbe_fd(gpu_lib, precision):
    """dE/dc* of the PBE energy (C2 from vpsi on V_eff with the divergence term) vs
    central differences of the GPU energy; mixed precision keeps |dE| <= 1e-6 Ha/atom."""
    cl = make_small_cell(10.26, 24, 10.0, 6, seed=5)
    b = cl.basis
    vps, isp, vext = setup(cl)
    ctx = ctx_for(b, precision)
    ctx.set_option("xc", 1)
    terms, c2, dv, fion = ctx.energy(cl.c0, cl.f, cl.tau, vps, isp, vext)
    E = lambda c: ctx.energy(c, cl.f, cl.tau, vps, isp, vext, grad=False)["etot"]  # noqa: E731
    rng = np.random.default_rng(11)
    dc = (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape)) * 1e-2
    dc[0] = dc[0].real
    w = np.ones(b.ngw)
    w[0] = 0.5
    hc = 1e-3
    fdc = (E(np.asfortranarray(cl.c0 + hc * dc)) - E(np.asfortranarray(cl.c0 - hc * dc))) / (2 * hc)
    an = -4.0 * np.sum(w[:, None] * (np.conj(dc) * c2).real)
    assert abs(fdc - an) < (1e-6 if precision == "fp64" else 1e-4) * abs(an)
    if precision == "mixed":
        ref = O.energy(cl.c0, cl.f, b, cl.tau, vps, isp, vext, grad=False, xc="pbe")
        assert abs(terms["etot"] - ref["etot"]) / len(cl.tau) < 1e-6
