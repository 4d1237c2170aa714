"""Entry points a CPMD caller needs around the band loop.

* gbcp_ovlap2: the reference's general overlap <c1|c2> (ovlap_utils.mod.F90:
  157-166, dgemm + dger), against the oracle's cross overlap at 1e-10 on both
  GEMM engines, with leading dimensions above ngw, host and device memory;
* gbcp_vofrho: rho -> V_eff, energies and local forces (vofrhoa/vofrhob),
  against the oracle's functional at 1e-10 (LDA and PBE), and the reference's
  order rhoofr -> vofrho -> vpsi reproducing the CP force of gbcp_energy.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def padded(c, ld):
    out = np.full((ld, c.shape[1]), 5.0 + 5.0j, dtype=np.complex128, order="F")
    out[: c.shape[0]] = c
    return out


@pytest.mark.parametrize("mode", ["host", "device"])
@pytest.mark.parametrize("precision,gemm", [("fp64", 0), ("fp64", 1), ("mixed", None)])
@pytest.mark.parametrize("nstate", [13, 130])
def test_ovlap2_matches_oracle(gpu_lib, mode, precision, gemm, nstate):
    import torch
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=80 + nstate)
    b = cl.basis
    rng = np.random.default_rng(81)
    c2 = cl.c0 + 0.1 * (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    c2[0] = c2[0].real
    ref = O.cross_overlap(cl.c0, c2, b.geq0)                       # ref[i, j] = <c1_i|c2_j>
    ctx = Context(b, precision)
    if gemm is not None:
        ctx.set_option("gemm", gemm)
    a1, a2 = padded(cl.c0, b.ngw + 3), padded(np.asfortranarray(c2), b.ngw + 7)
    if mode == "host":
        amat = ctx.ovlap2(a1[: b.ngw], a2[: b.ngw])
    else:
        # device: (nstate, ld) rows with the padding rows present
        d1 = torch.from_numpy(np.ascontiguousarray(a1.T)).cuda()
        d2 = torch.from_numpy(np.ascontiguousarray(a2.T)).cuda()
        amat = ctx.ovlap2(d1, d2).cpu().numpy()
    assert rel(amat.T, ref) < TOL                                  # amat[j, i] = a(i, j)


@pytest.fixture(scope="module")
def vcell():
    cl = make_cell("c0")
    b = cl.basis
    vps = np.stack([O.gaussian_vps(b.hg, b.tpiba2, b.omega),
                    O.gaussian_vps(b.hg, b.tpiba2, b.omega, amp=-2.5, width2=0.7)], axis=1)
    isp = (np.arange(len(cl.tau)) % 2).astype(np.int32)
    rng = np.random.default_rng(3)
    vext = np.zeros((b.kr[2], b.kr[1], b.kr[0]))
    vext[:b.nr[2], :b.nr[1], :b.nr[0]] = 0.05 * rng.standard_normal(b.nr[::-1])
    return cl, vps, isp, vext


@pytest.mark.parametrize("xc", ["lda", "pbe"])
@pytest.mark.parametrize("mode", ["host", "device"])
def test_vofrho_matches_oracle(gpu_lib, vcell, xc, mode):
    import torch
    from cpmd_gb300 import Context
    cl, vps, isp, vext = vcell
    b = cl.basis
    terms, c2r, dvr, fr, veffr = O.energy(cl.c0, cl.f, b, cl.tau, vps, isp, vext, xc=xc)
    rho = dvr * (float(np.prod(b.nr)) / b.omega)                  # dE/dV = rho Omega / N
    ctx = Context(b, "fp64")
    ctx.set_option("xc", 1 if xc == "pbe" else 0)
    if mode == "host":
        veff, e, fion = ctx.vofrho(rho, cl.tau, vps, isp, vext)
    else:
        d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()  # noqa: E731
        veff, e, fion = ctx.vofrho(d(rho), d(cl.tau), d(np.ascontiguousarray(vps.T)), isp, d(vext))
        veff, fion = veff.cpu().numpy(), fion.cpu().numpy()
    n1, n2, n3 = b.nr
    assert rel(veff[:n3, :n2, :n1], veffr) < TOL
    for k in ("eloc", "ehart", "exc", "eext"):
        assert abs(e[k] - terms[k]) <= TOL * max(abs(terms[k]), 1.0), k
    assert rel(fion, fr) < TOL
    # the reference's order: rhoofr -> vofrho -> vpsi gives the CP force of the functional
    c2 = np.zeros_like(cl.c0)
    ctx.vpsi(cl.c0, c2, cl.f, np.ascontiguousarray(veff))
    assert rel(c2, c2r) < TOL


def test_vofrho_without_atoms(gpu_lib, vcell):
    from cpmd_gb300 import Context
    cl, _, _, vext = vcell
    b = cl.basis
    terms, _, dvr, _, veffr = O.energy(cl.c0, cl.f, b, np.zeros((0, 3)), np.zeros((b.nhg, 1)),
                                       np.zeros(0, np.int32), vext)
    rho = dvr * (float(np.prod(b.nr)) / b.omega)
    ctx = Context(b, "fp64")
    veff, e, fion = ctx.vofrho(rho, vext=vext)
    n1, n2, n3 = b.nr
    assert fion is None
    assert rel(veff[:n3, :n2, :n1], veffr) < TOL
    assert abs(e["eloc"]) < 1e-12 and abs(e["ehart"] - terms["ehart"]) <= TOL * abs(terms["ehart"])
