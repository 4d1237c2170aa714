"""CPU checks of the FP64 oracle: G-vector list, FFT conventions, analytic
known-answer cases and the reference's own runtime invariants.

The reference has no test suite or golden vectors for this path; these KATs
and the invariants (charge consistency, rhoofr_utils.mod.F90:607-635;
orthonormality scond, csmat_utils.mod.F90:82-89) pin the oracle instead.
"""
import math

import numpy as np
import pytest

from cpmd_gb300 import cell
from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O


@pytest.mark.parametrize("alat,nr,ecut", [(10.26, 32, 20.0), (12.0, 36, 15.0), (9.0, 25, 12.0), (20.52, 120, 70.0)])
def test_gvectors_two_restatements_agree(alat, nr, ecut):
    b = cell.make_basis(alat, nr, ecut)
    m, hg, ngw = O.gvectors(alat, nr, ecut)
    assert ngw == b.ngw
    assert np.array_equal(m, b.mill.astype(np.int64))
    assert np.array_equal(hg, b.hg)
    # half sphere: G = 0 first, no G and -G both present
    assert tuple(m[0]) == (0, 0, 0)
    s = {tuple(x) for x in m[:ngw].tolist()}
    assert all(tuple(-np.array(x)) not in s for x in m[1:ngw].tolist())
    # sorted by |G|^2 and wavefunction sphere first
    assert np.all(np.diff(hg[:ngw]) >= 0)
    assert hg[ngw - 1] < ecut / b.tpiba2 <= hg[ngw:].min()


def test_gvector_counts_match_configs():
    # ngw of the benchmark cells (half sphere incl. G = 0)
    assert cell.make_basis(10.26, 32, 20.0).ngw == 824
    assert cell.make_basis(20.52, 120, 70.0).ngw == 42736


def test_leadim_is_odd():
    for n in (32, 33, 120, 144, 240):
        k = cell.leadim(n)
        assert k % 2 == 1 and k in (n, n + 1)


def test_fft_round_trip_and_convention():
    rng = np.random.default_rng(0)
    g = rng.standard_normal((6, 5, 8)) + 1j * rng.standard_normal((6, 5, 8))
    assert np.allclose(O.fwfftn(O.invfftn(g)), g, atol=1e-14)
    # single G: invfftn gives e^{+i G r}
    e = np.zeros((6, 5, 8), complex)
    e[0, 0, 1] = 1.0
    r = O.invfftn(e)
    x = np.arange(8)
    assert np.allclose(r[0, 0, :], np.exp(2j * np.pi * x / 8), atol=1e-14)


def _plane_wave_state(b, ig):
    c = np.zeros((b.ngw, 1), complex, order="F")
    c[ig, 0] = 1.0 if ig == 0 else 1.0 / math.sqrt(2.0)
    return c


def test_rhoofr_kat_constant_state():
    b = cell.make_basis(10.26, 32, 20.0)
    c = _plane_wave_state(b, 0)
    rho, ekin, csumg, csumr = O.rhoofr(c, np.array([2.0]), b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    n1, n2, n3 = b.nr
    assert np.allclose(rho[:n3, :n2, :n1], 2.0 / b.omega, rtol=1e-14)
    assert np.all(rho[n3:] == 0) and np.all(rho[:, n2:] == 0) and np.all(rho[:, :, n1:] == 0)
    assert ekin == 0.0
    assert abs(csumg - 2.0) < 1e-14 and abs(csumr - 2.0) < 1e-12


def test_rhoofr_kat_cosine_state():
    b = cell.make_basis(10.26, 32, 20.0)
    ig = 1  # (1,0,0)
    c = _plane_wave_state(b, ig)
    rho, ekin, csumg, csumr = O.rhoofr(c, np.array([2.0]), b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    n1, n2, n3 = b.nr
    x = np.arange(n1)
    gx, gy, gz = b.mill[ig]
    assert (gy, gz) == (0, 0)
    # psi(r) = 2 Re(c e^{iGr}) = sqrt(2) cos(2 pi gx x / n1)
    expect = 2.0 / b.omega * 2.0 * np.cos(2 * np.pi * gx * x / n1) ** 2
    assert np.allclose(rho[0, 0, :n1], expect, atol=1e-14)
    assert abs(ekin - 2.0 * b.tpiba2 * b.hg[ig] * 0.5) < 1e-13
    assert abs(csumr - csumg) < 1e-12


def test_rhoofr_pairs_equal_singles():
    cl = make_small_cell(10.26, 32, 20.0, 5, seed=3)
    b = cl.basis
    rho, *_ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    acc = 0
    for i in range(5):
        r1, *_ = O.rhoofr(cl.c0[:, i:i + 1].copy(order="F"), cl.f[i:i + 1], b.mill, b.nr, b.kr, b.omega, b.hg,
                          b.tpiba2, b.geq0)
        acc = acc + r1
    assert np.abs(acc - rho).max() < 1e-13 * np.abs(rho).max()


def test_charge_invariant_reference_check():
    cl = make_cell("c0")
    b = cl.basis
    rho, ekin, csumg, csumr = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    assert abs(csumr - csumg) <= 1e-6  # rhoofr_utils.mod.F90:625
    assert abs(csumg - 2.0 * cl.nstate) < 1e-10  # orthonormal states, f = 2


def test_vpsi_kat_constant_potential():
    cl = make_small_cell(10.26, 32, 20.0, 5, seed=4)
    b = cl.basis
    v = np.full(tuple(b.kr[::-1]), -0.37)
    c2 = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, v, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    kin = b.tpiba2 * b.hg[: b.ngw]
    expect = -(cl.f[None, :] / 2.0) * (kin[:, None] + 2 * (-0.37)) * cl.c0
    assert np.abs(c2 - expect).max() < 1e-14


def test_vpsi_is_gradient_of_potential_energy():
    """C2 = -f dE/dc* for E = E_kin/2... checked as linearity in V and the
    hermiticity <c_i|V|c_j> = <c_j|V|c_i> of the potential part."""
    cl = make_small_cell(10.26, 32, 20.0, 4, seed=5)
    b = cl.basis
    f = np.ones(4) * 2.0
    rng = np.random.default_rng(1)
    v1 = rng.standard_normal(tuple(b.kr[::-1]))
    v2 = rng.standard_normal(tuple(b.kr[::-1]))
    z = np.zeros_like(cl.c0)
    a = O.vpsi(cl.c0, z, f, v1, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    bb = O.vpsi(cl.c0, z, f, v2, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    ab = O.vpsi(cl.c0, z, f, v1 + v2, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    k = O.vpsi(cl.c0, z, f, 0 * v1, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    assert np.abs(a + bb - k - ab).max() < 1e-13
    # potential matrix M_ij = <c_i | (a - k)_j> in the Γ metric is symmetric
    p = -(a - k)
    M = 2 * (cl.c0.real.T @ p.real + cl.c0.imag.T @ p.imag) - np.outer(cl.c0[0].real, p[0].real)
    assert np.abs(M - M.T).max() < 1e-12


def test_rgs_orthonormalises_and_is_idempotent():
    cl = make_small_cell(10.26, 32, 20.0, 6, seed=6)
    b = cl.basis
    rng = np.random.default_rng(2)
    c = cl.c0 + 0.05 * (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    c[0] = c[0].real
    c = np.asfortranarray(c)
    o = O.rgs(c, b.geq0)
    assert O.scond(O.overlap(o, b.geq0)) < 1e-13
    o2 = O.rgs(o, b.geq0)
    assert np.abs(o2 - o).max() < 1e-13
    assert np.all(o[0].imag == 0.0)


def test_rgs_rejects_singular_overlap():
    cl = make_small_cell(10.26, 32, 20.0, 3, seed=6)
    c = cl.c0.copy(order="F")
    c[:, 2] = c[:, 1]
    with pytest.raises(np.linalg.LinAlgError):
        O.rgs(c, cl.basis.geq0)


def test_lowdin_symmetric_orthonormalisation():
    cl = make_small_cell(10.26, 32, 20.0, 6, seed=7)
    b = cl.basis
    rng = np.random.default_rng(3)
    c = np.asfortranarray(cl.c0 @ (np.eye(6) + 0.05 * rng.standard_normal((6, 6))))
    c[0] = c[0].real
    o, sc = O.lowdin(c, b.geq0)
    assert sc > 0.01
    assert O.scond(O.overlap(o, b.geq0)) < 1e-13
    # Loewdin is the orthonormal set closest to the input: C^T O symmetric
    m = 2 * (c.real.T @ o.real + c.imag.T @ o.imag) - np.outer(c[0].real, o[0].real)
    assert np.abs(m - m.T).max() < 1e-12


def _brute_fnl(c0, twnl, eigr, nghtol, geq0):
    ngw, n = c0.shape
    nat, ngh = eigr.shape[1], twnl.shape[1]
    out = np.zeros((nat, ngh, n))
    for ia in range(nat):
        for iv in range(ngh):
            scr = ((-1j) ** nghtol[iv]) * twnl[:, iv] * eigr[:, ia]
            w = np.full(ngw, 2.0)
            if geq0:
                w[0] = 1.0
            for i in range(n):
                out[ia, iv, i] = np.sum(w * (scr.real * c0[:, i].real + scr.imag * c0[:, i].imag))
    return out


def test_rnlsm1_and_fnonloc_against_loop_form():
    cl = make_small_cell(10.26, 32, 20.0, 3, seed=8, with_proj=True)
    b, p = cl.basis, cl.proj
    fnl = O.rnlsm1(cl.c0, p["twnl"], p["eigr"], p["nghtol"], b.geq0)
    assert np.abs(fnl - _brute_fnl(cl.c0, p["twnl"], p["eigr"], p["nghtol"], b.geq0)).max() < 1e-13
    f = np.array([2.0, 0.0, 1.0])
    c2 = O.fnonloc(np.zeros_like(cl.c0), f, fnl, p["twnl"], p["eigr"], p["nghtol"], p["wsg"])
    ref = np.zeros_like(cl.c0)
    for iv in range(8):
        for ia in range(cl.tau.shape[0]):
            for i in range(3):
                ffi = 1.0 if f[i] < 1e-5 else f[i]
                ref[:, i] += p["twnl"][:, iv] * ((-1j) ** p["nghtol"][iv]) * (-ffi * p["wsg"][iv]) * \
                    p["eigr"][:, ia] * fnl[ia, iv, i]
    assert np.abs(c2 - ref).max() < 1e-13


def test_golden_fixture_regression():
    """The committed fixture (tests/golden/make_golden.py) still matches the oracle."""
    from pathlib import Path
    fx = np.load(Path(__file__).parent / "golden" / "cell_small.npz")
    b = cell.make_basis(float(fx["alat"]), int(fx["nr"]), float(fx["ecut"]))
    assert b.ngw == int(fx["ngw"])
    c0 = np.asfortranarray(fx["c0"])
    f = fx["f"]
    rho, ekin, csumg, csumr = O.rhoofr(c0, f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    assert np.abs(rho - fx["rho"]).max() <= 1e-12 * np.abs(fx["rho"]).max()
    assert abs(ekin - float(fx["ekin"])) < 1e-10
    c2 = O.vpsi(c0, np.zeros_like(c0), f, fx["vpot"], b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    assert np.abs(c2 - fx["c2"]).max() <= 1e-12 * np.abs(fx["c2"]).max()
    o = O.rgs(np.asfortranarray(fx["c_pert"]), b.geq0)
    assert np.abs(o - fx["c_gs"]).max() < 1e-11


def test_factored_projector_forms_match_loop_forms():
    """The GEMM-ordered rnlsm1 / fnonloc used at the 512-atom size against the
    per-projector loop forms (same sums, reordered)."""
    from cpmd_gb300.synth import make_small_cell
    cl = make_small_cell(10.26, 32, 20.0, 9, seed=61, nat_rep=1, with_proj=True)
    p = cl.proj
    nghtol = np.array([0, 1, 2, 3, 0, 1, 2, 3], dtype=np.int32)
    a = O.rnlsm1(cl.c0, p["twnl"], p["eigr"], nghtol, cl.basis.geq0)
    b = O.rnlsm1_factored(cl.c0, p["twnl"], p["eigr"], nghtol, cl.basis.geq0)
    assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()
    f = cl.f.copy()
    f[2] = 0.0
    rng = np.random.default_rng(5)
    c2 = np.asfortranarray(rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    x = O.fnonloc(c2, f, a, p["twnl"], p["eigr"], nghtol, p["wsg"])
    y = O.fnonloc_factored(c2, f, a, p["twnl"], p["eigr"], nghtol, p["wsg"])
    assert np.abs(x - y).max() <= 1e-13 * np.abs(x - c2).max()
