"""Projector results in the reference's global fnl / dfnl arrays.

CPMD keeps one fnl(imagp, ions1%nat, maxsys%nhxs, nstate) for all species;
rnlsm1 writes the block of species is at fnl(1, isa0+1, iv, i) with leading
dimension ions1%nat*maxsys%nhxs (rnlsm1_utils.mod.F90:156-165) and fnonloc
reads it back the same way (fnonloc_utils.mod.F90:322-324).  Here two species
with different projector counts (4 and 8, nhxs = 10 > both) are written into
one global array through the C ABI (atom offset + leading dimensions), checked
against the oracle per species at 1e-10, with every entry outside the two
blocks left untouched; fnonloc, rnlsm2 and rnlfor read the same global arrays.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10
SENTINEL = 777.0


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _species(basis, rng):
    """(nat, ngh, nghtol, twnl, eigr, wsg) of two species of a 5-atom cell."""
    G = basis.gvec_bohr(basis.ngw)
    gn = np.sqrt((G * G).sum(axis=1))
    out = []
    for nat, sig, nghtol in ((3, (0.9,), np.array([0, 1, 1, 1], np.int32)),
                             (2, (0.7, 1.3), np.array([0, 1, 1, 1, 0, 1, 1, 1], np.int32))):
        cols = []
        for sg in sig:
            rad = np.exp(-0.5 * (gn * sg) ** 2)
            cols.append(rad / np.sqrt(4 * np.pi))
            for ax in range(3):
                cols.append(rad * np.sqrt(3 / (4 * np.pi)) * G[:, ax] * sg)
        twnl = np.asfortranarray(np.stack(cols, axis=1))
        tau = rng.uniform(0.0, 10.26, size=(nat, 3))
        eigr = np.asfortranarray(np.exp(-1j * (G @ tau.T)))
        wsg = rng.uniform(0.5, 1.5, size=len(nghtol))
        out.append((nat, len(nghtol), nghtol, twnl, eigr, wsg))
    return out


@pytest.mark.parametrize("mode", ["device", "host"])
@pytest.mark.parametrize("precision,gemm,tol", [("fp64", None, TOL), ("mixed", 0, TOL), ("mixed", None, 1e-4)])
def test_two_species_in_one_global_fnl(gpu_lib, mode, precision, gemm, tol):
    """(mixed, tensor cores: an index error would show as O(1); the split GEMM's own
    accuracy is tested elsewhere, so its tolerance here is loose)"""
    import torch
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, 7, seed=71)
    b = cl.basis
    n = cl.nstate
    rng = np.random.default_rng(72)
    sp = _species(b, rng)
    NAT, NHXS = 5, 10
    ctx = Context(b, precision)
    if gemm is not None:
        ctx.set_option("gemm", gemm)
    dev = mode == "device"
    T = (lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()) if dev else (lambda x: x)
    Tw = (lambda x: torch.from_numpy(np.ascontiguousarray(x.T)).cuda()) if dev else (lambda x: x)
    fnl_g = T(np.full((n, NHXS, NAT), SENTINEL))            # Fortran fnl(NAT, NHXS, n)
    dfnl_g = T(np.full((n, 3, NHXS, NAT), SENTINEL))        # Fortran dfnl(NAT, NHXS, 3, n)
    c0 = Tw(cl.c0)
    refs = []
    isa0 = 0
    for nat, ngh, nghtol, twnl, eigr, wsg in sp:
        ctx.rnlsm(c0, Tw(twnl), Tw(eigr), nghtol, fnl_g, isa0=isa0)
        ctx.rnlsm2(c0, Tw(twnl), Tw(eigr), nghtol, dfnl_g, isa0=isa0)
        refs.append((isa0, O.rnlsm1(cl.c0, twnl, eigr, nghtol, b.geq0),
                     O.rnlsm2(cl.c0, twnl, eigr, nghtol, b.mill, b.tpiba, b.geq0)))
        isa0 += nat
    fg = fnl_g.cpu().numpy() if dev else fnl_g
    dg = dfnl_g.cpu().numpy() if dev else dfnl_g
    seen = np.zeros_like(fg, dtype=bool)
    dseen = np.zeros_like(dg, dtype=bool)
    for (a0, fref, dref), (nat, ngh, *_rest) in zip(refs, sp):
        assert rel(np.transpose(fg[:, :ngh, a0:a0 + nat], (2, 1, 0)), fref) < tol
        assert rel(np.transpose(dg[:, :, :ngh, a0:a0 + nat], (3, 2, 1, 0)), dref) < tol
        seen[:, :ngh, a0:a0 + nat] = True
        dseen[:, :, :ngh, a0:a0 + nat] = True
    assert np.all(fg[~seen] == SENTINEL) and np.all(dg[~dseen] == SENTINEL)
    # fnonloc and rnlfor read the blocks from the same global arrays
    f = cl.f.copy()
    f[2] = 0.0
    c2in = np.asfortranarray((rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape)) * 0.1)
    ref = c2in
    c2 = Tw(c2in) if dev else c2in.copy(order="F")
    fion_ref = []
    for (a0, fref, dref), (nat, ngh, nghtol, twnl, eigr, wsg) in zip(refs, sp):
        ref = O.fnonloc(ref, f, fref, twnl, eigr, nghtol, wsg)
        ctx.fnonloc(c2, T(f), fnl_g, Tw(twnl), Tw(eigr), nghtol, T(wsg), isa0=a0)
        fion = T(np.zeros((nat, 3)))
        ctx.rnlfor(T(f), fnl_g, dfnl_g, T(wsg), fion, nat=nat, ngh=ngh, isa0=a0)
        fion = fion.cpu().numpy() if dev else fion
        fion_ref.append((fion, O.rnlfor(f, fref, dref, wsg)))
    got = np.asfortranarray(c2.cpu().numpy().T) if dev else c2
    assert rel(got - c2in, ref - c2in) < tol
    for fion, fr in fion_ref:
        assert rel(fion, fr) < tol


def test_fnl_leading_dimension_below_block_is_rejected(gpu_lib):
    import ctypes as C
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, 4, seed=73, with_proj=True)
    b, p = cl.basis, cl.proj
    ctx = Context(b, "fp64")
    fnl = np.zeros(4 * 8 * 8)
    nt = np.ascontiguousarray(p["nghtol"], dtype=np.int32)
    rc = ctx.lib.gbcp_rnlsm1(ctx.h, C.c_void_p(cl.c0.ctypes.data), b.ngw, 4, 8, 8, C.c_void_p(nt.ctypes.data),
                             C.c_void_p(p["twnl"].ctypes.data), C.c_void_p(p["eigr"].ctypes.data),
                             C.c_void_p(fnl.ctypes.data), 7, 8, 0)   # ld_atoms 7 < nat 8
    assert rc == 1
