"""Mixed-precision projector contractions on the tcgen05 tensor cores.

rnlsm1 and fnonloc in the mixed mode run as split-bf16 (three slices, six
slice pairs) GEMMs fed by TMA, accumulated in FP32: the accuracy of an FP32
GEMM.  The bound checked is that of an FP32 dot product, elementwise against
the sum of absolute terms: |D - D_ref| <= 1e-5 (|A| |B|) (the inputs alone are
rounded to 2^-24 relative); the FP64 engine stays selectable with
GBCP_OPT_GEMM = 0 and then matches to 1e-10 relative.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL_TC = 1e-5


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def ctx_for(basis, precision="mixed"):
    from cpmd_gb300 import Context
    return Context(basis, precision=precision)


def abs_bounds(cl, nghtol, f, fnl_ref):
    """|scr|^T |c| (fnl scale, G = 0 halved) and |Y| |Z| (fnonloc scale)."""
    b, p = cl.basis, cl.proj
    aw = np.abs(p["twnl"])
    ac = np.abs(cl.c0)
    if b.geq0:
        aw = aw.copy()
        aw[0] *= 0.5
    # |scr(G, ia, iv)| = |twnl(G, iv)| since |eigr| = 1, and |re a re b| + |im a im b| <= |a| |b|
    bf = 2.0 * np.einsum("gv,gi->vi", aw, ac)                       # (ngh, n), same for every atom
    ffi = np.where(f < 1e-5, 1.0, f)
    z = np.abs(fnl_ref) * (ffi[None, None, :] * np.abs(p["wsg"])[None, :, None])   # (nat, ngh, n)
    bc = np.einsum("gv,vi->gi", np.abs(p["twnl"]), z.sum(axis=0))  # (ngw, n)
    return bf, bc


def run_case(cl, nghtol, gemm=None, tol=TOL_TC, device=False):
    b, p = cl.basis, cl.proj
    f = cl.f.copy()
    f[min(4, len(f) - 1)] = 0.0
    fnl_ref = O.rnlsm1(cl.c0, p["twnl"], p["eigr"], nghtol, b.geq0)
    ctx = ctx_for(b)
    if gemm is not None:
        ctx.set_option("gemm", gemm)
    rng = np.random.default_rng(3)
    c2in = np.asfortranarray((rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape)) * 0.1)
    ref = O.fnonloc(c2in, f, fnl_ref, p["twnl"], p["eigr"], nghtol, p["wsg"])
    fnl_in = np.ascontiguousarray(np.transpose(fnl_ref, (2, 1, 0)))
    if device:
        import torch
        d = lambda x: torch.from_numpy(np.ascontiguousarray(x.T if x.ndim == 2 else x)).cuda()
        fnl = ctx.rnlsm(d(cl.c0), d(p["twnl"]), d(p["eigr"]), nghtol).cpu().numpy()
        c2d = d(c2in)
        ctx.fnonloc(c2d, d(f), torch.from_numpy(fnl_in).cuda(), d(p["twnl"]), d(p["eigr"]), nghtol,
                    torch.from_numpy(p["wsg"]).cuda())
        c2 = np.asfortranarray(c2d.cpu().numpy().T)
    else:
        fnl = ctx.rnlsm(cl.c0, p["twnl"], p["eigr"], nghtol)
        c2 = c2in.copy(order="F")
        ctx.fnonloc(c2, f, fnl_in, p["twnl"], p["eigr"], nghtol, p["wsg"])
    fnl_t = np.transpose(fnl, (2, 1, 0))
    if gemm == 0:
        assert rel(fnl_t, fnl_ref) < tol
        assert rel(c2 - c2in, ref - c2in) < tol
        return
    bf, bc = abs_bounds(cl, nghtol, f, fnl_ref)
    ef = float((np.abs(fnl_t - fnl_ref) / bf[None, :, :]).max())
    ec = float((np.abs(c2 - ref) / bc).max())
    print(f"normalised errors: fnl {ef:.2e}, c2 {ec:.2e}; max-norm rel fnl {rel(fnl_t, fnl_ref):.2e}")
    assert ef < tol
    assert ec < tol


def test_projectors_tc_small(gpu_lib):
    cl = make_small_cell(10.26, 32, 20.0, 9, seed=50, with_proj=True)
    run_case(cl, cl.proj["nghtol"])


def test_projectors_tc_all_angular_phases(gpu_lib):
    cl = make_small_cell(10.26, 32, 20.0, 7, seed=51, with_proj=True)
    run_case(cl, np.array([0, 1, 2, 3, 3, 2, 1, 0], dtype=np.int32), device=True)


def test_projectors_tc_medium_multi_tile(gpu_lib):
    """64 atoms x 8 projectors (M = 512), 128 states, K = 2 ngw = 85k: split-K and many fnonloc tiles."""
    cl = make_cell("c1", with_proj=True)
    run_case(cl, cl.proj["nghtol"])


def test_projectors_fp64_engine_in_mixed(gpu_lib):
    cl = make_small_cell(10.26, 32, 20.0, 9, seed=52, with_proj=True)
    run_case(cl, cl.proj["nghtol"], gemm=0, tol=1e-10)
