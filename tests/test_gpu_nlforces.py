"""GPU non-local forces: rnlsm2 (dfnl = d fnl / dR) and rnlfor.

FP64 drop-in vs the oracle to 1e-10 relative, host and device memory; the
mixed path (tcgen05 split-bf16 GEMM) to an FP32 dot-product bound; forces vs
central finite differences of E_nl computed through gbcp_rnlsm1 on the GPU.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _eigr(basis, tau):
    G = basis.gvec_bohr(basis.ngw)
    return np.asfortranarray(np.exp(-1j * (G @ np.asarray(tau).T)))


NGHTOL = np.array([0, 1, 1, 1, 0, 1, 1, 1], dtype=np.int32)


def ctx_for(basis, precision="fp64"):
    from cpmd_gb300 import Context
    return Context(basis, precision=precision)


@pytest.mark.parametrize("mode", ["host", "device"])
def test_rnlsm2_rnlfor_fp64(gpu_lib, mode):
    cl = make_small_cell(10.26, 32, 20.0, 9, seed=60, with_proj=True)
    b, p = cl.basis, cl.proj
    eig = p["eigr"]
    dref = O.rnlsm2(cl.c0, p["twnl"], eig, NGHTOL, b.mill, b.tpiba, b.geq0)       # (nat, ngh, 3, n)
    fnl_ref = O.rnlsm1(cl.c0, p["twnl"], eig, NGHTOL, b.geq0)
    f = cl.f.copy()
    f[2] = 0.0
    F_ref = O.rnlfor(f, fnl_ref, dref, p["wsg"])
    ctx = ctx_for(b)
    fion0 = np.random.default_rng(1).standard_normal((len(cl.tau), 3))
    if mode == "host":
        d = ctx.rnlsm2(cl.c0, p["twnl"], eig, NGHTOL)
        fion = fion0.copy()
        ctx.rnlfor(f, np.ascontiguousarray(np.transpose(fnl_ref, (2, 1, 0))), d, p["wsg"], fion)
    else:
        import torch
        t = lambda x: torch.from_numpy(np.ascontiguousarray(x.T if x.ndim == 2 else x)).cuda()
        d = ctx.rnlsm2(t(cl.c0), t(p["twnl"]), t(eig), NGHTOL)
        fion_t = torch.from_numpy(fion0.copy()).cuda()
        ctx.rnlfor(torch.from_numpy(f).cuda(), torch.from_numpy(np.ascontiguousarray(np.transpose(fnl_ref, (2, 1, 0)))).cuda(),
                   d, torch.from_numpy(p["wsg"]).cuda(), fion_t)
        d = d.cpu().numpy()
        fion = fion_t.cpu().numpy()
    assert rel(np.transpose(d, (3, 2, 1, 0)), dref) < 1e-10
    assert rel(fion - fion0, F_ref) < 1e-10


def test_rnlsm2_mixed_tensor_cores(gpu_lib):
    cl = make_cell("c1", with_proj=True)
    b, p = cl.basis, cl.proj
    dref = O.rnlsm2(cl.c0, p["twnl"], p["eigr"], NGHTOL, b.mill, b.tpiba, b.geq0)
    d = ctx_for(b, "mixed").rnlsm2(cl.c0, p["twnl"], p["eigr"], NGHTOL)
    d = np.transpose(d, (3, 2, 1, 0))
    # FP32 dot-product bound: sum over G of |twnl| |G_k| |c| (|eigr| = 1)
    g = np.abs(b.mill[: b.ngw].astype(float)) * b.tpiba
    bound = 2.0 * np.einsum("gv,gk,gi->vki", np.abs(p["twnl"]), g, np.abs(cl.c0))
    err = np.abs(d - dref) / (bound[None] + 1e-300)
    assert err.max() < 1e-5


def test_nl_forces_fd_gpu(gpu_lib):
    cl = make_small_cell(10.26, 24, 12.0, 6, seed=61, with_proj=True)
    b, p = cl.basis, cl.proj
    ctx = ctx_for(b)
    f = cl.f.copy()

    def enl(tau):
        fnl = ctx.rnlsm(cl.c0, p["twnl"], _eigr(b, tau), NGHTOL)          # (n, ngh, nat)
        return float(np.einsum("v,i,iva->", p["wsg"], f, fnl ** 2))

    eig = _eigr(b, cl.tau)
    fnl = ctx.rnlsm(cl.c0, p["twnl"], eig, NGHTOL)
    d = ctx.rnlsm2(cl.c0, p["twnl"], eig, NGHTOL)
    fion = np.zeros((len(cl.tau), 3))
    ctx.rnlfor(f, fnl, d, p["wsg"], fion)
    h = 1e-4
    for a in range(len(cl.tau)):
        for k in range(3):
            tp = cl.tau.copy(); tp[a, k] += h
            tm = cl.tau.copy(); tm[a, k] -= h
            fd = -(enl(tp) - enl(tm)) / (2 * h)
            assert abs(fd - fion[a, k]) < 1e-6 * np.abs(fion).max()
