"""tcgen05 split-precision overlap matrix: FP64 accuracy from bf16 tensor cores.

S = 2 Re(C^H C) - Re c0 Re c0^T computed on the tensor cores must match the
FP64 oracle to 1e-13 relative (max-norm), which is what the 1e-12
orthonormality gate after ortho needs, for state counts that exercise partial
tiles (16, 37), several row blocks (130, 200) and for the 85 472-row real view
of the 120^3 cell.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL_TC = 1e-13


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def perturbed(c0, scale, seed):
    rng = np.random.default_rng(seed)
    c = c0 + scale * (rng.standard_normal(c0.shape) + 1j * rng.standard_normal(c0.shape))
    c[0] = c[0].real
    return np.asfortranarray(c)


@pytest.mark.parametrize("nstate", [16, 37, 130, 200])
def test_ovlap_tensor_cores_match_oracle(gpu_lib, nstate):
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=80 + nstate)
    c = perturbed(cl.c0, 0.1, nstate)
    ctx = Context(cl.basis, "fp64")
    ctx.set_option("gemm", 1)
    s = ctx.ovlap(c)
    assert rel(s, O.overlap(c, cl.basis.geq0)) < TOL_TC
    assert np.array_equal(s, s.T)


def test_ovlap_tensor_cores_full_size(gpu_lib):
    import torch
    from cpmd_gb300 import Context
    cl = make_cell("c1")
    c = perturbed(cl.c0, 0.05, 1)
    ctx = Context(cl.basis, "mixed")
    ct = torch.from_numpy(np.ascontiguousarray(c.T)).cuda()
    s_tc = ctx.ovlap(ct).cpu().numpy()
    ctx.set_option("gemm", 0)
    s_64 = ctx.ovlap(ct).cpu().numpy()
    ref = O.overlap(c, cl.basis.geq0)
    assert rel(s_tc, ref) < TOL_TC
    assert rel(s_64, ref) < TOL_TC


def test_mixed_ortho_orthonormality_gate(gpu_lib):
    """After the mixed-mode ortho (tensor-core S, FP64 Cholesky), ||C^H C - I|| <= 1e-12."""
    import torch
    from cpmd_gb300 import Context
    cl = make_cell("c1")
    ctx = Context(cl.basis, "mixed")
    c = torch.from_numpy(np.ascontiguousarray(perturbed(cl.c0, 0.02, 2).T)).cuda()
    sc = ctx.ortho(c, "gs")
    assert sc > 1e-3
    ctx.set_option("gemm", 0)
    s = ctx.ovlap(c)
    dev = float((s - torch.eye(cl.nstate, dtype=torch.float64, device=s.device)).abs().max())
    assert dev <= 1e-12


@pytest.mark.parametrize("nstate,method", [(16, "gs"), (37, "gs"), (130, "gs"), (200, "gs"), (300, "gs"),
                                           (70, "lowdin"), (300, "lowdin")])
def test_ortho_tensor_cores_match_oracle(gpu_lib, nstate, method):
    """Both GEMMs of ortho (S and C M) on the tensor cores give the FP64 result.
    300 states: C M slices its rows with the separate row-maximum pass, runs
    three K-chunks (11 low bits dropped in the epilogue's window conversion) and
    ends on a 12-column tile."""
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=90 + nstate)
    c = perturbed(cl.c0, 0.03, nstate)
    ref = O.rgs(c, cl.basis.geq0) if method == "gs" else O.lowdin(c, cl.basis.geq0)[0]
    ctx = Context(cl.basis, "fp64")
    ctx.set_option("gemm", 1)
    out = c.copy(order="F")
    ctx.ortho(out, method)
    assert rel(out, ref) < 1e-12
    assert np.all(out[0].imag == 0.0)


@pytest.mark.parametrize("nstate", [16, 37, 100])
def test_simt_tile_32_matches_oracle(gpu_lib, nstate):
    """The 32 x 32 tile of the FP64 SIMT overlap and C M GEMMs (GBCP_OPT_SIMT_TILE)
    gives the oracle's overlap and Gram-Schmidt to 1e-12."""
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=500 + nstate)
    c = perturbed(cl.c0, 0.03, nstate)
    ctx = Context(cl.basis, "fp64")
    ctx.set_option("simt_tile", 32)
    assert rel(ctx.ovlap(c), O.overlap(c, cl.basis.geq0)) < 1e-13
    out = c.copy(order="F")
    ctx.ortho(out, "gs")
    assert rel(out, O.rgs(c, cl.basis.geq0)) < 1e-12
