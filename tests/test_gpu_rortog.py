"""GPU parity of the CP-dynamics constraint (gbcp_rortog: rortog -> rortho,
rortog_utils.mod.F90:315-498) against the oracle, through the C ABI.

Tolerances: the FP64 drop-in and the mixed mode (whose overlaps and c0 gam
update run as FP64-accurate split GEMMs on the tensor cores) both match the
oracle's gam and updated cm to 1e-10 relative; the iteration count matches
exactly."""
import numpy as np
import pytest

from cpmd_gb300 import Context
from tests.test_oracle_rortho import cp_pair
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("tnon", [False, True])
def test_rortog_parity_host(gpu_lib, precision, tnon):
    b, c0, cm = cp_pair(12, 21, step=2e-2, nonorth=1e-3 if tnon else 0.0)
    g_ref, cm_ref, it_ref = O.rortho(c0, cm, b.geq0, tnon=tnon, epsog=1e-9, maxit=30)
    ctx = Context(b, precision=precision)
    cmg = cm.copy(order="F")
    gam, it = ctx.rortog(c0, cmg, tnon=tnon, epsog=1e-9, maxit=30)
    assert it == it_ref
    assert rel(gam, g_ref) < TOL
    assert rel(cmg, cm_ref) < TOL
    assert np.array_equal(gam, gam.T)


def test_rortog_device_and_leading_dimension(gpu_lib):
    import torch
    b, c0, cm = cp_pair(10, 23, step=1e-2)
    g_ref, cm_ref, it_ref = O.rortho(c0, cm, b.geq0, epsog=1e-8, maxit=30)
    ctx = Context(b, precision="fp64")
    # device tensors are (nstate, ld) row-major == Fortran (ld, nstate); ld > ngw
    ld = b.ngw + 5
    d0 = torch.zeros((10, ld), dtype=torch.complex128, device="cuda")
    dm = torch.zeros((10, ld), dtype=torch.complex128, device="cuda")
    d0[:, : b.ngw] = torch.from_numpy(np.ascontiguousarray(c0.T))
    dm[:, : b.ngw] = torch.from_numpy(np.ascontiguousarray(cm.T))
    gam, it = ctx.rortog(d0, dm, epsog=1e-8, maxit=30)
    torch.cuda.synchronize()
    assert it == it_ref
    assert rel(gam.cpu().numpy(), g_ref) < TOL
    assert rel(dm[:, : b.ngw].cpu().numpy().T, cm_ref) < TOL
    assert torch.all(dm[:, b.ngw:] == 0)


def test_rortog_not_converged_leaves_cm(gpu_lib):
    from cpmd_gb300._lib import GbcpError
    b, c0, cm = cp_pair(8, 25, step=5e-2)
    ctx = Context(b, precision="fp64")
    cmg = cm.copy(order="F")
    with pytest.raises(GbcpError) as e:
        ctx.rortog(c0, cmg, epsog=1e-14, maxit=1)
    assert e.value.code == 8
    assert np.array_equal(cmg, cm)


def test_rortog_cp_step_keeps_orthonormality(gpu_lib):
    """A short CP-like sequence: cm = 2 c0 - c_prev + small force step, then the
    constraint; the states stay orthonormal to second order in the step."""
    b, c0, _ = cp_pair(16, 27)
    ctx = Context(b, precision="mixed")
    rng = np.random.default_rng(5)
    prev = c0.copy(order="F")
    cur = c0.copy(order="F")
    for _ in range(3):
        force = 1e-3 * (rng.standard_normal(cur.shape) + 1j * rng.standard_normal(cur.shape)) / np.sqrt(cur.shape[0])
        if b.geq0:
            force[0] = force[0].real
        nxt = np.asfortranarray(2 * cur - prev + force)
        ctx.rortog(cur, nxt, epsog=1e-10, maxit=30)
        err = np.abs(O.cross_overlap(nxt, nxt, b.geq0) - np.eye(16)).max()
        assert err < 1e-5
        prev, cur = cur, nxt
