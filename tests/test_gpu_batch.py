"""Many-cell batch (gbcp_batch_*): one CUDA-graph launch per step, autotuned per size class.

Every cell of a batch must give what a context of its own gives: rho, C2 and
the orthonormalised states to 1e-12 relative in FP64 (the autotuner may change
the pairs per launch and the FFT kernels, which reorders rounding only), the
energies E_kin and Omega/N sum V rho to 1e-12, and the oracle to 1e-10.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import batch_cell, make_batch
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def dev_io(cells):
    import torch
    io = []
    for cl in cells:
        b = cl.basis
        io.append(dict(c0=torch.from_numpy(np.ascontiguousarray(cl.c0.T)).cuda(),
                       f=torch.from_numpy(cl.f).cuda(), vpot=torch.from_numpy(cl.vpot).cuda(),
                       rhoe=torch.empty(tuple(b.kr[::-1]), dtype=torch.float64, device="cuda"),
                       c2=torch.zeros((cl.c0.shape[1], b.ngw), dtype=torch.complex128, device="cuda")))
    return io


def single(cl, precision):
    from cpmd_gb300 import Context
    ctx = Context(cl.basis, precision)
    rho, ekin, _, _ = ctx.rhoofr(cl.c0, cl.f)
    c2 = np.zeros_like(cl.c0)
    ctx.vpsi(cl.c0, c2, cl.f, cl.vpot)
    c = cl.c0.copy(order="F")
    ctx.ortho(c, "gs")
    b = cl.basis
    ev = b.omega / np.prod(b.nr) * float((rho * cl.vpot).sum())
    ctx.close()
    return rho, c2, c, ekin, ev


@pytest.fixture(scope="module")
def cells():
    # three size classes: 8 atoms (three cells), 16 (two), 32 (one)
    return [batch_cell(n, 100 + i) for i, n in enumerate((8, 16, 8, 32, 16, 8))]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-6)])
def test_batch_matches_single_contexts(gpu_lib, cells, precision, tol):
    from cpmd_gb300 import Batch
    bt = Batch([c.basis for c in cells], precision, nstreams=4)
    io = dev_io(cells)
    report = bt.tune(io)
    assert report.count("\n") == 3          # three size classes: 8, 16 and 32 atoms
    en, st = bt.step(io)
    assert (st == 0).all()
    assert bt.graph_kernels() > 0
    for cl, x, e in zip(cells, io, en):
        rho, c2, c, ekin, ev = single(cl, precision)
        assert rel(x["rhoe"].cpu().numpy(), rho) < tol
        assert rel(np.asfortranarray(x["c2"].cpu().numpy().T), c2) < tol
        assert rel(np.asfortranarray(x["c0"].cpu().numpy().T), c) < max(tol, 1e-12)
        assert abs(e[0] - ekin) <= 1e-12 * abs(ekin)
        assert abs(e[1] - ev) <= max(tol, 1e-12) * abs(ev)
    bt.close()


def test_batch_replay_and_oracle(gpu_lib, cells):
    """Second step replays the captured graph: c2 accumulates twice, c0 stays orthonormal."""
    from cpmd_gb300 import Batch
    bt = Batch([c.basis for c in cells], "fp64", nstreams=3)
    io = dev_io(cells)
    bt.step(io, ("rhoofr", "vpsi"))
    nk = bt.graph_kernels()
    en, st = bt.step(io, ("rhoofr", "vpsi"))
    assert bt.graph_kernels() == nk
    cl = cells[3]
    b = cl.basis
    rho, ekin, _, _ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    c2 = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    assert rel(io[3]["rhoe"].cpu().numpy(), rho) < 1e-10
    assert rel(np.asfortranarray(io[3]["c2"].cpu().numpy().T), 2 * c2) < 1e-10
    assert abs(en[3][0] - ekin) < 1e-10 * ekin
    bt.close()


def test_make_batch_shapes():
    cells = make_batch(8, seed=9)
    for cl in cells:
        nat = cl.tau.shape[0]
        assert nat in (8, 16, 32, 64)
        assert cl.c0.shape[1] == 2 * nat
        assert cl.basis.nr[0] in (32, 36, 40, 48, 60, 64, 72, 80, 96)


def test_batch_complex64_states(gpu_lib, cells):
    """Complex64 storage of the states (GBCP_STEP_PSI_C64, a mixed batch): rho and
    E_kin are those of a mixed context on the same (complex64-representable)
    states to FP32 rounding (the autotuner may pick other launch shapes), C2 too
    (the update runs in FP32 into complex64), and ortho gives the oracle's
    Gram-Schmidt of those states rounded to complex64."""
    import torch
    from cpmd_gb300 import Batch
    bt = Batch([c.basis for c in cells], "mixed", nstreams=4)
    io = dev_io(cells)
    for x in io:
        x["c0"] = x["c0"].to(torch.complex64)
        x["c2"] = x["c2"].to(torch.complex64)
    report = bt.tune(io)
    assert report.count("\n") == 3
    c0_in = [np.asfortranarray(x["c0"].cpu().numpy().T).astype(np.complex128) for x in io]
    en, st = bt.step(io)
    assert (st == 0).all()
    from cpmd_gb300 import Context
    for cl, x, e, c in zip(cells, io, en, c0_in):
        b = cl.basis
        ctx = Context(b, "mixed")
        rho, ekin, _, _ = ctx.rhoofr(c, cl.f)
        c2 = np.zeros_like(c)
        ctx.vpsi(c, c2, cl.f, cl.vpot)
        ctx.close()
        assert rel(x["rhoe"].cpu().numpy(), rho) < 2e-6
        assert abs(e[0] - ekin) <= 1e-7 * abs(ekin)
        assert rel(np.asfortranarray(x["c2"].cpu().numpy().T).astype(np.complex128), c2) < 1e-6
        out = np.asfortranarray(x["c0"].cpu().numpy().T).astype(np.complex128)
        ref = O.rgs(c, b.geq0)
        assert rel(out, ref) < 1e-6
        s = O.overlap(out, b.geq0)
        assert np.abs(s - np.eye(s.shape[0])).max() < 1e-6
    bt.close()
