"""vpsi reuses the Z stage of the rhoofr before it on the same device states (GBCP_OPT_ZKEEP).

A device-memory gbcp_vpsi that follows a device-memory gbcp_rhoofr on the same c0
(pointer, leading dimension and state count, both calls one launch batch) skips its
inverse z-transforms when a position-keyed checksum of all of c0, taken on the device
by both calls, is unchanged: zbuf still holds rhoofr's transforms.  The reference
reuses its device copy of c0 on a match of SUM(ABS(c0(:,1))) (vpsi_utils.mod.F90:
278-281).  C2 must equal that of a context with the option off bit for bit, on every
Z-stage kernel (four-step with and without the mirror-pair gather, Stockham); a change
of c0 between the calls (one coefficient, two states exchanged), a second vpsi, or a
rhoofr on another array in between must be noticed.  Host-memory calls keep the Z
stage only through the wavefunction cache: a vpsi on the staging copy the rhoofr
uploaded (its key confirmed) runs no Z stage.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell

pytestmark = pytest.mark.gpu


def dev(x):
    import torch
    if x.dtype == np.complex128 and x.ndim == 2:
        return torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def pair(basis, precision, **opts):
    from cpmd_gb300 import Context
    on, off = Context(basis, precision), Context(basis, precision)
    off.set_option("zkeep", 0)
    for k, v in opts.items():
        on.set_option(k, v)
        off.set_option(k, v)
    return on, off


def step(ctx, c0, f, v, c2in=None):
    import torch
    rho = ctx.rhoofr(c0, f)[0]
    c2 = torch.zeros_like(c0) if c2in is None else c2in.clone()
    ctx.vpsi(c0, c2, f, v)
    return rho.cpu().numpy(), c2.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("opts", [{}, {"zmirror": 1}, {"zmirror": 0}, {"fft": 2}, {"plane": 3}])
def test_kept_z_stage_gives_the_same_rho_and_c2(gpu_lib, precision, opts):
    cl = make_cell("c0")
    on, off = pair(cl.basis, precision, **opts)
    c0, f, v = dev(cl.c0), dev(cl.f), dev(cl.vpot)
    a, b = step(on, c0, f, v), step(off, c0, f, v)
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(a[1], b[1])


@pytest.mark.parametrize("nstate", [1, 5, 12])
def test_kept_z_stage_odd_counts_and_leading_dimension(gpu_lib, nstate):
    import torch
    cl = make_small_cell(10.26, 36, 20.0, nstate, seed=40 + nstate)
    on, off = pair(cl.basis, "mixed")
    ngw = cl.c0.shape[0]
    rng = np.random.default_rng(nstate)

    def wide(x):  # states in rows of ngw + 3 coefficients: leading dimension ngw + 3
        w = torch.from_numpy(rng.standard_normal((nstate, ngw + 3)) + 0j).cuda()
        w[:, :ngw] = dev(x)
        return w

    c0 = wide(cl.c0)
    c2in = wide(np.asfortranarray(rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape)))
    f, v = dev(cl.f), dev(cl.vpot)
    a, b = step(on, c0, f, v, c2in), step(off, c0, f, v, c2in)
    assert np.array_equal(a[1], b[1])
    # the padding is not part of the states: changing it keeps the Z stage, same C2
    on.rhoofr(c0, f)
    c0[:, ngw:] = 7.0
    c2 = c2in.clone()
    on.vpsi(c0, c2, f, v)
    assert np.array_equal(c2.cpu().numpy(), b[1])


@pytest.mark.parametrize("change", ["coefficient", "exchange", "other_rhoofr", "second_vpsi"])
def test_changes_between_the_calls_are_noticed(gpu_lib, change):
    import torch
    cl = make_cell("c0")
    on, off = pair(cl.basis, "mixed")
    c0, f, v = dev(cl.c0), dev(cl.f), dev(cl.vpot)
    on.rhoofr(c0, f)
    if change == "coefficient":
        c0[5, 17] = c0[5, 17] * 1.5  # one coefficient of state 6
    elif change == "exchange":
        c0[[2, 3]] = c0[[3, 2]].clone()  # states 3 and 4 exchanged: the same multiset of words
    elif change == "other_rhoofr":
        on.rhoofr(dev(np.asfortranarray(cl.c0[:, ::-1])), f)
    c2 = torch.zeros_like(c0)
    on.vpsi(c0, c2, f, v)
    if change == "second_vpsi":
        c2[:] = 0
        on.vpsi(c0, c2, f, v)
    c2r = torch.zeros_like(c0)
    off.vpsi(c0, c2r, f, v)
    assert torch.equal(c2, c2r)


def test_host_memory_calls_keep_nothing(gpu_lib):
    """Host-memory calls stage c0 in chunks: nothing is kept, and a device vpsi after a
    host rhoofr on equal values computes its own Z stage."""
    cl = make_cell("c0")
    on, off = pair(cl.basis, "mixed")
    on.rhoofr(cl.c0, cl.f)
    c2 = np.zeros_like(cl.c0)
    on.vpsi(cl.c0, c2, cl.f, cl.vpot)
    c2r = np.zeros_like(cl.c0)
    off.vpsi(cl.c0, c2r, cl.f, cl.vpot)
    assert np.array_equal(c2, c2r)
    c0, f, v = dev(cl.c0), dev(cl.f), dev(cl.vpot)
    on.rhoofr(cl.c0, cl.f)
    import torch
    c2d = torch.zeros_like(c0)
    on.vpsi(c0, c2d, f, v)
    c2dr = torch.zeros_like(c0)
    off.vpsi(c0, c2dr, f, v)
    assert torch.equal(c2d, c2dr)


def test_host_staged_vpsi_on_the_cached_copy_skips_the_z_stage(gpu_lib):
    """With the wavefunction cache, a host-memory vpsi on the array the host-memory
    rhoofr just uploaded finds rhoofr's inverse z-transforms of all pairs in zbuf and
    runs no Z stage; C2 equals that of the option off bit for bit.  A changed first
    column (a new key) uploads and transforms again."""
    from cpmd_gb300 import Context
    cl = make_cell("c1", nstate=64)
    on, off = pair(cl.basis, "mixed", wfn_cache=1)
    res = []
    for ctx in (on, off):
        c0 = cl.c0.copy(order="F")
        ctx.rhoofr(c0, cl.f)
        ctx.profile(True)
        c2 = np.zeros_like(c0)
        ctx.vpsi(c0, c2, cl.f, cl.vpot)
        names = [r[0] for r in ctx.profile_timeline()]
        ctx.profile(False)
        res.append((c2, names))
    assert np.array_equal(res[0][0], res[1][0])
    assert "k_zinv" not in res[0][1] and "k_zinv" in res[1][1]
    # a new key: the Z stage runs again and C2 is that of the changed states
    c0 = cl.c0.copy(order="F")
    on.rhoofr(c0, cl.f)
    c0[:, 0] *= 1.5
    c2 = np.zeros_like(c0)
    on.vpsi(c0, c2, cl.f, cl.vpot)
    c2r = np.zeros_like(c0)
    Context(cl.basis, "mixed").vpsi(c0, c2r, cl.f, cl.vpot)
    assert np.array_equal(c2, c2r)
