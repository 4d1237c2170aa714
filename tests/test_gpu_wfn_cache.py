"""The wavefunction cache across host-memory calls (GBCP_OPT_WFN_CACHE).

The reference keeps c0 on the device between rhoofr and vpsi, keyed by
SUM(ABS(c0(:,1))) (cp_cuwfn_put / cp_cuwfn_get, rhoofr_utils.mod.F90:240-245,
vpsi_utils.mod.F90:278-281).  Here rhoofr's upload is reused by vpsi and by the
Gram-Schmidt ortho on the same host array: rho, E_kin and C2 equal those of the
uncached calls bit for bit, and the orthonormalised states agree to rounding (a
cached ortho forms the overlap matrix in one pass, an uncached one in upload
ranges with per-range digit scales); the reused calls upload no states (profiler
timeline), a change of c0's first column is noticed, and setting the option
again drops the copy.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell

pytestmark = pytest.mark.gpu


def run_step(ctx, c0, f, vpot):
    rho, ek, cg, cr = ctx.rhoofr(c0, f)
    c2 = np.zeros_like(c0)
    ctx.vpsi(c0, c2, f, vpot)
    ctx.ortho(c0, "gs")
    return rho, ek, c2, c0


def test_cached_step_equals_uncached_and_skips_uploads(gpu_lib):
    from cpmd_gb300 import Context
    cl = make_cell("c1", nstate=64)
    plain = Context(cl.basis, "mixed")
    cached = Context(cl.basis, "mixed")
    cached.set_option("wfn_cache", 1)
    a = run_step(plain, cl.c0.copy(order="F"), cl.f, cl.vpot)
    cached.profile(True)
    b = run_step(cached, cl.c0.copy(order="F"), cl.f, cl.vpot)
    tl = cached.profile_timeline()
    cached.profile(False)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    assert np.abs(a[3] - b[3]).max() <= 1e-13 * np.abs(a[3]).max()
    # only rhoofr's state uploads: vpsi's c2 and ortho's states are not in 'h2d_states' of c0
    ups = [r for r in tl if r[0] == "h2d_states"]
    ups_plain = None
    plain.profile(True)
    run_step(plain, cl.c0.copy(order="F"), cl.f, cl.vpot)
    ups_plain = [r for r in plain.profile_timeline() if r[0] == "h2d_states"]
    plain.profile(False)
    assert 0 < len(ups) < len(ups_plain)


def test_changed_first_column_is_noticed_and_option_drops_copy(gpu_lib):
    from cpmd_gb300 import Context
    cl = make_cell("c1", nstate=32)
    ctx = Context(cl.basis, "fp64")
    ctx.set_option("wfn_cache", 1)
    ref = Context(cl.basis, "fp64")
    c0 = cl.c0.copy(order="F")
    ctx.rhoofr(c0, cl.f)
    # the caller changes the first column: the key changes, vpsi uploads again
    c0[:, 0] *= 1.5
    c2 = np.zeros_like(c0)
    ctx.vpsi(c0, c2, cl.f, cl.vpot)
    c2r = np.zeros_like(c0)
    ref.vpsi(c0, c2r, cl.f, cl.vpot)
    assert np.array_equal(c2, c2r)
    # a change elsewhere keeps the key: the documented remedy is to set the option again
    ctx.rhoofr(c0, cl.f)
    c0[:, 5] *= -1.0
    ctx.set_option("wfn_cache", 1)
    c2[:] = 0
    ctx.vpsi(c0, c2, cl.f, cl.vpot)
    c2r[:] = 0
    ref.vpsi(c0, c2r, cl.f, cl.vpot)
    assert np.array_equal(c2, c2r)


def test_ortho_on_changed_first_column_restarts_with_upload(gpu_lib):
    """On a likely hit (same array, leading dimension and state count) ortho starts
    the overlap and Cholesky on the cached copy while the host computes the key; a
    first column changed since rhoofr fails that check, the speculative work is
    dropped before C U^-1 writes anything, and the call restarts from the caller's
    array: the result equals that of a context without the cache, bit for bit."""
    from cpmd_gb300 import Context
    cl = make_cell("c1", nstate=32)
    ctx = Context(cl.basis, "mixed")
    ctx.set_option("wfn_cache", 1)
    ref = Context(cl.basis, "mixed")
    c0 = cl.c0.copy(order="F")
    ctx.rhoofr(c0, cl.f)
    c0[:, 0] *= 1.5
    a = c0.copy(order="F")
    ctx.ortho(c0, "gs")
    ref.ortho(a, "gs")
    assert np.array_equal(c0, a)
    # and a true hit after it still agrees with the uncached call to rounding
    b = c0.copy(order="F")
    ctx.rhoofr(c0, cl.f)
    ctx.ortho(c0, "gs")
    ref.ortho(b, "gs")
    assert np.abs(c0 - b).max() <= 1e-13 * np.abs(b).max()


@pytest.mark.parametrize("plan", [0, 4 + 256 * 4 + 65536 * 2, 8 + 256 * 3 + 65536 * 3 + 16777216 * 4,
                                  1 + 256 * 8 + 65536 * 1])
def test_staging_plans_give_the_device_results(gpu_lib, plan):
    """Host-memory rhoofr and vpsi under the automatic and fixed staging plans
    (GBCP_OPT_STAGES: first chunk, chunk count, density groups, last chunk), with and
    without c0 cached on the device, give the device-memory results: the plans only
    reorder copies and launches (rho and C2 to rounding, the scalars to 1e-12)."""
    import torch
    from cpmd_gb300 import Context
    cl = make_cell("c1", nstate=40)
    dev = Context(cl.basis, "fp64")
    c0d = torch.from_numpy(np.ascontiguousarray(cl.c0.T)).cuda()
    fd = torch.from_numpy(cl.f).cuda()
    vd = torch.from_numpy(cl.vpot).cuda()
    rho_d, ek_d, cg_d, cr_d = dev.rhoofr(c0d, fd)
    c2d = torch.zeros_like(c0d)
    dev.vpsi(c0d, c2d, fd, vd)
    rho_d = rho_d.cpu().numpy()
    c2_d = c2d.cpu().numpy().T
    for cache in (0, 1):
        ctx = Context(cl.basis, "fp64")
        ctx.set_option("stages", plan)
        if cache:
            ctx.set_option("wfn_cache", 1)
        c0 = cl.c0.copy(order="F")
        rho, ek, cg, cr = ctx.rhoofr(c0, cl.f)
        c2 = np.zeros_like(c0)
        ctx.vpsi(c0, c2, cl.f, cl.vpot)
        assert np.abs(rho - rho_d).max() <= 1e-13 * np.abs(rho_d).max()
        assert np.abs(c2 - c2_d).max() <= 1e-13 * np.abs(c2_d).max()
        for a, r in ((ek, ek_d), (cg, cg_d), (cr, cr_d)):
            assert abs(a - r) <= 1e-12 * abs(r)
