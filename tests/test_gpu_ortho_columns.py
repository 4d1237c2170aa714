"""Host-memory Gram-Schmidt by column blocks (GBCP_OPT_ORTHO_COLUMNS).

For 65 to 256 states the host-memory call runs C U^-1 and the download column
block by column block (32 states) as the blocked Cholesky chain finishes each
block of U^-1 (rgs_utils.mod.F90:63-74: C U^-1 with U from dpotrf/dtrtri), so the
copy to the host starts after the first diagonal block.  The states must equal
those of the G-row-range path (option 0) bit for bit, with and without the
wavefunction cache, in both precisions, match the oracle's rgs, and a failed
factorisation must leave the host array as it was.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu


def perturbed(c0, scale, seed):
    rng = np.random.default_rng(seed)
    c = c0 + scale * (rng.standard_normal(c0.shape) + 1j * rng.standard_normal(c0.shape))
    c[0] = c[0].real
    return np.asfortranarray(c)


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("nstate", [65, 97, 128, 200, 256])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("cached", [False, True])
def test_column_blocks_equal_row_ranges(gpu_lib, nstate, precision, cached):
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 36, 30.0, nstate, seed=600 + nstate)
    c = perturbed(cl.c0, 0.03, nstate)
    outs = []
    for cols in (0, 1):
        ctx = Context(cl.basis, precision)
        ctx.set_option("gemm", 1)
        ctx.set_option("ortho_columns", cols)
        out = c.copy(order="F")
        if cached:
            ctx.set_option("wfn_cache", 1)
            ctx.rhoofr(out, cl.f)  # uploads c0; ortho then starts on the device copy
        ctx.ortho(out, "gs")
        outs.append(out)
    assert np.array_equal(outs[0], outs[1])
    assert rel(outs[1], O.rgs(c, cl.basis.geq0)) < 1e-12
    assert np.all(outs[1][0].imag == 0.0)


def test_column_blocks_failed_factorisation_leaves_host_states(gpu_lib):
    from cpmd_gb300 import Context, GbcpError
    cl = make_small_cell(10.26, 36, 30.0, 130, seed=611)
    c = cl.c0.copy(order="F")
    c[:, 120] = c[:, 7]  # an exactly dependent pair: the pivot of state 121 vanishes
    keep = c.copy(order="F")
    ctx = Context(cl.basis, "mixed")
    with pytest.raises(GbcpError) as e:
        ctx.ortho(c, "gs")
    assert e.value.code == 2
    assert np.array_equal(c, keep)
    ok = perturbed(cl.c0, 0.03, 5)
    ref = O.rgs(ok, cl.basis.geq0)
    ctx.ortho(ok, "gs")
    assert rel(ok, ref) < 1e-12


@pytest.mark.parametrize("cached", [False, True])
def test_column_blocks_with_upload_ranges(gpu_lib, cached):
    """ngw = 42 736: four G-row upload ranges, whose overlap parts and row planes start
    as each range lands (uncached), or one pass on the cached copy."""
    from cpmd_gb300 import Context
    from cpmd_gb300.synth import make_cell
    cl = make_cell("c1", nstate=100)
    c = perturbed(cl.c0, 0.02, 100)
    outs = []
    for cols in (0, 1):
        ctx = Context(cl.basis, "mixed")
        ctx.set_option("ortho_columns", cols)
        out = c.copy(order="F")
        if cached:
            ctx.set_option("wfn_cache", 1)
            ctx.rhoofr(out, cl.f)
        ctx.ortho(out, "gs")
        outs.append(out)
    assert np.array_equal(outs[0], outs[1])
    assert rel(outs[1], O.rgs(c, cl.basis.geq0)) < 1e-12
