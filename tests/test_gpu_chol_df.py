"""The double-float Cholesky factor and inverse of ortho (GBCP_OPT_CHOL): one CTA
up to 64 states (128 with option 3), double-float diagonal blocks of the
blocked chain above.

Gram-Schmidt through them must match the oracle's rgs (dpotrf + dtrtri + dtrmm,
rgs_utils.mod.F90:63-74, 95-162) and keep ||C^H C - I|| <= 1e-12 at every size
(1..200 states: both one-CTA instances, partial column pairs, partial diagonal
blocks), be invariant to
positive scaling of the states (the power-of-two scaling of the overlap matrix
keeps any magnitude inside FP32's range) and report an exactly dependent set as
not positive definite, like the FP64 chain.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def perturbed(c0, scale, seed):
    rng = np.random.default_rng(seed)
    c = c0 + scale * (rng.standard_normal(c0.shape) + 1j * rng.standard_normal(c0.shape))
    c[0] = c[0].real
    return np.asfortranarray(c)


def orthonormality(c, geq0=True):
    s = O.overlap(c, geq0)
    return float(np.abs(s - np.eye(s.shape[0])).max())


@pytest.mark.parametrize("nstate,opt", [(1, 1), (5, 1), (33, 1), (64, 1), (65, 1), (97, 1), (128, 1), (200, 1),
                                       (65, 3), (128, 3)])
def test_gs_double_float_matches_oracle(gpu_lib, nstate, opt):
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=300 + nstate)
    c = perturbed(cl.c0, 0.03, nstate)
    ref = O.rgs(c, cl.basis.geq0)
    ctx = Context(cl.basis, "mixed")
    ctx.set_option("chol", opt)
    out = c.copy(order="F")
    ctx.ortho(out, "gs")
    assert rel(out, ref) < 1e-12
    assert orthonormality(out, cl.basis.geq0) <= 1e-12
    assert np.all(out[0].imag == 0.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_chol_option_engines_agree(gpu_lib, precision):
    """Options 0 (blocked FP64), 1 (double-float in the mixed precision, the
    default), 2 (double-float in both) and 3 (one CTA to 128 states) give the same
    orthonormal set to 1e-12."""
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, 100, seed=411)
    c = perturbed(cl.c0, 0.05, 7)
    ctx = Context(cl.basis, precision)
    outs = []
    for opt in (0, 1, 2, 3):
        ctx.set_option("chol", opt)
        out = c.copy(order="F")
        ctx.ortho(out, "gs")
        outs.append(out)
    for o in outs[1:]:
        assert rel(o, outs[0]) < 1e-12
        assert orthonormality(o, cl.basis.geq0) <= 1e-12


@pytest.mark.parametrize("nstate", [48, 100])
def test_gs_double_float_scale_invariant(gpu_lib, nstate):
    """Gram-Schmidt of states scaled by 2^-40 .. 2^40 (overlap entries 2^-80 ..
    2^80, far outside FP32's range unscaled) is the Gram-Schmidt of the states.
    FP64 GEMMs around the double-float kernel (option 2): the tensor-core C M
    bounds its error by the row maxima of C, which such a spread of state
    norms defeats whatever the Cholesky does."""
    from cpmd_gb300 import Context
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=412)
    c = perturbed(cl.c0, 0.02, 8)
    ref = O.rgs(c, cl.basis.geq0)
    scales = 2.0 ** np.linspace(-40, 40, nstate).round()
    cs = np.asfortranarray(c * scales[None, :])
    ctx = Context(cl.basis, "fp64")
    ctx.set_option("chol", 2)
    ctx.ortho(cs, "gs")
    assert rel(cs, ref) < 1e-12


@pytest.mark.parametrize("nstate,dup", [(4, (2, 3)), (100, (17, 90))])
def test_gs_double_float_dependent_states_not_spd(gpu_lib, nstate, dup):
    from cpmd_gb300 import Context, GbcpError
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=413)
    c = cl.c0.copy(order="F")
    c[:, dup[1]] = c[:, dup[0]]
    keep = c.copy(order="F")
    ctx = Context(cl.basis, "mixed")
    ctx.set_option("chol", 1)
    with pytest.raises(GbcpError) as e:
        ctx.ortho(c, "gs")
    assert e.value.code == 2
    assert np.array_equal(c, keep)  # a failed step leaves the states as they were
    ok = cl.c0.copy(order="F")
    ctx.ortho(ok, "gs")
    assert orthonormality(ok, cl.basis.geq0) <= 1e-12
