"""CPU checks of the oracle's CP-dynamics constraint (test infrastructure only).

The restated rortho iteration (rortog_utils.mod.F90:315-498) converges to gam
with sym<c0|cm> gam + gam sym<c0|cm> + gam^2 = I - <cm|cm> (its fixed point),
and cm + c0 gam is orthonormal up to the antisymmetric part of <c0|cm>, which
the reference's algorithm ignores by design."""
import numpy as np
import pytest

from cpmd_gb300.synth import make_small_cell
from oracle import cpmd_oracle as O


def cp_pair(nstate, seed, step=1e-2, nonorth=0.0):
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=seed)
    b = cl.basis
    c0 = O.rgs(cl.c0, b.geq0)
    rng = np.random.default_rng(seed + 100)
    d = (rng.standard_normal(c0.shape) + 1j * rng.standard_normal(c0.shape)) / np.sqrt(c0.shape[0])
    cm = c0 + step * d
    if nonorth:
        c0 = c0 + nonorth * (rng.standard_normal(c0.shape) + 1j * rng.standard_normal(c0.shape)) / np.sqrt(c0.shape[0])
    if b.geq0:
        cm[0] = cm[0].real
        c0[0] = c0[0].real
    return b, np.asfortranarray(c0), np.asfortranarray(cm)


def test_fixed_point_and_constraint():
    b, c0, cm = cp_pair(8, 3)
    gam, cn, it = O.rortho(c0, cm, b.geq0, epsog=1e-13, maxit=60)
    assert it >= 2
    a = O.cross_overlap(c0, cm, b.geq0)
    bs = 0.5 * (a + a.T)
    sig = np.eye(8) - O.cross_overlap(cm, cm, b.geq0)
    assert np.abs(gam - gam.T).max() == 0.0
    assert np.abs(bs @ gam + gam @ bs + gam @ gam - sig).max() < 1e-12
    # orthonormal up to the neglected antisymmetric part of <c0|cm> (second order in the step)
    asym = float(np.abs(0.5 * (a - a.T)).max())
    err = float(np.abs(O.cross_overlap(cn, cn, b.geq0) - np.eye(8)).max())
    assert err < 10 * asym ** 2 + 1e-12


def test_nonorthonormal_c0_fixed_point():
    """With tnon the fixed point carries the <c0|c0> = I - 2 del correction:
    B gam + gam B + gam (I - 2 del) gam = sig."""
    b, c0, cm = cp_pair(6, 5, step=1e-2, nonorth=1e-3)
    gam, _, _ = O.rortho(c0, cm, b.geq0, tnon=True, epsog=1e-13, maxit=60)
    a = O.cross_overlap(c0, cm, b.geq0)
    bs = 0.5 * (a + a.T)
    sig = np.eye(6) - O.cross_overlap(cm, cm, b.geq0)
    s00 = O.cross_overlap(c0, c0, b.geq0)
    assert np.abs(bs @ gam + gam @ bs + gam @ s00 @ gam - sig).max() < 1e-12
    g0, _, _ = O.rortho(c0, cm, b.geq0, tnon=False, epsog=1e-13, maxit=60)
    assert np.abs(g0 - gam).max() > 1e-12  # the term is present (second order in gam)


def test_iteration_limit_raises():
    b, c0, cm = cp_pair(6, 7, step=5e-2)
    with pytest.raises(RuntimeError):
        O.rortho(c0, cm, b.geq0, epsog=1e-14, maxit=1)
