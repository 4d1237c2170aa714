"""The C++/OpenMP FP64 restatement (oracle/cpmd_port.cpp), the timed CPU
baseline of the benchmark, against the numpy oracle: its mixed-radix FFT
against numpy's, and rhoofr / vpsi / Gram-Schmidt on the 8-atom cell and on
odd cases (odd state count, a 36^3 mesh, one state).  No GPU is involved."""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O
from oracle import cpmd_port as CP


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 8, 12, 15, 20, 32, 36, 60, 72, 96, 120, 144, 240])
def test_port_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert np.abs(CP.fft1(x, +1) - np.fft.ifft(x) * n).max() <= 1e-14 * np.abs(x).sum()
    assert np.abs(CP.fft1(x, -1) - np.fft.fft(x)).max() <= 1e-14 * np.abs(x).sum()


def test_port_rejects_non_smooth_length():
    with pytest.raises(ValueError):
        CP.fft1(np.ones(7, complex), 1)


@pytest.mark.parametrize("case", ["c0", "odd36", "one"])
def test_port_matches_oracle(case):
    if case == "c0":
        cl = make_cell("c0")
    elif case == "odd36":
        cl = make_small_cell(10.26, 36, 20.0, 7, seed=3)
    else:
        cl = make_small_cell(10.26, 32, 20.0, 1, seed=4)
    b = cl.basis
    port = CP.Port(b, threads=4)
    rho, ek, cg, cr = port.rhoofr(cl.c0, cl.f)
    rr, ek2, cg2, cr2 = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    assert rel(rho, rr) < 1e-13
    assert abs(ek - ek2) <= 1e-13 * abs(ek2) and abs(cg - cg2) <= 1e-13 * abs(cg2)
    assert abs(cr - cr2) <= 1e-13 * abs(cr2)
    c2 = np.zeros_like(cl.c0)
    port.vpsi(cl.c0, c2, cl.f, cl.vpot)
    c2r = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    assert rel(c2, c2r) < 1e-13
    rng = np.random.default_rng(9)
    cp = np.asfortranarray(cl.c0 + 0.02 * (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape)))
    cp[0] = cp[0].real
    co = cp.copy(order="F")
    port.rgs(co)
    assert rel(co, O.rgs(cp, b.geq0)) < 1e-12
    port.close()
