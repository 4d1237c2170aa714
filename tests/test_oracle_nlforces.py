"""CPU checks of the oracle's non-local forces (test infrastructure only):
rnlfor(rnlsm1, rnlsm2) is minus the R-derivative of E_nl = sum f wsg fnl^2,
checked by central finite differences of E_nl with eigr = e^{-iG.R} rebuilt."""
import numpy as np

from cpmd_gb300.synth import make_small_cell
from oracle import cpmd_oracle as O


def _eigr(basis, tau):
    G = basis.gvec_bohr(basis.ngw)
    return np.asfortranarray(np.exp(-1j * (G @ np.asarray(tau).T)))


def test_nl_forces_match_fd():
    cl = make_small_cell(10.26, 20, 8.0, 5, seed=13, with_proj=True)
    b, p = cl.basis, cl.proj
    nghtol = np.array([0, 1, 1, 1, 0, 1, 1, 1], dtype=np.int32)
    f = cl.f.copy()
    f[1] = 1.0
    eig = _eigr(b, cl.tau)
    fnl = O.rnlsm1(cl.c0, p["twnl"], eig, nghtol, b.geq0)
    dfnl = O.rnlsm2(cl.c0, p["twnl"], eig, nghtol, b.mill, b.tpiba, b.geq0)
    F = O.rnlfor(f, fnl, dfnl, p["wsg"])
    h = 1e-4
    for a in (0, 3, 6):
        for k in range(3):
            tp = cl.tau.copy(); tp[a, k] += h
            tm = cl.tau.copy(); tm[a, k] -= h
            ep = O.enl(cl.c0, f, p["twnl"], _eigr(b, tp), nghtol, p["wsg"], b.geq0)
            em = O.enl(cl.c0, f, p["twnl"], _eigr(b, tm), nghtol, p["wsg"], b.geq0)
            assert abs(-(ep - em) / (2 * h) - F[a, k]) < 1e-7 * np.abs(F).max()
