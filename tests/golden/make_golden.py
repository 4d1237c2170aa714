"""Regenerate tests/golden/cell_small.npz from the FP64 oracle.

The reference ships no golden vectors for this path and cannot be built here,
so this fixture is an oracle regression pin: a tiny seeded cell (alat 10.26,
mesh 20^3, 8 Ry, 5 states, one odd state) with rhoofr / vpsi / rgs outputs.
Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from cpmd_gb300.synth import make_small_cell  # noqa: E402
from oracle import cpmd_oracle as O  # noqa: E402


def main():
    alat, nr, ecut, n = 10.26, 20, 8.0, 5
    cl = make_small_cell(alat, nr, ecut, n, seed=2024)
    b = cl.basis
    rho, ekin, csumg, csumr = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    c2 = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    rng = np.random.default_rng(99)
    cp = cl.c0 + 0.05 * (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    cp[0] = cp[0].real
    cp = np.asfortranarray(cp)
    cgs = O.rgs(cp, b.geq0)
    np.savez_compressed(Path(__file__).parent / "cell_small.npz", alat=alat, nr=nr, ecut=ecut, ngw=b.ngw,
                        c0=cl.c0, f=cl.f, vpot=cl.vpot, rho=rho, ekin=ekin, csumg=csumg, csumr=csumr, c2=c2,
                        c_pert=cp, c_gs=cgs)


if __name__ == "__main__":
    main()
