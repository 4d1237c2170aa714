"""Plane-wave basis set-up for a cubic Γ-point cell (the caller's side of the boundary).

In CPMD the G-vector list, its ordering and the Miller-index table ``inyh`` are
built once by ``loadpa``/``rggen`` before any hot-path routine runs; the hot
path receives them as module globals.  The GB300 drop-in receives them
explicitly (``gbcp_ctx_create``), so a caller that is not CPMD itself needs the
same list.  This module rebuilds it:

* loop order and acceptance test  -- loadpa_utils.mod.F90:286-330
  (i = 0..nr1-1; j >= 0 when i = 0; k >= 0 when i = j = 0; g2 < gcut)
* tie-breaking sort key            -- loadpa_utils.mod.F90:324
  hg = g2*(1 + sqrt(ig-1)*epsgx*sign), sign = -1 inside the wavefunction
  sphere, +1 outside, epsgx = 1e-12 (gvec.mod.F90:12)
* sort and exact hg recompute      -- loadpa_utils.mod.F90:408, 748-792;
  rggen_utils.mod.F90:118-127
* cut-offs                         -- setsc_utils.mod.F90:169-184
  (gcutw = ecut/tpiba2, gcut = 4*gcutw, tpiba = 2*pi/alat)
* leading dimensions               -- loadpa_utils.mod.F90:509-525
  (kr = nr + mod(nr+1, 2): odd leading dimensions of real-space arrays)

Only the cubic cell (b1, b2, b3 = unit vectors in 2*pi/alat) is needed here.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

EPSGX = 1.0e-12


def leadim(nr: int) -> int:
    """Odd leading dimension used for real-space arrays (loadpa_utils.mod.F90:520)."""
    return nr + (nr + 1) % 2


@dataclass
class Basis:
    alat: float          # cubic cell edge (bohr)
    nr: tuple            # FFT mesh (nr1, nr2, nr3)
    kr: tuple            # leading dimensions (kr1, kr2, kr3) of real-space arrays
    ecut: float          # wavefunction cut-off (Ry)
    tpiba: float
    tpiba2: float
    omega: float
    ngw: int             # wavefunction half-sphere size (G = 0 first)
    nhg: int             # density half-sphere size
    inyh: np.ndarray     # int32 (3, nhg), Miller index + nh (1-based, centred), cppt::inyh
    mill: np.ndarray     # int32 (nhg, 3), signed Miller indices
    hg: np.ndarray       # float64 (nhg,), |G|^2 in (2*pi/alat)^2
    geq0: bool

    @property
    def nnr1(self) -> int:
        return self.kr[0] * self.kr[1] * self.kr[2]

    def gvec_bohr(self, n: int | None = None) -> np.ndarray:
        """Cartesian G vectors (bohr^-1) of the first ``n`` entries."""
        m = self.mill if n is None else self.mill[:n]
        return m.astype(np.float64) * self.tpiba


def make_basis(alat: float, nr, ecut: float, dual: float = 4.0) -> Basis:
    nr1, nr2, nr3 = (int(nr), int(nr), int(nr)) if np.isscalar(nr) else tuple(int(x) for x in nr)
    tpiba = 2.0 * math.pi / alat
    tpiba2 = tpiba * tpiba
    gcutw = ecut / tpiba2
    gcut = gcutw * dual
    rmax = int(math.floor(math.sqrt(gcut))) + 1
    # The loop runs over the whole mesh box in the reference; restricting it to
    # the bounding box of the density sphere keeps the same acceptance order.
    imax = min(nr1 - 1, rmax)
    jr = np.arange(max(-nr2 + 1, -rmax), min(nr2 - 1, rmax) + 1)
    kr_ = np.arange(max(-nr3 + 1, -rmax), min(nr3 - 1, rmax) + 1)
    pts = []
    for i in range(0, imax + 1):
        J, K = np.meshgrid(jr, kr_, indexing="ij")
        J = J.ravel()
        K = K.ravel()
        if i == 0:
            keep = (J > 0) | ((J == 0) & (K >= 0))
            J = J[keep]
            K = K[keep]
        g2 = float(i * i) + (J * J + K * K).astype(np.float64)
        acc = g2 < gcut
        if np.any(acc):
            pts.append(np.stack([np.full(acc.sum(), i), J[acc], K[acc]], axis=1))
    mill = np.concatenate(pts, axis=0).astype(np.int64)
    g2 = (mill.astype(np.float64) ** 2).sum(axis=1)
    # generation counter ig is 1-based over accepted points
    ig = np.arange(1, mill.shape[0] + 1, dtype=np.float64)
    sign = np.where(g2 < gcutw, -1.0, 1.0)
    key = g2 * (1.0 + np.sqrt(ig - 1.0) * EPSGX * sign)
    order = np.argsort(key, kind="stable")
    mill = mill[order]
    g2 = g2[order]
    ngw = int((g2 < gcutw).sum())
    nhg = mill.shape[0]
    # every mesh must hold the density sphere without aliasing
    for ax, n in enumerate((nr1, nr2, nr3)):
        if 2 * int(np.abs(mill[:, ax]).max()) + 1 > n:
            raise ValueError(f"mesh {n} along axis {ax} too small for ecut={ecut} Ry, alat={alat}")
    nh = np.array([nr1 // 2 + 1, nr2 // 2 + 1, nr3 // 2 + 1], dtype=np.int64)
    inyh = (mill + nh[None, :]).T.astype(np.int32).copy()
    return Basis(alat=alat, nr=(nr1, nr2, nr3), kr=(leadim(nr1), leadim(nr2), leadim(nr3)),
                 ecut=ecut, tpiba=tpiba, tpiba2=tpiba2, omega=alat ** 3,
                 ngw=ngw, nhg=nhg, inyh=inyh, mill=mill.astype(np.int32), hg=g2.copy(),
                 geq0=bool(g2[0] < 1e-5))
