"""Seeded synthetic Γ-point cells used by the tests and the benchmark.

A cell is a cubic diamond supercell (8-atom conventional basis), optionally
jittered, with:

* psi(G) = (N(0,1) + i N(0,1)) * exp(-|G|^2/4) on the wavefunction half sphere,
  Im psi(G=0) = 0, then orthonormalised (Cholesky Gram-Schmidt in the Γ
  inner product <a|b> = 2 Re sum a*b - a0 b0, see dotp_utils.mod.F90:45-52);
* V_loc(r) = sum_atoms -4 exp(-|r-R|^2 / 1.0) on the mesh, minimum image,
  stored in the reference's padded layout (kr1, kr2, kr3), x fastest;
* f_i = 2 (doubly occupied);
* optional Kleinman-Bylander-like projectors: 8 per atom, two Gaussian radial
  channels times {s, p_x, p_y, p_z} (real spherical harmonics), eigr =
  exp(-i G.R) (phfac_utils.mod.F90:126-195), weights wsg from the seed.

The orthonormalisation here prepares inputs only; it is not part of any
measured path.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .cell import Basis, make_basis

DIAMOND = np.array([
    [0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0],
    [0.25, 0.25, 0.25], [0.25, 0.75, 0.75], [0.75, 0.25, 0.75], [0.75, 0.75, 0.25],
])

# configurations of the wavefunction hot path: edge of the 8-atom diamond
# cell (the supercell edge is alat * rep), supercell repeat, states, cut-off
# (Ry), mesh, jitter (bohr)
CONFIGS = {
    "c0": dict(alat=10.26, rep=1, nstate=16, ecut=20.0, nr=32, jitter=0.0),     # L = 10.26
    "c1": dict(alat=10.26, rep=2, nstate=128, ecut=70.0, nr=120, jitter=0.05),  # L = 20.52
    "c2": dict(alat=10.26, rep=3, nstate=432, ecut=50.0, nr=144, jitter=0.1),   # L = 30.78
    "c4": dict(alat=10.26, rep=4, nstate=1024, ecut=70.0, nr=240, jitter=0.05, nproj=8),  # L = 41.04
}


@dataclass
class Cell:
    basis: Basis
    tau: np.ndarray            # (nat, 3) bohr
    c0: np.ndarray             # complex128 (ngw, nstate), Fortran order
    f: np.ndarray              # (nstate,)
    vpot: np.ndarray           # float64 padded real-space array (kr3, kr2, kr1) C-order == Fortran (kr1,kr2,kr3)
    seed: int
    proj: dict = field(default_factory=dict)

    @property
    def nstate(self) -> int:
        return self.c0.shape[1]


def gamma_overlap(c: np.ndarray, geq0: bool = True) -> np.ndarray:
    """S = 2 Re(C^H C) - Re c(0) Re c(0)^T (rgs_utils.mod.F90:63-68)."""
    s = 2.0 * (c.real.T @ c.real + c.imag.T @ c.imag)
    if geq0:
        s -= np.outer(c[0].real, c[0].real)
    return s


def orthonormalise(c: np.ndarray, geq0: bool = True) -> np.ndarray:
    s = gamma_overlap(c, geq0)
    u = np.linalg.cholesky(s).T          # S = U^T U
    c = c @ np.linalg.inv(u)
    if geq0:
        c[0] = c[0].real
    return c


def atoms(alat8: float, rep: int, jitter: float, rng) -> tuple[np.ndarray, float]:
    alat = alat8 * rep
    pos = []
    for a in range(rep):
        for b in range(rep):
            for c in range(rep):
                pos.append((DIAMOND + np.array([a, b, c])) * alat8)
    tau = np.concatenate(pos, axis=0)
    if jitter > 0:
        tau = tau + rng.uniform(-jitter, jitter, size=tau.shape)
    return tau, alat


def vloc_grid(basis: Basis, tau: np.ndarray, amp: float = -4.0, width2: float = 1.0) -> np.ndarray:
    """Gaussian local potential on the mesh, padded layout (kr3, kr2, kr1)."""
    n1, n2, n3 = basis.nr
    k1, k2, k3 = basis.kr
    L = basis.alat
    x = np.arange(n1) * (L / n1)
    y = np.arange(n2) * (L / n2)
    z = np.arange(n3) * (L / n3)
    v = np.zeros((n3, n2, n1))
    for R in tau:
        dx = x - R[0]
        dy = y - R[1]
        dz = z - R[2]
        dx -= L * np.round(dx / L)
        dy -= L * np.round(dy / L)
        dz -= L * np.round(dz / L)
        ex = np.exp(-dx * dx / width2)
        ey = np.exp(-dy * dy / width2)
        ez = np.exp(-dz * dz / width2)
        v += amp * ez[:, None, None] * ey[None, :, None] * ex[None, None, :]
    out = np.zeros((k3, k2, k1))
    out[:n3, :n2, :n1] = v
    return out


def random_states(basis: Basis, nstate: int, rng) -> np.ndarray:
    ngw = basis.ngw
    g2 = basis.hg[:ngw] * basis.tpiba2
    amp = np.exp(-g2 / 4.0)
    c = (rng.standard_normal((ngw, nstate)) + 1j * rng.standard_normal((ngw, nstate))) * amp[:, None]
    if basis.geq0:
        c[0] = c[0].real
    return np.asfortranarray(orthonormalise(c, basis.geq0))


def projectors(basis: Basis, tau: np.ndarray, rng, sigmas=(0.8, 1.4)) -> dict:
    """8 projectors per atom: 2 Gaussian radial channels x {s, p_x, p_y, p_z}."""
    ngw = basis.ngw
    G = basis.gvec_bohr(ngw)
    gn = np.sqrt((G * G).sum(axis=1))
    twnl = np.zeros((ngw, 8))
    nghtol = np.zeros(8, dtype=np.int32)
    ys = 1.0 / np.sqrt(4 * np.pi)
    yp = np.sqrt(3.0 / (4 * np.pi))
    iv = 0
    for sg in sigmas:
        rad = np.exp(-0.5 * (gn * sg) ** 2)
        twnl[:, iv] = rad * ys
        nghtol[iv] = 0
        iv += 1
        for ax in range(3):
            twnl[:, iv] = rad * yp * G[:, ax] * sg  # |G| Y_1m = sqrt(3/4pi) G_ax
            nghtol[iv] = 1
            iv += 1
    phase = G @ tau.T                                   # (ngw, nat)
    eigr = np.asfortranarray(np.exp(-1j * phase))       # e^{-i G.R}
    wsg = rng.uniform(0.5, 1.5, size=8)
    return dict(twnl=np.asfortranarray(twnl), nghtol=nghtol, eigr=eigr, wsg=wsg)


def make_cell(name: str = "c0", seed: int = 1234, nstate: int | None = None,
              with_proj: bool | None = None) -> Cell:
    cfg = CONFIGS[name]
    rng = np.random.default_rng(seed)
    tau, alat = atoms(cfg["alat"], cfg["rep"], cfg["jitter"], rng)
    basis = make_basis(alat, cfg["nr"], cfg["ecut"])
    ns = cfg["nstate"] if nstate is None else nstate
    c0 = random_states(basis, ns, rng)
    v = vloc_grid(basis, tau)
    f = np.full(ns, 2.0)
    proj = {}
    if (with_proj is None and cfg.get("nproj")) or with_proj:
        proj = projectors(basis, tau, rng)
    return Cell(basis=basis, tau=tau, c0=c0, f=f, vpot=v, seed=seed, proj=proj)


def make_small_cell(alat: float, nr: int, ecut: float, nstate: int, seed: int = 7,
                    nat_rep: int = 1, jitter: float = 0.0, with_proj: bool = False) -> Cell:
    """A cell of arbitrary size for edge-case tests (odd state counts, tiny meshes)."""
    rng = np.random.default_rng(seed)
    tau, _ = atoms(alat / nat_rep, nat_rep, jitter, rng)
    basis = make_basis(alat, nr, ecut)
    c0 = random_states(basis, nstate, rng)
    v = vloc_grid(basis, tau)
    f = np.full(nstate, 2.0)
    proj = projectors(basis, tau, rng) if with_proj else {}
    return Cell(basis=basis, tau=tau, c0=c0, f=f, vpot=v, seed=seed, proj=proj)


def gaussian_form_factor(basis: Basis, amp: float = -4.0, width2: float = 1.0) -> np.ndarray:
    """vps(G) over the density half sphere for v(r) = amp exp(-r^2/width2):
    amp (pi width2)^(3/2) exp(-width2 G^2 / 4) / Omega, so that
    V_ion(G) = sum_a vps(G) e^{-iG.R_a} is the periodic sum of the Gaussians."""
    g2 = basis.hg * basis.tpiba2
    return amp * (np.pi * width2) ** 1.5 * np.exp(-width2 * g2 / 4.0) / basis.omega


@dataclass
class DeviceCell:
    """The same construction as :class:`Cell`, generated on the GPU with torch
    (torch's generator instead of numpy's, same distributions); arrays are torch
    tensors in the device layouts of the API: c0 (nstate, ngw), vpot (kr3, kr2, kr1),
    twnl (ngh, ngw), eigr (nat, ngw)."""
    basis: Basis
    tau: np.ndarray
    c0: object
    f: object
    vpot: object
    seed: int
    proj: dict = field(default_factory=dict)

    @property
    def nstate(self) -> int:
        return int(self.c0.shape[0])


def make_cell_device(name: str, seed: int = 1234, nstate: int | None = None, with_proj: bool | None = None,
                     ctx=None) -> DeviceCell:
    """Large cells without host-side O(n^2 ngw) work: psi orthonormalised on the
    device by the library's own FP64 Gram-Schmidt (two passes), V_loc and the
    projectors evaluated on the device."""
    import torch
    from .api import Context
    cfg = CONFIGS[name]
    rng = np.random.default_rng(seed)
    tau, alat = atoms(cfg["alat"], cfg["rep"], cfg["jitter"], rng)
    basis = make_basis(alat, cfg["nr"], cfg["ecut"])
    ns = cfg["nstate"] if nstate is None else nstate
    dev = torch.device("cuda")
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    ngw = basis.ngw
    g2 = torch.from_numpy(basis.hg[:ngw] * basis.tpiba2).to(dev)
    amp = torch.exp(-g2 / 4.0)
    re = torch.randn((ns, ngw), generator=gen, device=dev, dtype=torch.float64)
    im = torch.randn((ns, ngw), generator=gen, device=dev, dtype=torch.float64)
    c0 = torch.complex(re * amp, im * amp)
    if basis.geq0:
        c0[:, 0] = c0[:, 0].real.to(torch.complex128)
    own = ctx is None
    ctx = ctx or Context(basis, "fp64")
    ctx.ortho(c0, "gs")
    ctx.ortho(c0, "gs")
    torch.cuda.synchronize()
    if own:
        ctx.close()
    # V_loc: separable Gaussians, minimum image
    n1, n2, n3 = basis.nr
    k1, k2, k3 = basis.kr
    L = basis.alat
    v = torch.zeros((n3, n2, n1), dtype=torch.float64, device=dev)
    ax = [torch.arange(n, dtype=torch.float64, device=dev) * (L / n) for n in (n1, n2, n3)]
    for R in tau:
        e = []
        for d in range(3):
            dd = ax[d] - float(R[d])
            dd = dd - L * torch.round(dd / L)
            e.append(torch.exp(-dd * dd))
        v += -4.0 * e[2][:, None, None] * e[1][None, :, None] * e[0][None, None, :]
    vpot = torch.zeros((k3, k2, k1), dtype=torch.float64, device=dev)
    vpot[:n3, :n2, :n1] = v
    f = torch.full((ns,), 2.0, dtype=torch.float64, device=dev)
    proj = {}
    if (with_proj is None and cfg.get("nproj")) or with_proj:
        G = torch.from_numpy(basis.gvec_bohr(ngw)).to(dev)
        gn = torch.sqrt((G * G).sum(dim=1))
        twnl = torch.zeros((8, ngw), dtype=torch.float64, device=dev)
        nghtol = np.zeros(8, dtype=np.int32)
        ys = 1.0 / np.sqrt(4 * np.pi)
        yp = np.sqrt(3.0 / (4 * np.pi))
        iv = 0
        for sg in (0.8, 1.4):
            rad = torch.exp(-0.5 * (gn * sg) ** 2)
            twnl[iv] = rad * ys
            iv += 1
            for a in range(3):
                twnl[iv] = rad * yp * G[:, a] * sg
                nghtol[iv] = 1
                iv += 1
        t = torch.from_numpy(tau).to(dev)
        eigr = torch.exp(-1j * (t @ G.T))                     # (nat, ngw) == Fortran eigr(ngw, nat)
        proj = dict(twnl=twnl, nghtol=nghtol, eigr=eigr,
                    wsg=torch.from_numpy(rng.uniform(0.5, 1.5, size=8)).to(dev))
    return DeviceCell(basis=basis, tau=tau, c0=c0, f=f, vpot=vpot, seed=seed, proj=proj)


MESHES = (32, 36, 40, 48, 60, 64, 72, 80, 96, 120, 144, 240)


def batch_cell(nat: int, seed: int, ecut: float = 30.0, alat8: float = 10.26) -> Cell:
    """One cell of the many-cell batch: nat atoms at seeded uniform positions in a
    cube of edge alat8 (nat/8)^(1/3) (the 8-atom cell's density), 2 nat doubly
    occupied states, the smallest planned mesh that holds the density sphere."""
    rng = np.random.default_rng(seed)
    L = alat8 * (nat / 8.0) ** (1.0 / 3.0)
    basis = None
    for m in MESHES:
        try:
            basis = make_basis(L, m, ecut)
            break
        except ValueError:
            continue
    if basis is None:
        raise ValueError("no planned mesh holds the density sphere")
    tau = rng.uniform(0.0, L, size=(nat, 3))
    ns = 2 * nat
    c0 = random_states(basis, ns, rng)
    return Cell(basis=basis, tau=tau, c0=c0, f=np.full(ns, 2.0), vpot=vloc_grid(basis, tau), seed=seed)


def make_batch(ncells: int = 64, seed: int = 4321, atoms_choice=(8, 16, 32, 64)) -> list:
    """ncells independent cells, atom counts drawn uniformly from atoms_choice."""
    rng = np.random.default_rng(seed)
    nats = rng.choice(np.asarray(atoms_choice), size=ncells)
    return [batch_cell(int(n), seed + 1 + i) for i, n in enumerate(nats)]
