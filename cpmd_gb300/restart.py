"""RESTART wavefunction files of the Gamma point, through the C ABI
(``gbcp_restart_write`` / ``gbcp_restart_read``).

``write_restart`` mirrors the reference's zhwwf/wv30 (wv30_utils.mod.F90:99-233,
235-1300) and ``read_restart`` its zhrwf/rv30 (rv30_utils.mod.F90:104-2242) for
the records the wavefunction path needs: sections 1-8 (header, cell, species,
coordinates, velocities, initial coordinates, cutoff/electrons/mesh, state and
plane-wave counts), section 9, the states C0 in the w_wfnio layout
(wfnio_utils.mod.F90:52-233; compress.F90 for icompr 1 = FP64 and 2 = 32-bit),
section 10, the wavefunction velocities cm of CP dynamics (wr30wfn_utils.mod.F90:
569-693), and sections 23-24, the occupation numbers, Fermi energy and eigenvalues.
The coefficients are stored in the reference's global G order, which is the
order ``cell.make_basis`` generates, so a state column maps row for row onto a
context's basis.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


@dataclass
class RestartData:
    """The contents of sections 1-10, 23 and 24 of a RESTART file."""
    c0: np.ndarray | None                 # (ngw, nstate_read) complex128, column-major
    na: np.ndarray                        # atoms per species
    tau0: np.ndarray | None               # (nat, 3), species-major
    taum: np.ndarray | None = None        # (nat, 3) velocities (section 5)
    taui: np.ndarray | None = None        # (nat, 3) initial coordinates (section 6)
    ibrav: int = 0
    indpg: int = 0
    celldm: np.ndarray = field(default_factory=lambda: np.zeros(6))
    ecut: float = 0.0
    cdual: float = 0.0
    dual: bool = False
    nel: int = 0
    nr: tuple = (0, 0, 0)
    nstate: int = 0
    ngwks: int = 0
    ngwls: int = 0
    nhgs: int = 0
    nhgls: int = 0
    icompr: int = 1
    scale: float = 0.0
    nstate_file: int = 0
    sections: int = 0
    f: np.ndarray | None = None           # (nstate) occupation numbers (section 23)
    eigv: np.ndarray | None = None        # (nstate) eigenvalues (section 24)
    amu: float = 0.0                      # Fermi energy (section 24)
    cm: np.ndarray | None = None          # (ngw, n) wavefunction velocities (section 10)

    def has_section(self, k: int) -> bool:
        return bool(self.sections >> (k - 1) & 1)


def _ptr(a):
    return None if a is None else a.ctypes.data


def _check(fn, rc):
    if rc != L.GBCP_OK:
        raise L.GbcpError(fn, rc)


def write_restart(path: str | os.PathLike, c0, *, na, tau0, ecut: float, nel: int, nr, alat: float,
                  taum=None, taui=None, ibrav: int = 1, indpg: int = 0, celldm=None, cdual: float = 4.0,
                  dual: bool = False, ngwls: int = 0, nhgs: int = 0, nhgls: int = 0, icompr: int = 1,
                  f=None, eigv=None, amu: float = 0.0, cm=None) -> None:
    """Write a RESTART file: c0 (ngw, nstate) complex, na per species, tau0 (nat, 3)
    species-major, ecut in Ry, nel electrons, nr the mesh, alat the cubic cell edge
    (celldm(1), unless celldm is given).  icompr 1 stores FP64 as is, 2 as 32-bit
    fixed point on the largest coefficient's modulus.  f (occupations) and eigv
    (eigenvalues, with the Fermi energy amu) fill sections 23 and 24 when given,
    cm (ngw, nstate) the velocities of section 10."""
    lib = L.load()
    c = np.asfortranarray(np.asarray(c0, dtype=np.complex128))
    ngw, nstate = c.shape
    na_ = np.ascontiguousarray(np.asarray(na, dtype=np.int32))
    t0 = np.ascontiguousarray(np.asarray(tau0, dtype=np.float64).reshape(-1, 3))
    tm = None if taum is None else np.ascontiguousarray(np.asarray(taum, dtype=np.float64).reshape(-1, 3))
    ti = None if taui is None else np.ascontiguousarray(np.asarray(taui, dtype=np.float64).reshape(-1, 3))
    if int(na_.sum()) != t0.shape[0]:
        raise ValueError("sum(na) must equal the number of rows of tau0")
    r = L.Restart()
    r.ibrav, r.indpg = ibrav, indpg
    cd = np.zeros(6) if celldm is None else np.asarray(celldm, dtype=np.float64)
    if celldm is None:
        cd[0], cd[1], cd[2] = alat, 1.0, 1.0
    for i in range(6):
        r.celldm[i] = float(cd[i])
    r.nsp, r.nat = len(na_), t0.shape[0]
    r.na, r.tau0, r.taum, r.taui = _ptr(na_), _ptr(t0), _ptr(tm), _ptr(ti)
    r.ecut, r.cdual, r.dual, r.nel = float(ecut), float(cdual), int(bool(dual)), int(nel)
    nr1, nr2, nr3 = (nr, nr, nr) if np.isscalar(nr) else tuple(nr)
    r.nr1s, r.nr2s, r.nr3s = int(nr1), int(nr2), int(nr3)
    r.nstate, r.nkpts = nstate, 0
    r.ngwks, r.ngwls, r.nhgs, r.nhgls = ngw, int(ngwls), int(nhgs), int(nhgls)
    r.c0, r.ldc, r.ngw, r.icompr = _ptr(c), ngw, ngw, int(icompr)
    f_ = None if f is None else np.ascontiguousarray(np.asarray(f, dtype=np.float64))
    e_ = None if eigv is None else np.ascontiguousarray(np.asarray(eigv, dtype=np.float64))
    for a in (f_, e_):
        if a is not None and a.size != nstate:
            raise ValueError("f and eigv need one entry per state")
    r.f, r.eigv, r.amu = _ptr(f_), _ptr(e_), float(amu)
    cm_ = None if cm is None else np.asfortranarray(np.asarray(cm, dtype=np.complex128))
    if cm_ is not None and cm_.shape != c.shape:
        raise ValueError("cm must have the shape of c0")
    r.cm = _ptr(cm_)
    _check("gbcp_restart_write", lib.gbcp_restart_write(os.fsencode(os.fspath(path)), C.byref(r)))


def read_restart(path: str | os.PathLike, ngw: int | None = None, nstate: int | None = None) -> RestartData:
    """Read sections 1-10, 23 and 24.  ngw: rows of the returned states (default: the file's
    plane waves; more rows are zero, fewer truncate); nstate: states to read
    (default: all of the file's)."""
    lib = L.load()
    p = os.fsencode(os.fspath(path))
    r = L.Restart()
    _check("gbcp_restart_read", lib.gbcp_restart_read(p, C.byref(r)))  # sizes
    na = np.zeros(max(r.nsp, 1), np.int32)
    tau0 = np.zeros((max(r.nat, 1), 3))
    taum = np.zeros((max(r.nat, 1), 3))
    taui = np.zeros((max(r.nat, 1), 3))
    ng = int(r.ngwks if ngw is None else ngw)
    ns = int(r.nstate_file if nstate is None else min(nstate, r.nstate_file))
    c0 = np.zeros((max(ng, 1), max(ns, 1)), dtype=np.complex128, order="F")
    occ = np.zeros(max(r.nstate, 1))
    eig = np.zeros(max(r.nstate, 1))
    r2 = L.Restart()
    r2.na, r2.tau0, r2.taum, r2.taui = _ptr(na), _ptr(tau0), _ptr(taum), _ptr(taui)
    r2.f, r2.eigv = _ptr(occ), _ptr(eig)
    cmv = np.zeros_like(c0)
    if ng > 0 and ns > 0:
        r2.c0, r2.ldc, r2.ngw, r2.nstate_cap = _ptr(c0), c0.shape[0], ng, ns
        r2.cm = _ptr(cmv)
    _check("gbcp_restart_read", lib.gbcp_restart_read(p, C.byref(r2)))
    sec = r2.sections
    nat = r2.nat
    return RestartData(
        c0=c0[:ng, :r2.nstate_read] if r2.nstate_read else None, na=na[:r2.nsp].copy(),
        tau0=tau0[:nat].copy() if sec >> 3 & 1 else None,
        taum=taum[:nat].copy() if sec >> 4 & 1 else None,
        taui=taui[:nat].copy() if sec >> 5 & 1 else None,
        ibrav=r2.ibrav, indpg=r2.indpg, celldm=np.array(list(r2.celldm)), ecut=r2.ecut, cdual=r2.cdual,
        dual=bool(r2.dual), nel=r2.nel, nr=(r2.nr1s, r2.nr2s, r2.nr3s), nstate=r2.nstate, ngwks=r2.ngwks,
        ngwls=r2.ngwls, nhgs=r2.nhgs, nhgls=r2.nhgls, icompr=r2.icompr, scale=r2.scale,
        nstate_file=r2.nstate_file, sections=sec,
        f=occ[:r2.nstate].copy() if sec >> 22 & 1 else None,
        eigv=eig[:r2.nstate].copy() if sec >> 23 & 1 else None, amu=r2.amu,
        cm=cmv[:ng, :r2.ncm_read] if r2.ncm_read else None)
