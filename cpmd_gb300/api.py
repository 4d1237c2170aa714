"""Host-side mirror of CPMD's Fortran entry points over the GB300 C ABI.

The reference routines take their grid and basis from module globals; here a
:class:`Context` holds them (one ``gbcp_ctx``), and each method is the routine
of the same name:

=================  =========================================  ==============================
method             reference routine                          file:line
=================  =========================================  ==============================
``rhoofr``         rhoofr(c0, rhoe, psi, nstate)              rhoofr_utils.mod.F90:122
``vpsi``           vpsi(c0, c2, f, vpot, psi, nstate, ...)    vpsi_utils.mod.F90:120
``ortho``          ortho(nstate, c0, cscr)                    ortho_utils.mod.F90:124
``ovlap``          ovlap(nstate, a, c1, c2) (c1 == c2)         ovlap_utils.mod.F90:57
``invfftn``        invfftn(f, sparse=.FALSE., ...)            fftmain_utils.mod.F90:373
``fwfftn``         fwfftn(f, sparse=.FALSE., ...)             fftmain_utils.mod.F90:403
``rnlsm``          rnlsm(c0, nstate, ...) -> rnlsm1           rnlsm_utils.mod.F90:23
``fnonloc``        fnonloc(c2, f, nstate, ...)                fnonloc_utils.mod.F90:55
=================  =========================================  ==============================

Arrays may be numpy arrays (host memory; the call stages them and
synchronises) or torch CUDA tensors (device memory; the call is queued on the
context's stream).  Layouts follow the reference:

* wavefunctions: Fortran ``c0(ngw, nstate)`` complex128 -> numpy
  ``order='F'`` array of shape (ngw, nstate), or a torch tensor of shape
  (nstate, ngw) (row-major), i.e. the same bytes;
* real-space arrays: Fortran ``rhoe(kr1, kr2, kr3)`` -> numpy / torch array
  of shape (kr3, kr2, kr1);
* fnl: Fortran ``fnl(nat, ngh, nstate)`` -> shape (nstate, ngh, nat).

Errors raise :class:`GbcpError` (the reference aborts via stopgm).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import MEM_DEVICE, MEM_HOST, ORTHO, PREC, GbcpError

# gbcp_set_option keys: GBCP_OPT_<NAME> of include/cpmd_gb300.h, by lower-case name
OPTIONS = {"gemm": 1, "batch": 2, "fft": 3, "xchunks": 4, "xc": 5, "wfn_cache": 6, "plane": 7, "chol": 8,
           "simt_tile": 9, "stages": 10, "zmirror": 11, "zkeep": 12, "ortho_columns": 13, "test_timeout": 90}


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(x):
    if x is None:
        return None
    if _is_torch(x):
        if not x.is_cuda:
            raise ValueError("torch tensors must live on a CUDA device (use numpy for host arrays)")
        if not x.is_contiguous():
            raise ValueError("torch tensors must be contiguous")
        return C.c_void_p(x.data_ptr())
    if not (x.flags["F_CONTIGUOUS"] or x.flags["C_CONTIGUOUS"]):
        # column-major wavefunction views with a leading dimension are allowed
        if not (x.ndim == 2 and x.strides[0] == x.itemsize):
            raise ValueError("numpy arrays must be contiguous")
    return C.c_void_p(x.ctypes.data)


def _mem(*arrs) -> int:
    kinds = {(_is_torch(a)) for a in arrs if a is not None}
    if len(kinds) != 1:
        raise ValueError("all array arguments of one call must be either numpy (host) or torch CUDA (device)")
    return MEM_DEVICE if kinds.pop() else MEM_HOST


def _ld_wfn(c, ngw: int, allow_c64: bool = False) -> tuple[int, int]:
    """(leading dimension, nstate) of a wavefunction array (complex64 tensors only
    where allow_c64: the batch's complex64 storage)."""
    if _is_torch(c):
        if c.dim() != 2:
            raise ValueError("wavefunction tensor must be (nstate, ngw)")
        import torch
        if c.dtype != torch.complex128 and not (allow_c64 and c.dtype == torch.complex64):
            raise ValueError("wavefunctions are complex128")
        return int(c.shape[1]), int(c.shape[0])
    if c.dtype != np.complex128 or c.ndim != 2:
        raise ValueError("wavefunctions are complex128 (ngw, nstate)")
    if c.shape[0] < ngw:
        raise ValueError(f"wavefunction leading dimension {c.shape[0]} < ngw {ngw}")
    # Fortran column-major, possibly a leading-dimension view c(1:ngw, :) of a larger array
    if c.shape[1] > 1 and (c.strides[0] != 16 or c.strides[1] % 16 != 0):
        raise ValueError("numpy wavefunctions must be column-major (ngw, nstate)")
    ld = c.strides[1] // 16 if c.shape[1] > 1 else c.shape[0]
    return int(ld), int(c.shape[1])


class Context:
    """One drop-in context: grid + basis + precision + stream."""

    def __init__(self, basis, precision: str = "fp64", batch: int = 0, stream=None):
        self.lib = _lib.load()
        self.basis = basis
        self.ngw = basis.ngw
        self.kr = tuple(basis.kr)
        self.nr = tuple(basis.nr)
        self._inyh = np.ascontiguousarray(basis.inyh[:, : basis.ngw].T.astype(np.int32))  # (ngw, 3) == Fortran (3, ngw)
        self._hg = np.ascontiguousarray(basis.hg[: basis.ngw], dtype=np.float64)
        g = _lib.GridDesc()
        g.nr1, g.nr2, g.nr3 = basis.nr
        g.kr1, g.kr2, g.kr3 = basis.kr
        g.ngw = basis.ngw
        g.geq0 = 1 if basis.geq0 else 0
        g.omega = basis.omega
        g.tpiba2 = basis.tpiba2
        g.inyh = self._inyh.ctypes.data_as(C.POINTER(C.c_int32))
        g.hg = self._hg.ctypes.data_as(C.POINTER(C.c_double))
        h = C.c_void_p()
        st = C.c_void_p(stream) if stream is not None else None
        rc = self.lib.gbcp_ctx_create(C.byref(g), PREC[precision], int(batch), st, C.byref(h))
        if rc != 0:
            raise GbcpError("gbcp_ctx_create", rc)
        self.h = h
        self.precision = precision

    # -- housekeeping --------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.gbcp_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_precision(self, precision: str):
        self._check("gbcp_set_precision", self.lib.gbcp_set_precision(self.h, PREC[precision]))
        self.precision = precision

    def set_option(self, key: str, value: int):
        """key: a name of OPTIONS (GBCP_OPT_<NAME> of the C header, lower case), e.g.
        'gemm' (-1 by precision, 0 FP64 SIMT, 1 tensor cores), 'batch' (pairs per
        launch), 'fft' (0 four-step, 2 Stockham), 'xc' (0 LDA-PZ, 1 PBE), 'wfn_cache',
        'zkeep', 'ortho_columns'; the values are those the header documents."""
        self._check("gbcp_set_option", self.lib.gbcp_set_option(self.h, OPTIONS[key], int(value)))

    def synchronize(self):
        self._check("gbcp_synchronize", self.lib.gbcp_synchronize(self.h))

    def last_error(self) -> str:
        buf = C.create_string_buffer(512)
        self.lib.gbcp_last_error(self.h, buf, 512)
        return buf.value.decode(errors="replace")

    def profile(self, enable: bool = True):
        """Start (clear) or stop the per-kernel CUDA-event timers."""
        self._check("gbcp_profile_enable", self.lib.gbcp_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        """{kernel name: (total ms, launches)} since the last profile(True)."""
        out = {}
        i = 0
        buf = C.create_string_buffer(128)
        ms = C.c_double()
        n = C.c_int64()
        while self.lib.gbcp_profile_read(self.h, i, buf, 128, C.byref(ms), C.byref(n)) == 0:
            out[buf.value.decode()] = (ms.value, int(n.value))
            i += 1
        return out

    def profile_timeline(self) -> list:
        """[(name, lane, start ms, end ms)] since the last profile(True); lane 0 is the
        context stream, 1 host->device staging copies, 2 device->host copies."""
        out = []
        i = 0
        buf = C.create_string_buffer(128)
        lane = C.c_int()
        t0 = C.c_double()
        t1 = C.c_double()
        while self.lib.gbcp_profile_timeline(self.h, i, buf, 128, C.byref(lane), C.byref(t0), C.byref(t1)) == 0:
            out.append((buf.value.decode(), lane.value, t0.value, t1.value))
            i += 1
        return out

    def _check(self, fn: str, rc: int):
        if rc != 0:
            raise GbcpError(fn, rc, self.last_error())

    def _prep(self, *arrs) -> int:
        """Memory kind of a call; device calls are queued on torch's current
        stream so they order with the caller's torch work."""
        mem = _mem(*arrs)
        if mem == MEM_DEVICE:
            import torch
            # handle 0 is the legacy default stream: pass cudaStreamLegacy (0x1)
            s = torch.cuda.current_stream().cuda_stream or 1
        else:
            s = None
        self._check("gbcp_set_stream", self.lib.gbcp_set_stream(self.h, C.c_void_p(s) if s else None))
        return mem

    # -- hot path ------------------------------------------------------------
    def rhoofr(self, c0, f, rhoe=None, energies: bool = True):
        """Density (padded layout) and, if ``energies``, (ekin, csumg, csumr)."""
        ldc, n = _ld_wfn(c0, self.ngw)
        if rhoe is None:
            if _is_torch(c0):
                import torch
                rhoe = torch.empty(self.kr[::-1], dtype=torch.float64, device=c0.device)
            else:
                rhoe = np.empty(self.kr[::-1])
        mem = self._prep(c0, f, rhoe)
        ek, cg, cr = C.c_double(), C.c_double(), C.c_double()
        refs = (C.byref(ek), C.byref(cg), C.byref(cr)) if energies else (None, None, None)
        self._check("gbcp_rhoofr", self.lib.gbcp_rhoofr(self.h, _ptr(c0), ldc, n, _ptr(f), _ptr(rhoe), *refs, mem))
        if energies:
            return rhoe, ek.value, cg.value, cr.value
        return rhoe

    def vpsi(self, c0, c2, f, vpot):
        """c2 += -f (1/2 G^2 c0 + [V psi](G)); returns c2."""
        ldc, n = _ld_wfn(c0, self.ngw)
        ld2, n2 = _ld_wfn(c2, self.ngw)
        if n2 != n:
            raise ValueError("c0 and c2 state counts differ")
        mem = self._prep(c0, c2, f, vpot)
        self._check("gbcp_vpsi", self.lib.gbcp_vpsi(self.h, _ptr(c0), ldc, _ptr(c2), ld2, _ptr(f), _ptr(vpot), n, mem))
        return c2

    def ortho(self, c0, method: str = "gs"):
        """Orthonormalise c0 in place; returns scond = max|S - I| of the input."""
        ldc, n = _ld_wfn(c0, self.ngw)
        sc = C.c_double()
        self._check("gbcp_ortho", self.lib.gbcp_ortho(self.h, _ptr(c0), ldc, n, ORTHO[method], C.byref(sc), self._prep(c0)))
        return sc.value

    def ovlap(self, c0, smat=None):
        ldc, n = _ld_wfn(c0, self.ngw)
        if smat is None:
            if _is_torch(c0):
                import torch
                smat = torch.empty((n, n), dtype=torch.float64, device=c0.device)
            else:
                smat = np.empty((n, n))
        self._check("gbcp_ovlap", self.lib.gbcp_ovlap(self.h, _ptr(c0), ldc, n, _ptr(smat), self._prep(c0, smat)))
        return smat

    def ovlap2(self, c1, c2, amat=None):
        """a(i, j) = <c1_i|c2_j> in the Γ metric (the reference's ovlap with c1 != c2),
        returned column-major like a(nstate, nstate): a torch tensor / numpy array whose
        element [j, i] is a(i, j)."""
        ld1, n = _ld_wfn(c1, self.ngw)
        ld2, n2 = _ld_wfn(c2, self.ngw)
        if n2 != n:
            raise ValueError("c1 and c2 hold different numbers of states")
        if amat is None:
            if _is_torch(c1):
                import torch
                amat = torch.empty((n, n), dtype=torch.float64, device=c1.device)
            else:
                amat = np.empty((n, n))
        self._check("gbcp_ovlap2", self.lib.gbcp_ovlap2(self.h, _ptr(c1), ld1, _ptr(c2), ld2, n, _ptr(amat),
                                                        self._prep(c1, c2, amat)))
        return amat

    def rortog(self, c0, cm, tnon: bool = False, epsog: float = 1e-6, maxit: int = 30):
        """CP-dynamics orthonormality constraint (rortog -> rortho): updates cm in place
        to cm + c0 gam and returns (gam, iterations); gam is symmetric (nstate x nstate)."""
        ldc0, n = _ld_wfn(c0, self.ngw)
        ldcm, n2 = _ld_wfn(cm, self.ngw)
        if n2 != n:
            raise ValueError("c0 and cm hold different numbers of states")
        if _is_torch(cm):
            import torch
            gam = torch.empty((n, n), dtype=torch.float64, device=cm.device)
        else:
            gam = np.empty((n, n))
        it = C.c_int(0)
        self._check("gbcp_rortog", self.lib.gbcp_rortog(self.h, _ptr(c0), ldc0, _ptr(cm), ldcm, n, int(bool(tnon)),
                                                       float(epsog), int(maxit), _ptr(gam), C.byref(it),
                                                       self._prep(c0, cm, gam)))
        return gam, it.value

    def invfftn(self, grid):
        """In-place inverse 3D FFT of a complex grid shaped (nr3, kr2, kr1)."""
        self._check("gbcp_invfftn", self.lib.gbcp_invfftn(self.h, _ptr(grid), self._prep(grid)))
        return grid

    def fwfftn(self, grid):
        self._check("gbcp_fwfftn", self.lib.gbcp_fwfftn(self.h, _ptr(grid), self._prep(grid)))
        return grid

    @staticmethod
    def _fnl_block(arr, isa0):
        """(pointer, ld_atoms, ld_proj) of a species block: the whole dense array when
        isa0 is None, else the block at atom isa0 of a global array shaped like the
        reference's fnl(nat_total, nhxs, nstate) -> (nstate, nhxs, nat_total) (dfnl:
        (nstate, 3, nhxs, nat_total)), written or read in place."""
        if isa0 is None:
            return _ptr(arr), 0, 0
        base = _ptr(arr)
        return C.c_void_p(base.value + 8 * int(isa0)), int(arr.shape[-1]), int(arr.shape[-2])

    def rnlsm(self, c0, twnl, eigr, nghtol, fnl=None, isa0=None):
        """fnl (nstate, ngh, nat) == Fortran fnl(nat, ngh, nstate); with ``isa0`` the
        species block of a global (nstate, nhxs, nat_total) array at atom isa0."""
        ldc, n = _ld_wfn(c0, self.ngw)
        ngh = int(len(nghtol))
        nat = int(eigr.shape[1] if not _is_torch(eigr) else eigr.shape[0])
        nt = np.ascontiguousarray(np.asarray(nghtol, dtype=np.int32))
        if fnl is None:
            if _is_torch(c0):
                import torch
                fnl = torch.empty((n, ngh, nat), dtype=torch.float64, device=c0.device)
            else:
                fnl = np.empty((n, ngh, nat))
        mem = self._prep(c0, twnl, eigr, fnl)
        fp, la, lp = self._fnl_block(fnl, isa0)
        self._check("gbcp_rnlsm1", self.lib.gbcp_rnlsm1(self.h, _ptr(c0), ldc, n, nat, ngh, _ptr(nt), _ptr(twnl),
                                                        _ptr(eigr), fp, la, lp, mem))
        return fnl

    def rnlsm2(self, c0, twnl, eigr, nghtol, dfnl=None, isa0=None):
        """dfnl (nstate, 3, ngh, nat) == Fortran dfnl(nat, ngh, 3, nstate) = d fnl / d R; with
        ``isa0`` the species block of a global (nstate, 3, nhxs, nat_total) array."""
        ldc, n = _ld_wfn(c0, self.ngw)
        ngh = int(len(nghtol))
        nat = int(eigr.shape[1] if not _is_torch(eigr) else eigr.shape[0])
        nt = np.ascontiguousarray(np.asarray(nghtol, dtype=np.int32))
        if dfnl is None:
            if _is_torch(c0):
                import torch
                dfnl = torch.empty((n, 3, ngh, nat), dtype=torch.float64, device=c0.device)
            else:
                dfnl = np.empty((n, 3, ngh, nat))
        mem = self._prep(c0, twnl, eigr, dfnl)
        fp, la, lp = self._fnl_block(dfnl, isa0)
        self._check("gbcp_rnlsm2", self.lib.gbcp_rnlsm2(self.h, _ptr(c0), ldc, n, nat, ngh, _ptr(nt), _ptr(twnl),
                                                        _ptr(eigr), fp, la, lp, mem))
        return dfnl

    def rnlfor(self, f, fnl, dfnl, wsg, fion, nat=None, ngh=None, isa0=None):
        """fion (nat, 3) == Fortran fion(3, nat) -= the non-local forces (accumulated).  With
        ``isa0``, fnl / dfnl are the global arrays and nat, ngh the species block's sizes."""
        n = int(f.shape[0])
        if isa0 is None:
            nat, ngh = int(fnl.shape[2]), int(fnl.shape[1])
        mem = self._prep(f, fnl, dfnl, wsg, fion)
        fp, la, lp = self._fnl_block(fnl, isa0)
        dp, _, _ = self._fnl_block(dfnl, isa0)
        self._check("gbcp_rnlfor", self.lib.gbcp_rnlfor(self.h, n, _ptr(f), nat, ngh, _ptr(wsg), fp, dp, la, lp,
                                                        _ptr(fion), mem))
        return fion

    def fnonloc(self, c2, f, fnl, twnl, eigr, nghtol, wsg, isa0=None):
        """c2 += the non-local term of one species; fnl dense (nstate, ngh, nat) or, with
        ``isa0``, the global (nstate, nhxs, nat_total) array read at atom isa0."""
        ld2, n = _ld_wfn(c2, self.ngw)
        ngh = int(len(nghtol))
        nat = int(eigr.shape[1] if not _is_torch(eigr) else eigr.shape[0])
        nt = np.ascontiguousarray(np.asarray(nghtol, dtype=np.int32))
        mem = self._prep(c2, f, fnl, twnl, eigr, wsg)
        fp, la, lp = self._fnl_block(fnl, isa0)
        self._check("gbcp_fnonloc", self.lib.gbcp_fnonloc(self.h, _ptr(c2), ld2, n, _ptr(f), nat, ngh, _ptr(nt),
                                                          _ptr(twnl), _ptr(eigr), fp, la, lp, _ptr(wsg), mem))
        return c2


    # -- energy functional and its adjoint --------------------------------------
    def _ensure_dens_sphere(self):
        if getattr(self, "_dens_set", False):
            return
        b = self.basis
        inyh = np.ascontiguousarray(b.inyh.T.astype(np.int32))            # (nhg, 3) == Fortran (3, nhg)
        hg = np.ascontiguousarray(b.hg, dtype=np.float64)
        self._check("gbcp_set_dens_sphere",
                    self.lib.gbcp_set_dens_sphere(self.h, int(b.nhg), inyh.ctypes.data_as(C.c_void_p),
                                                  hg.ctypes.data_as(C.c_void_p)))
        self._dens_set = True

    def _species_args(self, tau, vps, isp, dev):
        nhg = int(self.basis.nhg)
        nat = 0 if tau is None else int(tau.shape[0])
        if nat:
            if isp is None:
                isp = np.zeros(nat, dtype=np.int32)
            isp = np.ascontiguousarray(np.asarray(isp, dtype=np.int32))
            nsp = int(isp.max()) + 1
            if dev:
                if vps.dim() == 1:
                    vps = vps.reshape(1, nhg)
                if tuple(vps.shape) != (nsp, nhg):
                    raise ValueError("vps must be (nsp, nhg) on the device")
            else:
                vps = np.asarray(vps, dtype=np.float64).reshape(nhg, -1, order="F")
                if vps.shape[1] != nsp:
                    raise ValueError("vps must be (nhg, nsp)")
                vps = np.asfortranarray(vps)
                tau = np.ascontiguousarray(tau, dtype=np.float64)
            return nat, nsp, isp, vps, tau
        return 0, 1, None, None, None

    def vofrho(self, rhoe, tau=None, vps=None, isp=None, vext=None, forces: bool = True):
        """Density -> potential (vofrho): returns (veff, terms, fion) with veff on the
        padded mesh, terms = {eloc, ehart, exc, eext} and the local-potential forces
        (nat, 3) (None without atoms or with forces=False).  Arguments as in energy()."""
        self._ensure_dens_sphere()
        dev = _is_torch(rhoe)
        nat, nsp, isp, vps, tau = self._species_args(tau, vps, isp, dev)
        if dev:
            import torch
            veff = torch.empty(self.kr[::-1], dtype=torch.float64, device=rhoe.device)
            fion = torch.empty((nat, 3), dtype=torch.float64, device=rhoe.device) if (forces and nat) else None
        else:
            veff = np.empty(self.kr[::-1])
            fion = np.empty((nat, 3)) if (forces and nat) else None
        mem = self._prep(rhoe, tau, vps, vext, veff, fion)
        e = (C.c_double * 4)()
        isp_p = isp.ctypes.data_as(C.c_void_p) if isp is not None else None
        self._check("gbcp_vofrho", self.lib.gbcp_vofrho(self.h, _ptr(rhoe), nat, nsp, isp_p, _ptr(tau), _ptr(vps),
                                                        _ptr(vext), _ptr(veff), e, _ptr(fion), mem))
        return veff, dict(eloc=e[0], ehart=e[1], exc=e[2], eext=e[3]), fion

    def energy(self, c0, f, tau=None, vps=None, isp=None, vext=None, grad: bool = True, forces: bool = True):
        """E[psi, V, R] = E_kin + E_loc + E_H + E_xc (+ E_ext) and its adjoint.

        ``tau``: (nat, 3) == Fortran tau(3, nat); ``vps``: numpy (nhg,) or
        (nhg, nsp) / torch (nhg,) or (nsp, nhg); ``isp``: host ints (nat,);
        ``vext``: padded mesh potential or None.  Returns ``terms`` (dict) and,
        with ``grad``, also (c2, dvloc, fion) -- see include/cpmd_gb300.h.
        """
        self._ensure_dens_sphere()
        ldc, n = _ld_wfn(c0, self.ngw)
        dev = _is_torch(c0)
        nhg = int(self.basis.nhg)
        nat = 0 if tau is None else int(tau.shape[0])
        if nat:
            if isp is None:
                isp = np.zeros(nat, dtype=np.int32)
            isp = np.ascontiguousarray(np.asarray(isp, dtype=np.int32))
            nsp = int(isp.max()) + 1
            if dev:
                if vps.dim() == 1:
                    vps = vps.reshape(1, nhg)
                if tuple(vps.shape) != (nsp, nhg):
                    raise ValueError("vps must be (nsp, nhg) on the device")
            else:
                vps = np.asarray(vps, dtype=np.float64).reshape(nhg, -1, order="F")
                if vps.shape[1] != nsp:
                    raise ValueError("vps must be (nhg, nsp)")
                vps = np.asfortranarray(vps)
                tau = np.ascontiguousarray(tau, dtype=np.float64)
        else:
            nsp, isp, vps, tau = 1, None, None, None
        c2 = dv = fion = None
        if grad:
            if dev:
                import torch
                c2 = torch.empty((n, self.ngw), dtype=torch.complex128, device=c0.device)
                dv = torch.empty(self.kr[::-1], dtype=torch.float64, device=c0.device)
                fion = torch.empty((max(nat, 1), 3), dtype=torch.float64, device=c0.device) if (forces and nat) else None
            else:
                c2 = np.zeros((self.ngw, n), dtype=np.complex128, order="F")
                dv = np.empty(self.kr[::-1])
                fion = np.empty((nat, 3)) if (forces and nat) else None
        mem = self._prep(c0, f, tau, vps, vext, c2, dv, fion)
        e = (C.c_double * 6)()
        isp_p = isp.ctypes.data_as(C.c_void_p) if isp is not None else None
        self._check("gbcp_energy", self.lib.gbcp_energy(
            self.h, _ptr(c0), ldc, n, _ptr(f), nat, nsp, isp_p, _ptr(tau), _ptr(vps), _ptr(vext), e,
            _ptr(c2), self.ngw, _ptr(dv), _ptr(fion), mem))
        terms = dict(etot=e[0], ekin=e[1], eloc=e[2], ehart=e[3], exc=e[4], eext=e[5])
        if grad:
            return terms, c2, dv, fion
        return terms


STEP = {"rhoofr": 1, "vpsi": 2, "ortho": 4, "psi_c64": 8}


def _grid_desc(basis):
    """GridDesc of a basis plus the arrays it points into (keep them alive)."""
    inyh = np.ascontiguousarray(basis.inyh[:, : basis.ngw].T.astype(np.int32))
    hg = np.ascontiguousarray(basis.hg[: basis.ngw], dtype=np.float64)
    g = _lib.GridDesc()
    g.nr1, g.nr2, g.nr3 = basis.nr
    g.kr1, g.kr2, g.kr3 = basis.kr
    g.ngw = basis.ngw
    g.geq0 = 1 if basis.geq0 else 0
    g.omega = basis.omega
    g.tpiba2 = basis.tpiba2
    g.inyh = inyh.ctypes.data_as(C.POINTER(C.c_int32))
    g.hg = hg.ctypes.data_as(C.POINTER(C.c_double))
    return g, (inyh, hg)


class Batch:
    """Many independent cells per step, one CUDA-graph launch (gbcp_batch_*).

    ``cells`` passed to :meth:`tune` / :meth:`step` is a list of dicts with
    torch CUDA tensors ``c0`` (nstate, ngw) complex128 -- or complex64 in a
    mixed-precision batch (GBCP_STEP_PSI_C64, added to the flags by itself) --,
    ``f`` (nstate,), ``vpot`` and ``rhoe`` (kr3, kr2, kr1) float64 and ``c2``
    like ``c0``.  ``flags``: an int or an iterable of "rhoofr", "vpsi", "ortho".
    """

    def __init__(self, bases, precision: str = "mixed", nstreams: int = 8):
        self.lib = _lib.load()
        self.bases = list(bases)
        keep = []
        arr = (_lib.GridDesc * len(self.bases))()
        for i, b in enumerate(self.bases):
            g, k = _grid_desc(b)
            arr[i] = g
            keep.append(k)
        h = C.c_void_p()
        rc = self.lib.gbcp_batch_create(len(self.bases), C.cast(arr, C.c_void_p), PREC[precision], int(nstreams),
                                        C.byref(h))
        if rc != 0:
            raise GbcpError("gbcp_batch_create", rc)
        self.h = h
        self._keep = keep

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbcp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        buf = C.create_string_buffer(512)
        self.lib.gbcp_batch_last_error(self.h, buf, 512)
        return buf.value.decode()

    @staticmethod
    def _flags(flags) -> int:
        if isinstance(flags, int):
            return flags
        return sum(STEP[f] for f in flags)

    def _io(self, cells):
        if len(cells) != len(self.bases):
            raise ValueError("one io entry per cell")
        io = (_lib.CellIO * len(cells))()
        c64 = {str(x["c0"].dtype) == "torch.complex64" for x in cells}
        if len(c64) != 1:
            raise ValueError("all cells complex128, or all complex64")
        self._c64 = c64.pop()
        for i, (x, b) in enumerate(zip(cells, self.bases)):
            ldc, n = _ld_wfn(x["c0"], b.ngw, allow_c64=True)
            if x.get("c2") is not None and x["c2"].dtype != x["c0"].dtype:
                raise ValueError("c2 must have the dtype of c0")
            io[i].c0 = _ptr(x["c0"]).value
            io[i].ldc = ldc
            io[i].nstate = n
            io[i].f = _ptr(x["f"]).value
            io[i].vpot = _ptr(x.get("vpot")).value if x.get("vpot") is not None else None
            io[i].rhoe = _ptr(x.get("rhoe")).value if x.get("rhoe") is not None else None
            if x.get("c2") is not None:
                io[i].c2 = _ptr(x["c2"]).value
                io[i].ldc2 = _ld_wfn(x["c2"], b.ngw, allow_c64=True)[0]
        return io

    def _step_flags(self, flags) -> int:
        return self._flags(flags) | (STEP["psi_c64"] if getattr(self, "_c64", False) else 0)

    def tune(self, cells, flags=("rhoofr", "vpsi", "ortho")) -> str:
        import torch
        torch.cuda.synchronize()
        buf = C.create_string_buffer(8192)
        io = self._io(cells)
        rc = self.lib.gbcp_batch_tune(self.h, C.cast(io, C.c_void_p), self._step_flags(flags), buf, 8192)
        if rc != 0:
            raise GbcpError("gbcp_batch_tune", rc, self.last_error())
        return buf.value.decode()

    def step(self, cells, flags=("rhoofr", "vpsi", "ortho")):
        """Returns (energies (ncells, 2): E_kin, Omega/N sum V rho; status (ncells,))."""
        import torch
        torch.cuda.synchronize()
        n = len(self.bases)
        en = np.zeros((n, 2))
        st = np.zeros(n, dtype=np.int32)
        io = self._io(cells)
        rc = self.lib.gbcp_batch_step(self.h, C.cast(io, C.c_void_p), self._step_flags(flags),
                                      en.ctypes.data_as(C.c_void_p), st.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise GbcpError("gbcp_batch_step", rc, self.last_error())
        return en, st

    def graph_kernels(self) -> int:
        k = C.c_int64()
        self.lib.gbcp_batch_graph_kernels(self.h, C.byref(k))
        return int(k.value)


def kernel_launches() -> int:
    return int(_lib.load().gbcp_kernel_launches())
