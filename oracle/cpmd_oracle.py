"""FP64 CPU oracle for CPMD's Γ-point wavefunction hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``cpmd_gb300``, the CUDA
library, the C ABI) imports, calls or links this file; only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it,
and only as the checker or as the timed CPU stand-in for the reference.

The reference (CPMD 4.3, Fortran + FFTW3 + BLAS/LAPACK) cannot be compiled in
this environment (no Fortran compiler, no FFTW, no BLAS/LAPACK), so this module
restates its arithmetic in numpy/scipy, following the cited lines:

* G-vector list / ordering ......... loadpa_utils.mod.F90:286-330, 408, 748-792
* Γ pair packing ................... state_utils.mod.F90:165-189
* inverse / forward FFT convention . fftmain_utils.mod.F90:90-154,
                                     mltfft_utils.mod.F90:513-517
  (invfftn: isign=-1 -> FFTW_BACKWARD, e^{+iGr}, unscaled;
   fwfftn: isign=+1 -> FFTW_FORWARD, e^{-iGr}, scaled 1/(nr1 nr2 nr3))
* density .......................... rhoofr_utils.mod.F90:305-409, 607-635;
                                     density_utils.mod.F90:61-83
* kinetic energy / charge .......... kin_energy_utils.mod.F90:62-108;
                                     dotp_utils.mod.F90:45-52
* vpsi decode + kinetic ............ vpsi_utils.mod.F90:627-671, 717
* Gram-Schmidt ortho ............... rgs_utils.mod.F90:63-74, 127-158;
                                     ortho_utils.mod.F90:264-268 (zclean)
* Loewdin ortho .................... lowdin_utils.mod.F90:58-89;
                                     csmat_utils.mod.F90:51, 82-89;
                                     ovlap_utils.mod.F90:150-165
* projector overlaps ............... rnlsm1_utils.mod.F90:83-167
* non-local force on C2 ............ fnonloc_utils.mod.F90:306-354

Parity status: the reference ships no test suite, fixtures or golden vectors
for this path, and its third-party FFT/BLAS calls are not pinned by any test,
so this oracle is "parity unpinned" at the FFTW/BLAS boundary.  It is pinned
instead by the reference's own runtime invariants (charge consistency
|csumr - csumg| <= 1e-6, rhoofr_utils.mod.F90:625; scond = max|S-I|,
csmat_utils.mod.F90:82-89) and by analytic known-answer tests kept in
``tests/test_oracle.py`` and ``tests/golden/``.

Real-space phase: the reference stores G on a centred index (inyh = i + nr/2+1),
so its sparse inverse FFT yields (-1)^(x+y+z) psi(r).  Density (psi^2) and the
forward FFT of V*psi are unchanged by that sign, so rhoe and C2 agree with the
plain FFT-ordered transform used here.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.fft as sfft
import scipy.linalg as sla

EPSGX = 1.0e-12
WORKERS = -1


# ----------------------------------------------------------------------------
# G vectors (independent restatement of loadpa's loop; cross-checked in tests)
# ----------------------------------------------------------------------------
def gvectors(alat: float, nr: int, ecut: float, dual: float = 4.0):
    """Return (mill[nhg,3], hg[nhg], ngw) in the reference's sorted order."""
    tpiba2 = (2.0 * math.pi / alat) ** 2
    gcutw = ecut / tpiba2
    gcut = gcutw * dual
    r = int(math.isqrt(int(gcut))) + 1
    rows = []
    ig = 0
    for i in range(0, min(nr - 1, r) + 1):
        jmin = 0 if i == 0 else max(-nr + 1, -r)
        for j in range(jmin, min(nr - 1, r) + 1):
            kmin = 0 if (i == 0 and j == 0) else max(-nr + 1, -r)
            k = np.arange(kmin, min(nr - 1, r) + 1)
            g2 = float(i * i + j * j) + (k * k).astype(np.float64)
            k = k[g2 < gcut]
            g2 = g2[g2 < gcut]
            for kk, gg in zip(k.tolist(), g2.tolist()):
                ig += 1
                sgn = -1.0 if gg < gcutw else 1.0
                rows.append((gg * (1.0 + math.sqrt(ig - 1.0) * EPSGX * sgn), i, j, kk, gg))
    rows.sort(key=lambda t: t[0])
    mill = np.array([[t[1], t[2], t[3]] for t in rows], dtype=np.int64)
    hg = np.array([t[4] for t in rows])
    ngw = int((hg < gcutw).sum())
    return mill, hg, ngw


# ----------------------------------------------------------------------------
# FFT conventions
# ----------------------------------------------------------------------------
def invfftn(grid: np.ndarray) -> np.ndarray:
    """G -> r, e^{+iGr}, unscaled.  grid indexed [z, y, x]."""
    n = grid.size
    return sfft.ifftn(grid, workers=WORKERS) * n


def fwfftn(grid: np.ndarray) -> np.ndarray:
    """r -> G, e^{-iGr}, scaled by 1/(nr1 nr2 nr3)."""
    return sfft.fftn(grid, workers=WORKERS) / grid.size


def _grid_index(mill: np.ndarray, nr):
    n1, n2, n3 = nr
    return (np.mod(mill[:, 2], n3), np.mod(mill[:, 1], n2), np.mod(mill[:, 0], n1))


def pack_pair(c1, c2, mill, nr, geq0: bool):
    """set_psi_2_states_g / set_psi_1_state_g (state_utils.mod.F90:165-189)."""
    n1, n2, n3 = nr
    psi = np.zeros((n3, n2, n1), dtype=np.complex128)
    ip = _grid_index(mill, nr)
    im = _grid_index(-mill, nr)
    if c2 is None:
        psi[ip] = c1
        psi[im] = np.conj(c1)
        if geq0:
            psi[ip[0][0], ip[1][0], ip[2][0]] = c1[0]
    else:
        psi[ip] = c1 + 1j * c2
        psi[im] = np.conj(c1) + 1j * np.conj(c2)
        if geq0:
            psi[ip[0][0], ip[1][0], ip[2][0]] = c1[0] + 1j * c2[0]
    return psi


def dotp(a, b, geq0: bool):
    """Γ inner product (dotp_utils.mod.F90:45-52): with geq0 the G=0 term is
    Re a0 Re b0 only; every other G counts 2 (Re a Re b + Im a Im b)."""
    s = 2.0 * (np.dot(a[1:].real, b[1:].real) + np.dot(a[1:].imag, b[1:].imag))
    if geq0:
        s += a[0].real * b[0].real
    else:
        s += 2.0 * (a[0].real * b[0].real + a[0].imag * b[0].imag)
    return s


def kin_energy(c0, f, hg, tpiba2, geq0):
    """E_kin = tpiba2 sum_i f_i sum_G hg |c|^2 and rsum = sum f_i <c_i|c_i>."""
    rsum = 0.0
    xkin = 0.0
    for i in range(c0.shape[1]):
        if f[i] != 0.0:
            rsum += f[i] * dotp(c0[:, i], c0[:, i], geq0)
            xkin += f[i] * float(np.sum(hg[: c0.shape[0]] * (np.abs(c0[:, i]) ** 2)))
    return xkin * tpiba2, rsum


def pairs(nstate: int):
    return [(i, i + 1 if i + 1 < nstate else None) for i in range(0, nstate, 2)]


def rhoofr(c0, f, mill, nr, kr, omega, hg, tpiba2, geq0):
    """Density on the padded real-space layout (kr3, kr2, kr1) plus ekin, csumg, csumr."""
    n1, n2, n3 = nr
    ngw = c0.shape[0]
    m = mill[:ngw]
    ekin, rsum = kin_energy(c0, f, hg, tpiba2, geq0)
    rho = np.zeros((n3, n2, n1))
    for is1, is2 in pairs(c0.shape[1]):
        c2 = None if is2 is None else c0[:, is2]
        tf = (f[is1] != 0.0) or (is2 is not None and f[is2] != 0.0)
        if not tf:
            continue
        psi = invfftn(pack_pair(c0[:, is1], c2, m, nr, geq0))
        coef3 = f[is1] / omega
        coef4 = 0.0 if is2 is None else f[is2] / omega
        rho += coef3 * psi.real ** 2 + coef4 * psi.imag ** 2
    out = np.zeros((kr[2], kr[1], kr[0]))
    out[:n3, :n2, :n1] = rho
    csumr = float(out.sum()) * omega / float(n1 * n2 * n3)
    return out, ekin, rsum, csumr


def vpsi(c0, c2, f, vpot, mill, nr, hg, tpiba2, geq0, tksham: bool = False):
    """c2 += C2_vpsi; vpot in padded layout (kr3, kr2, kr1)."""
    n1, n2, n3 = nr
    ngw, nstate = c0.shape
    m = mill[:ngw]
    v = vpot[:n3, :n2, :n1]
    ip = _grid_index(m, nr)
    im = _grid_index(-m, nr)
    out = np.array(c2, dtype=np.complex128, copy=True, order="F")
    kin = tpiba2 * hg[:ngw]
    for is1, is2 in pairs(nstate):
        cc2 = None if is2 is None else c0[:, is2]
        psi = invfftn(pack_pair(c0[:, is1], cc2, m, nr, geq0))
        q = fwfftn(v * psi)
        psin = q[ip]
        psii = q[im]
        fp = psin + psii
        fm = psin - psii
        fi = f[is1] * 0.5
        if fi == 0.0:
            fi = 0.5 if tksham else 1.0
        fip1 = 0.0 if is2 is None else f[is2] * 0.5
        if fip1 == 0.0:
            fip1 = 0.5 if tksham else 1.0
        out[:, is1] += -fi * (kin * c0[:, is1] + (fp.real + 1j * fm.imag))
        if is2 is not None:
            out[:, is2] += -fip1 * (kin * c0[:, is2] + (fp.imag - 1j * fm.real))
    return out


# ----------------------------------------------------------------------------
# Orthogonalisation
# ----------------------------------------------------------------------------
def overlap(c, geq0):
    """S = 2 Re(C^H C) - Re c(0) Re c(0)^T (rgs_utils.mod.F90:63-68)."""
    s = 2.0 * (c.real.T @ c.real + c.imag.T @ c.imag)
    if geq0:
        s -= np.outer(c[0].real, c[0].real)
    return s


def rgs(c0, geq0):
    """Cholesky Gram-Schmidt: S = U^T U, C <- C U^{-1}, zclean."""
    s = overlap(c0, geq0)
    u, info = sla.lapack.dpotrf(s, lower=0)
    if info != 0:
        raise np.linalg.LinAlgError("UINV: ILLEGAL RESULTS DPOTRF")
    u = np.triu(u)
    uinv, info = sla.lapack.dtrtri(u, lower=0)
    if info != 0:
        raise np.linalg.LinAlgError("UINV: ILLEGAL RESULTS DTRTRI")
    c = c0 @ np.triu(uinv)
    if geq0:
        c[0] = c[0].real
    return np.asfortranarray(c)


def scond(s):
    d = np.abs(s - np.eye(s.shape[0]))
    return float(d.max())


def lowdin(c0, geq0):
    """Loewdin: S = Z w Z^T, A = Z w^{-1/2} Z^T, C <- C A; returns (C, scond of input S)."""
    s = overlap(c0, geq0)
    w, z = np.linalg.eigh(s)
    a = (z * (1.0 / np.sqrt(w))[None, :]) @ z.T
    c = c0 @ a
    if geq0:
        c[0] = c[0].real
    return np.asfortranarray(c), scond(s)


# ----------------------------------------------------------------------------
# Non-local projectors (one species, nat atoms, ngh projectors per atom)
# ----------------------------------------------------------------------------
def _ci(l: int) -> complex:
    return (-1j) ** int(l)


def rnlsm1(c0, twnl, eigr, nghtol, geq0):
    """fnl(isa, iv, i) = 2 sum_{real view} scr * c with scr = (-i)^l twnl eigr, G=0 halved."""
    ngw, nstate = c0.shape
    nat = eigr.shape[1]
    ngh = twnl.shape[1]
    fnl = np.zeros((nat, ngh, nstate))
    for iv in range(ngh):
        scr = (_ci(nghtol[iv]) * twnl[:, iv])[:, None] * eigr      # (ngw, nat)
        if geq0:
            scr = scr.copy()
            scr[0] *= 0.5
        fnl[:, iv, :] = 2.0 * (scr.real.T @ c0.real + scr.imag.T @ c0.imag)
    return fnl


def fnonloc(c2, f, fnl, twnl, eigr, nghtol, wsg):
    """c2 += twnl (-i)^l (-f wsg) sum_ia eigr fnl (BHS/KB branch)."""
    out = np.array(c2, dtype=np.complex128, copy=True, order="F")
    ngh = twnl.shape[1]
    ffi = np.where(f < 1e-5, 1.0, f)
    for iv in range(ngh):
        auxc = eigr @ fnl[:, iv, :]                                # (ngw, nstate)
        ctm = _ci(nghtol[iv]) * (-ffi * wsg[iv])                   # (nstate,)
        out += twnl[:, iv][:, None] * (auxc * ctm[None, :])
    return out
