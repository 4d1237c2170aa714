"""Python loader of the C++/OpenMP FP64 restatement (``oracle/cpmd_port.cpp``).

TEST INFRASTRUCTURE AND TIMED CPU BASELINE ONLY: the tests use it as a second
checker beside ``cpmd_oracle.py``, and ``bench.py`` times it as the CPU
stand-in for the reference's rhoofr / vpsi / rgs path (the reference itself,
Fortran + FFTW + BLAS/LAPACK, cannot be built here).  Nothing in the product
imports it.  ``build()`` compiles the shared library with g++ (no cmake, no
machine-specific flags, so the same recipe builds on x86-64 and aarch64).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpmd_port.cpp"
LIB = HERE / "libcpmd_port.so"
_lib = None


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        cmd = ["g++", "-O3", "-std=c++17", "-fcx-limited-range", "-fopenmp", "-fPIC", "-shared", str(SRC), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cpmd_port build failed:\n" + r.stdout + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        P, I, D = C.c_void_p, C.c_int, C.c_double
        DP = C.POINTER(C.c_double)
        lib.port_create.restype = P
        lib.port_create.argtypes = [I, I, I, I, I, I, I, I, D, D, P, P, I]
        lib.port_destroy.argtypes = [P]
        lib.port_fft1.restype = I
        lib.port_fft1.argtypes = [I, P, I]
        lib.port_rhoofr.restype = I
        lib.port_rhoofr.argtypes = [P, P, I, I, P, P, DP, DP, DP]
        lib.port_vpsi.restype = I
        lib.port_vpsi.argtypes = [P, P, I, P, I, P, P, I]
        lib.port_rgs.restype = I
        lib.port_rgs.argtypes = [P, P, I, I]
        lib.port_threads.restype = I
        lib.port_threads.argtypes = [P]
        _lib = lib
    return _lib


def fft1(x: np.ndarray, sign: int) -> np.ndarray:
    """One length-n transform (e^{sign 2 pi i jk/n}, unscaled) of a complex vector."""
    y = np.ascontiguousarray(x, dtype=np.complex128).copy()
    rc = load().port_fft1(len(y), y.ctypes.data, int(sign))
    if rc:
        raise ValueError(f"length {len(y)} is not 2,3,5-smooth")
    return y


def _c(x):
    return C.c_void_p(x.ctypes.data)


class Port:
    """The restated CPU path on one cell; arrays are numpy, laid out like the
    reference's (c0(ngw, n) column-major complex, rhoe/vpot (kr3, kr2, kr1))."""

    def __init__(self, basis, threads: int = 0):
        self.lib = load()
        self.b = basis
        mill = np.ascontiguousarray(basis.mill[: basis.ngw], dtype=np.int32)
        hg = np.ascontiguousarray(basis.hg[: basis.ngw], dtype=np.float64)
        self.h = self.lib.port_create(*basis.nr, *basis.kr, basis.ngw, 1 if basis.geq0 else 0, basis.omega,
                                      basis.tpiba2, _c(mill), _c(hg), int(threads))
        if not self.h:
            raise ValueError("mesh is not 2,3,5-smooth")
        self.threads = self.lib.port_threads(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.port_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @staticmethod
    def _ld(c):
        assert c.dtype == np.complex128 and c.ndim == 2 and c.strides[0] == 16
        return c.strides[1] // 16 if c.shape[1] > 1 else c.shape[0], c.shape[1]

    def rhoofr(self, c0, f):
        ld, n = self._ld(c0)
        rho = np.empty(tuple(self.b.kr[::-1]))
        ek, cg, cr = C.c_double(), C.c_double(), C.c_double()
        f = np.ascontiguousarray(f, dtype=np.float64)
        self.lib.port_rhoofr(self.h, _c(c0), ld, n, _c(f), _c(rho), C.byref(ek), C.byref(cg), C.byref(cr))
        return rho, ek.value, cg.value, cr.value

    def vpsi(self, c0, c2, f, vpot):
        ld, n = self._ld(c0)
        ld2, _ = self._ld(c2)
        f = np.ascontiguousarray(f, dtype=np.float64)
        vpot = np.ascontiguousarray(vpot, dtype=np.float64)
        self.lib.port_vpsi(self.h, _c(c0), ld, _c(c2), ld2, _c(f), _c(vpot), n)
        return c2

    def rgs(self, c0):
        ld, n = self._ld(c0)
        rc = self.lib.port_rgs(self.h, _c(c0), ld, n)
        if rc:
            raise ValueError("overlap matrix not positive definite")
        return c0


def host_threads() -> int:
    """Host cores this process may use (the OpenMP default)."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1
