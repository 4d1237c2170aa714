"""ctypes binding of ``libcpmd_gb300.so`` (the C ABI in include/cpmd_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libcpmd_gb300.so"

GBCP_OK = 0
STATUS = {
    0: "OK", 1: "ERR_ARG", 2: "ERR_NOT_SPD", 3: "ERR_NONFINITE", 4: "ERR_TIMEOUT",
    5: "ERR_CUDA", 6: "ERR_NOMEM", 7: "ERR_UNSUPPORTED", 8: "ERR_NOT_CONVERGED", 9: "ERR_IO",
    10: "ERR_CHARGE",
}
PREC = {"fp64": 0, "mixed": 1}
MEM_HOST, MEM_DEVICE = 0, 1
ORTHO = {"gs": 0, "lowdin": 1}


class GbcpError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str = ""):
        super().__init__(f"{fn}: {STATUS.get(code, code)} {msg}".strip())
        self.code = code


class GridDesc(C.Structure):
    _fields_ = [
        ("nr1", C.c_int32), ("nr2", C.c_int32), ("nr3", C.c_int32),
        ("kr1", C.c_int32), ("kr2", C.c_int32), ("kr3", C.c_int32),
        ("ngw", C.c_int32), ("geq0", C.c_int32),
        ("omega", C.c_double), ("tpiba2", C.c_double),
        ("inyh", C.POINTER(C.c_int32)), ("hg", C.POINTER(C.c_double)),
    ]


_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_DP = C.POINTER(C.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "gbcp_ctx_create": (_I, [C.POINTER(GridDesc), _I, _I, _P, C.POINTER(_P)]),
    "gbcp_ctx_destroy": (_I, [_P]),
    "gbcp_set_precision": (_I, [_P, _I]),
    "gbcp_set_stream": (_I, [_P, _P]),
    "gbcp_set_option": (_I, [_P, _I, _I]),
    "gbcp_synchronize": (_I, [_P]),
    "gbcp_last_error": (_I, [_P, C.c_char_p, _I]),
    "gbcp_kernel_launches": (C.c_int64, []),
    "gbcp_profile_enable": (_I, [_P, _I]),
    "gbcp_profile_read": (_I, [_P, _I, C.c_char_p, _I, _DP, C.POINTER(C.c_int64)]),
    "gbcp_rhoofr": (_I, [_P, _P, _I, _I, _P, _P, _DP, _DP, _DP, _I]),
    "gbcp_vpsi": (_I, [_P, _P, _I, _P, _I, _P, _P, _I, _I]),
    "gbcp_ortho": (_I, [_P, _P, _I, _I, _I, _DP, _I]),
    "gbcp_ovlap": (_I, [_P, _P, _I, _I, _P, _I]),
    "gbcp_profile_timeline": (_I, [_P, _I, C.c_char_p, _I, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gbcp_rortog": (_I, [_P, _P, _I, _P, _I, _I, _I, _D, _I, _P, _P, _I]),
    "gbcp_ovlap_noalloc": (_I, [_P, _I, _I, _I, _I, _P, _P]),
    "gbcp_ovlap2": (_I, [_P, _P, _I, _P, _I, _I, _P, _I]),
    "gbcp_vofrho": (_I, [_P, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _I]),
    "gbcp_invfftn": (_I, [_P, _P, _I]),
    "gbcp_fwfftn": (_I, [_P, _P, _I]),
    "gbcp_rnlsm1": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _I, _I, _I]),
    "gbcp_fnonloc": (_I, [_P, _P, _I, _I, _P, _I, _I, _P, _P, _P, _P, _I, _I, _P, _I]),
    "gbcp_rnlsm2": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _I, _I, _I]),
    "gbcp_rnlfor": (_I, [_P, _I, _P, _I, _I, _P, _P, _P, _I, _I, _P, _I]),
    "gbcp_set_dens_sphere": (_I, [_P, _I, _P, _P]),
    "gbcp_energy": (_I, [_P, _P, _I, _I, _P, _I, _I, _P, _P, _P, _P, _P, _P, _I, _P, _P, _I]),
    "gbcp_batch_create": (_I, [_I, _P, _I, _I, C.POINTER(_P)]),
    "gbcp_batch_destroy": (_I, [_P]),
    "gbcp_batch_tune": (_I, [_P, _P, _I, _P, _I]),
    "gbcp_batch_step": (_I, [_P, _P, _I, _P, _P]),
    "gbcp_batch_graph_kernels": (_I, [_P, C.POINTER(C.c_int64)]),
    "gbcp_batch_last_error": (_I, [_P, _P, _I]),
    "gbcp_restart_write": (_I, [C.c_char_p, _P]),
    "gbcp_restart_read": (_I, [C.c_char_p, _P]),
}


class CellIO(C.Structure):
    _fields_ = [("c0", C.c_void_p), ("ldc", C.c_int32), ("nstate", C.c_int32), ("f", C.c_void_p),
                ("vpot", C.c_void_p), ("rhoe", C.c_void_p), ("c2", C.c_void_p), ("ldc2", C.c_int32)]



class Restart(C.Structure):
    """gbcp_restart of include/cpmd_gb300.h."""
    _fields_ = [("ibrav", C.c_int32), ("indpg", C.c_int32), ("celldm", C.c_double * 6),
                ("nsp", C.c_int32), ("nat", C.c_int32), ("na", C.c_void_p),
                ("tau0", C.c_void_p), ("taum", C.c_void_p), ("taui", C.c_void_p),
                ("ecut", C.c_double), ("cdual", C.c_double), ("dual", C.c_int32), ("nel", C.c_int32),
                ("nr1s", C.c_int32), ("nr2s", C.c_int32), ("nr3s", C.c_int32),
                ("nstate", C.c_int32), ("nkpts", C.c_int32),
                ("ngwks", C.c_int32), ("ngwls", C.c_int32), ("nhgs", C.c_int32), ("nhgls", C.c_int32),
                ("c0", C.c_void_p), ("ldc", C.c_int32), ("ngw", C.c_int32), ("nstate_cap", C.c_int32),
                ("icompr", C.c_int32), ("scale", C.c_double),
                ("nstate_read", C.c_int32), ("nstate_file", C.c_int32), ("sections", C.c_int32),
                ("f", C.c_void_p), ("eigv", C.c_void_p), ("amu", C.c_double),
                ("cm", C.c_void_p), ("ncm_read", C.c_int32), ("pad_", C.c_int32)]


_lib = None


def load(path: str | os.PathLike | None = None):
    """Load the CUDA library; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with cpmd_gb300.build.build() "
                           "(the hot path has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
