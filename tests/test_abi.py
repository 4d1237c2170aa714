"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports
every entry point declared in include/cpmd_gb300.h.  No compute call is made
(there is no GPU here); argument validation that returns before any CUDA call
is exercised."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "cpmd_gb300.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gbcp_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from cpmd_gb300 import build as B
    B.build()
    from cpmd_gb300 import _lib
    return _lib.load()


def test_header_declares_hot_path_entry_points():
    syms = declared_symbols()
    for s in ("gbcp_rhoofr", "gbcp_vpsi", "gbcp_ortho", "gbcp_invfftn", "gbcp_fwfftn", "gbcp_rnlsm1",
              "gbcp_fnonloc", "gbcp_ctx_create", "gbcp_ctx_destroy"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_python_binding_covers_header():
    from cpmd_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_create_rejects_bad_arguments_without_gpu(lib):
    from cpmd_gb300 import _lib
    h = C.c_void_p()
    assert lib.gbcp_ctx_create(None, 0, 0, None, C.byref(h)) == 1
    g = _lib.GridDesc()
    g.nr1 = g.nr2 = g.nr3 = 32
    g.kr1 = g.kr2 = g.kr3 = 31  # leading dim below the mesh
    inyh = np.zeros(3, np.int32)
    hg = np.zeros(1)
    g.inyh = inyh.ctypes.data_as(C.POINTER(C.c_int32))
    g.hg = hg.ctypes.data_as(C.POINTER(C.c_double))
    g.ngw = 1
    g.omega = 1.0
    g.tpiba2 = 1.0
    assert lib.gbcp_ctx_create(C.byref(g), 0, 0, None, C.byref(h)) == 1
    g.kr1 = g.kr2 = g.kr3 = 33
    assert lib.gbcp_ctx_create(C.byref(g), 7, 0, None, C.byref(h)) == 1  # unknown precision
    # NULL context on every entry point
    assert lib.gbcp_rhoofr(None, None, 0, 0, None, None, None, None, None, 0) == 1
    assert lib.gbcp_vpsi(None, None, 0, None, 0, None, None, 0, 0) == 1
    assert lib.gbcp_ortho(None, None, 0, 0, 0, None, 0) == 1
    assert lib.gbcp_invfftn(None, None, 0) == 1
    assert lib.gbcp_rnlsm1(None, None, 0, 0, 0, 0, None, None, None, None, 0, 0, 0) == 1
    assert lib.gbcp_kernel_launches() >= 0


def test_built_for_sm103a():
    from cpmd_gb300 import build as B
    assert "arch=compute_103a,code=sm_103a" in " ".join(B.ARCH)


def test_python_options_match_header_enum():
    """Every GBCP_OPT_* of the header is reachable from Context.set_option under its
    lower-case name, with the header's value, and nothing else is."""
    from cpmd_gb300.api import OPTIONS
    txt = (ROOT / "include" / "cpmd_gb300.h").read_text()
    body = re.search(r"enum gbcp_option\s*\{(.*?)\}", txt, flags=re.S).group(1)
    enum = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"GBCP_OPT_([A-Z0-9_]+)\s*=\s*(\d+)", body)}
    assert enum == OPTIONS


def test_fortran_module_options_match_header_enum():
    """The option constants of the Fortran module in INTEGRATION.md are the header's
    (the test hook GBCP_OPT_TEST_TIMEOUT is left out there)."""
    txt = (ROOT / "include" / "cpmd_gb300.h").read_text()
    body = re.search(r"enum gbcp_option\s*\{(.*?)\}", txt, flags=re.S).group(1)
    enum = {m.group(1): int(m.group(2)) for m in re.finditer(r"(GBCP_OPT_[A-Z0-9_]+)\s*=\s*(\d+)", body)}
    enum.pop("GBCP_OPT_TEST_TIMEOUT")
    fort = (ROOT / "INTEGRATION.md").read_text()
    got = {m.group(1): int(m.group(2)) for m in re.finditer(r"(GBCP_OPT_[A-Z0-9_]+) = (\d+)", fort)}
    assert got == enum
