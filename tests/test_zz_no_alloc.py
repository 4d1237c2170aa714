"""gbcp_ovlap_noalloc: the overlap matrix for callers that cannot allocate.

Some callers cannot call cudaMalloc (their device memory is all owned by a
pool allocator, or their time-stepping loop must not stall the device with an
allocation's implicit synchronisation).  The allocation-free entry point keeps
its scratch in a fixed device array inside the library; these tests call it
through the C ABI with device pointers, twice in a row on different inputs,
and check each result against the oracle's FP64 overlap (the reference's
dsyrk + dger Γ form) and against the regular gbcp_ovlap entry point.  The
second call also shows that the shared array's leftover contents from the
first call do not leak into the result.  The largest accepted state count
(1024, where the split-K partials fill the whole array) and a leading
dimension above ngw are covered too.  This file is collected last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-13  # relative to max|S|, FP64 on both sides


def _states(ngw, ldc, n, scale, seed):
    """(ldc, n) column-major complex states, rows beyond ngw filled with junk
    that must not be read, Im c(G=0) = 0."""
    rng = np.random.default_rng(seed)
    c = np.full((ldc, n), 7.0e3 + 3.0e3j, dtype=np.complex128, order="F")
    g = np.exp(-np.linspace(0.0, 4.0, ngw))[:, None]
    c[:ngw] = scale * g * (rng.standard_normal((ngw, n)) + 1j * rng.standard_normal((ngw, n)))
    c[0] = c[0].real
    return c


def _call(lib, c, ngw, n, stream):
    import torch
    ldc = c.shape[0]
    dev = torch.from_numpy(np.ascontiguousarray(c.T)).cuda()  # (n, ldc) rows = Fortran columns
    s = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib.gbcp_ovlap_noalloc(C.c_void_p(dev.data_ptr()), ldc, ngw, n, 1, C.c_void_p(s.data_ptr()),
                                C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, s.cpu().numpy(), dev


@pytest.mark.parametrize("ngw,pad,nstate", [(824, 0, 37), (824, 0, 130), (1473, 5, 96), (2100, 3, 1024)])
def test_ovlap_noalloc_matches_oracle_twice(gpu_lib, ngw, pad, nstate):
    import torch
    from cpmd_gb300 import Context
    from cpmd_gb300.cell import make_basis

    lib = gpu_lib
    stream = torch.cuda.current_stream().cuda_stream or 1
    b = make_basis(10.26, 32, 20.0) if ngw == 824 else None
    ctx = Context(b, "fp64") if b is not None and b.ngw == ngw and pad == 0 else None
    for call, (scale, seed) in enumerate([(1.0, 11 + nstate), (0.3, 29 + nstate)]):
        c = _states(ngw, ngw + pad, nstate, scale, seed)
        rc, s, dev = _call(lib, c, ngw, nstate, stream)
        assert rc == 0, f"call {call}: status {rc}"
        ref = O.overlap(c[:ngw], True)
        err = float(np.abs(s - ref).max() / np.abs(ref).max())
        assert err < TOL, f"call {call}: rel err vs oracle {err}"
        if ctx is not None:  # the regular entry point on the same device data
            reg = ctx.ovlap(dev).cpu().numpy()
            err = float(np.abs(s - reg).max() / np.abs(reg).max())
            assert err < TOL, f"call {call}: rel err vs gbcp_ovlap {err}"
    if ctx is not None:
        ctx.close()


def test_ovlap_noalloc_rejects_too_many_states(gpu_lib):
    import torch
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = gpu_lib.gbcp_ovlap_noalloc(C.c_void_p(x.data_ptr()), 10, 10, 1025, 1, C.c_void_p(x.data_ptr()), None)
    assert rc == 1
    rc = gpu_lib.gbcp_ovlap_noalloc(C.c_void_p(x.data_ptr()), 9, 10, 4, 1, C.c_void_p(x.data_ptr()), None)
    assert rc == 1  # leading dimension below ngw
