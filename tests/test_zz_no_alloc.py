"""gbcp_ovlap_noalloc: the overlap matrix for callers that cannot allocate.

Some callers cannot call cudaMalloc (their device memory is all owned by a
pool allocator, or their time-stepping loop must not stall the device with an
allocation's implicit synchronisation).  The allocation-free entry point keeps
its scratch in a fixed device array inside the library; this test calls it
through the C ABI with device pointers, twice in a row on different inputs,
and checks each result against the regular gbcp_ovlap entry point.  The
second call also shows that the shared array's leftover contents from the
first call do not leak into the result.  This file is collected last so that
a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from cpmd_gb300.synth import make_small_cell

pytestmark = pytest.mark.gpu


def _dev(c):
    import torch
    return torch.from_numpy(np.ascontiguousarray(c.T)).cuda()


def _perturbed(cl, scale, seed):
    rng = np.random.default_rng(seed)
    c = cl.c0 + scale * (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    c[0] = c[0].real
    return np.asfortranarray(c)


@pytest.mark.parametrize("nstate", [37, 130])
def test_ovlap_noalloc_matches_ovlap_twice(gpu_lib, nstate):
    import torch
    from cpmd_gb300 import Context

    lib = gpu_lib
    cl = make_small_cell(10.26, 32, 20.0, nstate, seed=70 + nstate)
    b = cl.basis
    ctx = Context(b, "fp64")
    stream = torch.cuda.current_stream().cuda_stream or 1
    for call, (scale, seed) in enumerate([(0.1, 1), (0.3, 2)]):
        c = _dev(_perturbed(cl, scale, seed))
        ref = ctx.ovlap(c)                                  # existing entry point
        s = torch.full((nstate, nstate), float("nan"), dtype=torch.float64, device=c.device)
        rc = lib.gbcp_ovlap_noalloc(C.c_void_p(c.data_ptr()), b.ngw, b.ngw, nstate, 1 if b.geq0 else 0,
                                    C.c_void_p(s.data_ptr()), C.c_void_p(stream))
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        err = float((s - ref).abs().max() / ref.abs().max())
        assert err < 1e-13, f"call {call}: rel err {err}"


def test_ovlap_noalloc_rejects_too_many_states(gpu_lib):
    import torch
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = gpu_lib.gbcp_ovlap_noalloc(C.c_void_p(x.data_ptr()), 10, 10, 1025, 1, C.c_void_p(x.data_ptr()), None)
    assert rc == 1
