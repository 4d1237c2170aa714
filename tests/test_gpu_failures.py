"""Failure detection on the GPU, in forms that can neither fault nor hang it.

* Non-finite input, injected on the host: a NaN in c0 makes gbcp_ortho
  (both overlap engines, host and device memory) and gbcp_rhoofr return
  GBCP_ERR_NONFINITE with c0 bit-identical to the input; a NaN in the external
  potential V makes gbcp_vofrho do the same.  The next call on the same
  context succeeds and matches the oracle.
* A bounded device wait that runs out: the context's test hook makes the next
  tensor-core overlap issue no operand loads, so the MMA thread's first wait
  on a stage (towards which no copy is in flight) expires after about a
  millisecond.  The kernel frees its TMEM and returns, gbcp_ortho reports
  GBCP_ERR_TIMEOUT with c0 untouched, and the following call succeeds.
"""
import numpy as np
import pytest

from cpmd_gb300.synth import make_cell, make_small_cell
from oracle import cpmd_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def same_bits(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def perturbed(cl, seed=5, scale=0.02):
    rng = np.random.default_rng(seed)
    c = cl.c0 + scale * (rng.standard_normal(cl.c0.shape) + 1j * rng.standard_normal(cl.c0.shape))
    c[0] = c[0].real
    return np.asfortranarray(c)


@pytest.mark.parametrize("mode", ["host", "device"])
@pytest.mark.parametrize("precision,gemm", [("fp64", 0), ("mixed", 1)])
def test_nan_in_c0_ortho_reports_nonfinite(gpu_lib, mode, precision, gemm):
    import torch
    from cpmd_gb300 import Context, GbcpError
    cl = make_small_cell(10.26, 32, 20.0, 24, seed=90)
    b = cl.basis
    good = perturbed(cl)
    bad = good.copy(order="F")
    bad[17, 5] = complex(np.nan, 0.3)
    ctx = Context(b, precision)
    ctx.set_option("gemm", gemm)
    c = bad.copy(order="F") if mode == "host" else torch.from_numpy(np.ascontiguousarray(bad.T)).cuda()
    with pytest.raises(GbcpError) as e:
        ctx.ortho(c, "gs")
    assert e.value.code == 3, ctx.last_error()
    after = c if mode == "host" else np.asfortranarray(c.cpu().numpy().T)
    assert same_bits(after, bad)                                   # c0 untouched
    # the next call on the same context
    c = good.copy(order="F") if mode == "host" else torch.from_numpy(np.ascontiguousarray(good.T)).cuda()
    ctx.ortho(c, "gs")
    got = c if mode == "host" else np.asfortranarray(c.cpu().numpy().T)
    assert rel(got, O.rgs(good, b.geq0)) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_in_c0_rhoofr_reports_nonfinite(gpu_lib, precision):
    import torch
    from cpmd_gb300 import Context, GbcpError
    cl = make_cell("c0")
    b = cl.basis
    bad = cl.c0.copy(order="F")
    bad[40, 2] = np.nan
    ctx = Context(b, precision)
    c = torch.from_numpy(np.ascontiguousarray(bad.T)).cuda()
    with pytest.raises(GbcpError) as e:
        ctx.rhoofr(c, torch.from_numpy(cl.f).cuda())
    assert e.value.code == 3
    assert same_bits(np.asfortranarray(c.cpu().numpy().T), bad)
    rho, ekin, csumg, csumr = ctx.rhoofr(cl.c0, cl.f)
    rr, ek, _, _ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    assert rel(rho, rr) < (1e-10 if precision == "fp64" else 2e-5)


def test_nan_in_potential_reports_nonfinite(gpu_lib):
    from cpmd_gb300 import Context, GbcpError
    cl = make_cell("c0")
    b = cl.basis
    rho, _, _, _ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    vext = np.zeros(tuple(b.kr[::-1]))
    vext[3, 4, 5] = np.nan
    ctx = Context(b, "fp64")
    vps = O.gaussian_vps(b.hg, b.tpiba2, b.omega)[:, None]
    with pytest.raises(GbcpError) as e:
        ctx.vofrho(rho, cl.tau, vps, None, vext)
    assert e.value.code == 3
    vext[3, 4, 5] = 0.0
    veff, terms, _ = ctx.vofrho(rho, cl.tau, vps, None, vext)
    assert np.all(np.isfinite(veff))


@pytest.mark.parametrize("mode", ["device", "host"])
def test_tensor_core_wait_timeout_is_reported_and_recovered(gpu_lib, mode):
    import torch
    from cpmd_gb300 import Context, GbcpError
    cl = make_cell("c1", nstate=64)
    b = cl.basis
    good = perturbed(cl, seed=7)
    ctx = Context(b, "mixed")
    ctx.set_option("gemm", 1)
    ctx.set_option("test_timeout", 1)
    c = good.copy(order="F") if mode == "host" else torch.from_numpy(np.ascontiguousarray(good.T)).cuda()
    with pytest.raises(GbcpError) as e:
        ctx.ortho(c, "gs")
    assert e.value.code == 4, ctx.last_error()
    after = c if mode == "host" else np.asfortranarray(c.cpu().numpy().T)
    assert same_bits(after, good)                                  # nothing written
    # the hook cleared itself: the next call on the same context succeeds
    ctx.ortho(c, "gs")
    got = c if mode == "host" else np.asfortranarray(c.cpu().numpy().T)
    assert rel(got, O.rgs(good, b.geq0)) < 1e-10
    s = ctx.ovlap(torch.from_numpy(np.ascontiguousarray(got.T)).cuda())
    assert float((s - torch.eye(64, dtype=torch.float64, device=s.device)).abs().max()) < 1e-12
