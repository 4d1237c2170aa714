"""torch.autograd wrapper of the energy functional's hand-written adjoint.

``energy_fn(ctx, c0, vext, tau, f, vps, isp)`` returns E[psi, V, R] as a 0-d
tensor whose backward pass is the C-ABI adjoint (``gbcp_energy``): no graph of
the band loop is recorded, psi(r) is recomputed on the device, and the three
gradients come out of one call:

* c0 (nstate, ngw) complex128: torch's convention for a real loss is
  dL/dRe + i dL/dIm; with the reference's CP force C2 (vpsi applied to V_eff)
  that is -4 w_G C2, w = 1/2 at G = 0 (the Γ half sphere counts +G and -G);
  states with f = 0 carry no energy and get a zero gradient;
* vext (kr3, kr2, kr1) float64: rho(r) Omega / N;
* tau (nat, 3) float64: -F (forces from the structure factor, potfor).
"""
from __future__ import annotations

import torch


class EnergyFunction(torch.autograd.Function):
    @staticmethod
    def forward(actx, gctx, c0, vext, tau, f, vps, isp):
        terms, c2, dv, fion = gctx.energy(c0.detach(), f, tau.detach() if tau is not None else None, vps, isp,
                                          vext.detach() if vext is not None else None, grad=True, forces=True)
        w = torch.ones(gctx.ngw, dtype=torch.float64, device=c0.device)
        if gctx.basis.geq0:
            w[0] = 0.5
        occ = (f != 0).to(torch.float64)[:, None]
        gc = (-4.0) * c2 * (w[None, :] * occ)
        actx.save_for_backward(gc, dv, fion if fion is not None else torch.zeros(0, device=c0.device))
        actx.has_tau = tau is not None
        actx.has_vext = vext is not None
        actx.terms = terms
        return torch.tensor(terms["etot"], dtype=torch.float64, device=c0.device)

    @staticmethod
    def backward(actx, g):
        gc, dv, fion = actx.saved_tensors
        gtau = (-g) * fion if actx.has_tau else None
        gv = g * dv if actx.has_vext else None
        return None, g * gc, gv, gtau, None, None, None


def energy_fn(gctx, c0, vext, tau, f, vps, isp=None):
    """E as a differentiable function of (c0, vext, tau); f, vps, isp are constants."""
    return EnergyFunction.apply(gctx, c0, vext, tau, f, vps, isp)
