"""torch.autograd binding of the hand-written adjoint (a small test binding).

``power_spectrum(pos, masses, ctx, boxsize, mass, quirk)`` returns the
auto P(k) of one species as a differentiable CUDA tensor; its backward calls
genpk_adjoint through the C ABI (mode gradient -> c2r -> CIC gather).  The
normalisation mass is M = sum(masses) + quirk (or n*mass + quirk), the way
gen-pk forms total_mass (read_fieldize.cpp:79-94), so dL/dmass includes the
dependence of M on the masses.
"""
from __future__ import annotations

import numpy as np
import torch


class _PowerSpectrum(torch.autograd.Function):
    @staticmethod
    def forward(fctx, pos, masses, gctx, field, boxsize, mass, quirk):
        n = pos.shape[0]
        if masses is not None:
            m_norm = float(masses.double().sum()) + quirk
        else:
            m_norm = n * float(mass) + quirk
        gctx.zero(field)
        gctx.deposit(field, boxsize, pos, masses, mass)
        p, _, _ = gctx.power(field, field, m_norm, m_norm)
        fctx.gctx, fctx.field, fctx.boxsize, fctx.mass, fctx.m_norm = gctx, field, boxsize, mass, m_norm
        fctx.save_for_backward(pos, masses if masses is not None else torch.empty(0))
        fctx.has_masses = masses is not None
        return torch.from_numpy(p).to(pos.device)

    @staticmethod
    def backward(fctx, grad_p):
        pos, masses = fctx.saved_tensors
        masses = masses if fctx.has_masses else None
        g = grad_p.detach().double().cpu().numpy()
        gpos, gmass, _ = fctx.gctx.adjoint(fctx.field, fctx.boxsize, pos, g, fctx.m_norm,
                                           masses=masses, mass=fctx.mass)
        return gpos, gmass, None, None, None, None, None


def power_spectrum(pos, masses, gctx, boxsize, mass=0.0, quirk=1.0, field=0):
    """Differentiable auto spectrum P_b (float64 tensor on pos.device)."""
    return _PowerSpectrum.apply(pos, masses, gctx, field, float(boxsize), float(mass), float(quirk))


def relative_loss(p, target, count):
    """Sum_b (P_b - T_b)^2 / T_b^2 over non-empty bins, and dL/dP."""
    ok = torch.as_tensor(np.asarray(count) > 0, device=p.device)
    t = torch.as_tensor(target, device=p.device, dtype=torch.float64)
    d = torch.where(ok, (p - t) / t, torch.zeros_like(p))
    return (d * d).sum()
