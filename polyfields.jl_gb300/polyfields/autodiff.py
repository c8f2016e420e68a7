"""Differentiable density and free energy of a FieldSystem as torch autograd ops.

``density(sys, fields)`` takes a dict {monomer id: torch tensor of the grid shape (float64,
any device)} and returns {monomer id: density tensor}; backpropagation runs the engine's
adjoint (``FieldSystem.density_pullback``, C ABI ``pf_density_pullback``), the counterpart
of a ChainRulesCore.rrule for density!(sys) on the Julia side.  ``free_energy(sys, fields)``
returns free_energy as a 0-d tensor; its backward is ``pf_free_energy_pullback``.  Cell,
composition and chi gradients are not tensors of these ops: read them from
``density_pullback`` / ``free_energy_pullback`` directly.
"""
from typing import Dict

import numpy as np
import torch


class _Density(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sys, mids, *ws):
        for mid, w in zip(mids, ws):
            sys.fields[mid] = w.detach().to("cpu", torch.float64).numpy()
        sys.density_update()
        ctx.sys, ctx.mids = sys, mids
        ctx.devices = [w.device for w in ws]
        outs = [torch.from_numpy(np.ascontiguousarray(sys.density[mid])).to(ws[0].device) for mid in sys.monomers]
        ctx.out_mids = list(sys.monomers)
        return tuple(outs)

    @staticmethod
    def backward(ctx, *grads):
        rbar = {}
        for mid, g in zip(ctx.out_mids, grads):
            if g is not None:
                rbar[mid] = g.detach().to("cpu", torch.float64).numpy()
        pb = ctx.sys.density_pullback(rbar)
        wgrads = [torch.from_numpy(pb["w"][mid]).to(dev) for mid, dev in zip(ctx.mids, ctx.devices)]
        return (None, None, *wgrads)


def density(sys, fields: Dict[int, torch.Tensor]) -> Dict[int, torch.Tensor]:
    """Densities of ``sys`` for the given fields, differentiable with respect to them."""
    mids = list(fields.keys())
    outs = _Density.apply(sys, mids, *[fields[m] for m in mids])
    return dict(zip(list(sys.monomers), outs))


class _FreeEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sys, mids, *ws):
        for mid, w in zip(mids, ws):
            sys.fields[mid] = w.detach().to("cpu", torch.float64).numpy()
        pb = sys.free_energy_pullback()
        ctx.grads = [torch.from_numpy(pb["w"][mid]).to(w.device) for mid, w in zip(mids, ws)]
        return torch.tensor(pb["fhelm"], dtype=torch.float64, device=ws[0].device)

    @staticmethod
    def backward(ctx, g):
        return (None, None, *[g * x for x in ctx.grads])


def free_energy(sys, fields: Dict[int, torch.Tensor]) -> torch.Tensor:
    """free_energy of ``sys`` at the given fields (a 0-d tensor), differentiable with respect to them."""
    mids = list(fields.keys())
    return _FreeEnergy.apply(sys, mids, *[fields[m] for m in mids])
