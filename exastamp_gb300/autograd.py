"""torch.autograd.Function bindings of the parameter adjoints.

* ``LJLoss.apply(params, context, rcut, f_target, e_target, w_force,
  w_energy)`` -- params = tensor [epsilon, sigma]; one system held by a
  ``_capi.Context`` (gbmd_lj_loss_grad).
* ``LJMultiLoss.apply(eps, sigma, context, rc, f_target, e_target, w_force,
  w_energy)`` -- eps, sigma = symmetric (ntypes, ntypes) tensors, rc the
  per-pair cutoffs (lj_multi_force; gbmd_lj_multi_loss_grad).  An (a, b)
  entry and its (b, a) mirror are one parameter of the potential; backward
  gives each of them half of that parameter's derivative (a != b), so a
  symmetric parametrisation (e.g. U + U.T) receives the exact gradient.
* ``EamLoss.apply(params, batch, cfg, rcut, f_target, e_target, w_force,
  w_energy)`` -- params = tensor of the 9 analytic parameters in
  ``setfl.PARAM_NAMES`` order; the configurations held by a ``_capi.Batch``
  (persistent forward + adjoint launch).  The tables and their parameter
  derivatives are re-tabulated on the host at ``params``.

Both return the force-matching + energy loss
``w_force sum |F - F*|^2 + w_energy sum (E - E*)^2`` as a 0-d tensor; the
backward pass hands back grad_output times the gradient that the adjoint
kernel computed in the same forward call (every pair term recomputed on the
device, nothing stored).  The bindings are thin: no torch code touches the
device data, and a forward call runs the C ABI synchronously.
"""
from __future__ import annotations

import numpy as np
import torch

from . import setfl


class LJLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, context, rcut, f_target, e_target, w_force, w_energy):
        eps, sig = (float(v) for v in params.detach().to("cpu", torch.float64))
        context.set_lj(eps, sig, rcut)
        loss, g = context.lj_loss_grad(f_target, e_target, w_force, w_energy)
        ctx.save_for_backward(torch.as_tensor(g, dtype=params.dtype))
        return torch.as_tensor(loss, dtype=params.dtype)

    @staticmethod
    def backward(ctx, g_out):
        (g,) = ctx.saved_tensors
        return g_out * g, None, None, None, None, None, None


class LJMultiLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps, sigma, context, rc, f_target, e_target, w_force, w_energy):
        e = eps.detach().to("cpu", torch.float64).numpy()
        sg = sigma.detach().to("cpu", torch.float64).numpy()
        if not (np.array_equal(e, e.T) and np.array_equal(sg, sg.T)):
            raise ValueError("eps and sigma must be symmetric")
        context.set_lj_multi(e, sg, np.asarray(rc, dtype=np.float64), 0.0)
        loss, ge, gs = context.lj_multi_loss_grad(f_target, e_target, w_force, w_energy)
        half = np.where(np.eye(len(e), dtype=bool), 1.0, 0.5)
        ctx.save_for_backward(torch.as_tensor(ge * half, dtype=eps.dtype), torch.as_tensor(gs * half, dtype=eps.dtype))
        return torch.as_tensor(loss, dtype=eps.dtype)

    @staticmethod
    def backward(ctx, g_out):
        ge, gs = ctx.saved_tensors
        return g_out * ge, g_out * gs, None, None, None, None, None, None


class EamLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, batch, cfg, rcut, f_target, e_target, w_force, w_energy):
        p = dict(zip(setfl.PARAM_NAMES, params.detach().to("cpu", torch.float64).tolist()))
        batch.set_eam_alloy(setfl.tabulate(cfg, p), rcut)
        batch.set_param_derivatives(*setfl.table_param_jacobian(cfg, p))
        batch.set_targets(f_target, e_target, w_force, w_energy)
        batch.run(adjoint=True)
        d = batch.download()
        ctx.save_for_backward(torch.as_tensor(np.asarray(d["grad"]), dtype=params.dtype))
        return torch.as_tensor(d["loss"], dtype=params.dtype)

    @staticmethod
    def backward(ctx, g_out):
        (g,) = ctx.saved_tensors
        return g_out * g, None, None, None, None, None, None, None
