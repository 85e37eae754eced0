"""Differentiable rendering: a ``torch.autograd.Function`` whose backward is the library's
hand-written adjoint (``ap_render_vjp``) instead of autograd through the render graph.

``render(batch, params, psf)`` maps value-space parameters ``[n, 8]`` (full-vector slots
[cx, cy, q, PA, n, Re, Ie, F]) to the packed model images of a ``StampBatch``; the gradient
flows to the batch's fitted slots (``options.free_mask``) and is zero for the locked ones.
The reference obtains the same gradient with autograd through ``Component_Model.sample``
(``negative_log_likelihood().backward()``, astrophot/models/core_model.py:220-256).
"""

from __future__ import annotations

import torch

__all__ = ("RenderFunction", "render")


class RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, batch, psf, reference_center):
        ctx.batch = batch
        ctx.psf = psf
        ctx.reference_center = reference_center
        ctx.save_for_backward(params)
        return batch.render(params.detach(), psf)

    @staticmethod
    def backward(ctx, grad_model):
        (params,) = ctx.saved_tensors
        batch = ctx.batch
        g = batch.vjp(params.detach(), ctx.psf, grad_model, reference_center=ctx.reference_center)
        full = torch.zeros(params.shape, dtype=params.dtype, device=params.device)
        slots = [i for i in range(8) if batch.options.free_mask & (1 << i)]
        full[:, slots] = g.to(params.dtype)
        return full, None, None, None


def render(batch, params, psf=None, reference_center=False):
    """Differentiable ``batch.render``.  ``reference_center=True`` gives the center entries the
    value the reference's reverse-mode autograd gives under PSF shift (derivative through the
    sub-pixel PSF shift plus the sampling-coordinate path); the default is the derivative of the
    render itself (finite differences, ``StampBatch.jacobian``)."""
    return RenderFunction.apply(params, batch, psf, reference_center)
