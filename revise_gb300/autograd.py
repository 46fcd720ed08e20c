"""torch.autograd binding of the batched ray caster and its hand-written adjoint,
for checking gradients with torch tooling only (forward: s3r_frame_render,
backward: s3r_render_argb_backward).  One FramePlan with FP32 bricks, exact
filtering; the differentiable inputs are the transfer-function table and the
plan's own brick store."""
from __future__ import annotations

from . import _lib
from .api import _torch


def _function():
    torch = _torch()

    class RenderFrame(torch.autograd.Function):
        @staticmethod
        def forward(ctx, tf, bricks, plan, view):
            store, _ = plan.bricks()
            if bricks.data_ptr() != store.data_ptr() or bricks.numel() != store.numel():
                raise ValueError("bricks must be the plan's brick store (FramePlan.bricks())")
            if view.filter != _lib.FILTER_EXACT:
                raise ValueError("the adjoint needs FILTER_EXACT")
            tf = tf.contiguous()
            rgba = torch.empty(view.W * view.H * 4, device=tf.device, dtype=torch.float32)
            plan.render(view, tf, rgba)
            ctx.plan, ctx.view = plan, view
            ctx.save_for_backward(tf, rgba)
            return rgba.view(view.H, view.W, 4)

        @staticmethod
        def backward(ctx, grad):
            tf, rgba = ctx.saved_tensors
            dtf = torch.zeros(tf.numel(), device=tf.device, dtype=torch.float32)
            store, _ = ctx.plan.bricks()
            ddense = torch.zeros(store.numel(), device=tf.device, dtype=torch.float32)
            ctx.plan.backward(ctx.view, tf, rgba, grad.contiguous().view(-1), dtf, ddense)
            return dtf.view_as(tf), ddense, None, None

    return RenderFrame


_RenderFrame = None


def render_frame(plan, view, tf, bricks):
    """Image (H, W, 4) of plan's bricks under view and tf, differentiable in tf and bricks.
    Rows run top to bottom as in s3r_frame_render's output."""
    global _RenderFrame
    if _RenderFrame is None:
        _RenderFrame = _function()
    return _RenderFrame.apply(tf, bricks, plan, view)
