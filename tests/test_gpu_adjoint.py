"""Hand-written adjoint of the batched ray caster: GPU gradient vs the FP64
oracle gradient (relative error < 1e-3) and central finite differences
(eps = 1e-3) of the FP64 oracle forward at 64 random coordinates."""
import numpy as np
import pytest

import oracle
from revise_gb300 import host, workloads

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3


def _setup(W, H):
    w = workloads.cfg5(W=W, H=H)
    w.tf = np.clip(w.tf, 0.0, 1.0)
    return w


def _gpu_grad(ctx, w, target_img, keep=None):
    import torch
    from revise_gb300.api import FramePlan
    view = host.view_for(w)
    plan = FramePlan(ctx, w)
    sp = torch.from_numpy(w.sparse).cuda()
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    rgba = torch.zeros(w.W * w.H * 4, device="cuda")
    plan.interp(sp)
    plan.render(view, tf, rgba)
    tgt = torch.from_numpy(np.ascontiguousarray(target_img, np.float32).ravel()).cuda()
    dl = rgba - tgt
    if keep is not None:  # pixels whose sample sets float and FP64 arithmetic agree on
        dl = dl * torch.from_numpy(np.repeat(keep.astype(np.float32), 4)).cuda()
    dtf = torch.zeros(w.tf.size, device="cuda")
    bricks, offs = plan.bricks()
    dd = torch.zeros(bricks.numel(), device="cuda")
    plan.backward(view, tf, rgba, dl, dtf, dd)
    torch.cuda.synchronize()
    loss = 0.5 * float((dl.double() ** 2).sum())
    dd = plan.dense(dd)
    plan.close()
    return view, loss, dtf.cpu().numpy().reshape(-1, 4), dd.cpu().numpy()


def _rects(w, view):
    return np.array([host.block_view_rect(view, w.blocks[b, :3]) for b in range(w.nblocks)], np.int32)


def test_adjoint_matches_fp64_gradient(ctx):
    """Pixels where a block-local early-termination test lands within 1e-5 of its
    threshold (the FP64 oracle flags them) are left out of both gradients: there
    float and FP64 arithmetic may keep different sample sets."""
    w = _setup(160, 160)
    view = host.view_for(w)
    ov = oracle.view_from(view)
    dense = oracle.interp_workload(w)
    rects = _rects(w, view)
    target, _ = oracle.render_frame_f64(ov, w, dense, rects, w.meta["target_tf"])
    _, flags = oracle.render_frame_f64(ov, w, dense, rects, w.tf)
    keep = flags == 0
    assert keep.mean() > 0.97
    p = np.arange(w.W * w.H)[keep]
    pixels = np.stack([p % w.W, w.H - 1 - p // w.W], 1)
    loss64, dtf64, dd64 = oracle.render_frame_grad_f64(ov, w, dense, rects, w.tf, target[keep], pixels)
    view, loss, dtf, dd = _gpu_grad(ctx, w, target, keep)
    assert abs(loss - loss64) <= 1e-4 * loss64
    e_tf = np.linalg.norm(dtf - dtf64) / np.linalg.norm(dtf64)
    m = ~np.isnan(dense)
    e_dd = np.linalg.norm(dd[m] - dd64[m]) / np.linalg.norm(dd64[m])
    assert e_tf < REL_TOL, e_tf
    assert e_dd < REL_TOL, e_dd


def test_adjoint_vs_central_differences(ctx):
    w = _setup(48, 48)
    view = host.view_for(w)
    ov = oracle.view_from(view)
    dense = oracle.interp_workload(w)
    rects = _rects(w, view)
    target, _ = oracle.render_frame_f64(ov, w, dense, rects, w.meta["target_tf"])
    _, _, dtf, dd = _gpu_grad(ctx, w, target)

    def loss(tf, dn):
        img, _ = oracle.render_frame_f64(ov, w, dn, rects, tf)
        return 0.5 * float(((img.astype(np.float64) - target) ** 2).sum())

    rng = np.random.default_rng(64)
    eps = 1e-3
    # 32 transfer-function coordinates with nonzero gradient and 32 dense values
    tf_cand = np.flatnonzero(np.abs(dtf.ravel()) > 1e-3 * np.abs(dtf).max())
    dn_cand = np.flatnonzero(np.abs(dd) > 1e-3 * np.abs(dd).max())
    tf_sel = rng.choice(tf_cand, min(32, tf_cand.size), replace=False)
    dn_sel = rng.choice(dn_cand, 64 - tf_sel.size, replace=False)
    errs = []
    for i in tf_sel:
        p, m = w.tf.copy().ravel(), w.tf.copy().ravel()
        p[i] += eps
        m[i] -= eps
        fd = (loss(p.reshape(-1, 4), dense) - loss(m.reshape(-1, 4), dense)) / (2 * eps)
        errs.append(abs(fd - dtf.ravel()[i]) / max(abs(fd), 1e-3 * np.abs(dtf).max()))
    for i in dn_sel:
        p, m = dense.copy(), dense.copy()
        p[i] += eps
        m[i] -= eps
        fd = (loss(w.tf, p) - loss(w.tf, m)) / (2 * eps)
        errs.append(abs(fd - dd[i]) / max(abs(fd), 1e-3 * np.abs(dd).max()))
    errs = np.array(errs)
    assert len(errs) == 64
    # piecewise-linear transfer functions put kinks inside some +-eps intervals
    assert np.median(errs) < REL_TOL, np.sort(errs)
    assert np.mean(errs < 1e-2) >= 0.9, np.sort(errs)


def test_autograd_binding_matches_the_adjoint(ctx):
    """torch.autograd through revise_gb300.autograd.render_frame gives the same
    gradients as calling s3r_render_argb_backward directly (reductions run in
    another order between the two calls: 1e-5 relative)."""
    import torch
    from revise_gb300.api import FramePlan
    from revise_gb300.autograd import render_frame
    w = _setup(64, 64)
    view = host.view_for(w)
    plan = FramePlan(ctx, w)
    plan.interp(torch.from_numpy(w.sparse).cuda())
    bricks, _ = plan.bricks()
    bricks.requires_grad_(True)
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda().requires_grad_(True)
    target = torch.rand(w.H, w.W, 4, device="cuda")
    img = render_frame(plan, view, tf, bricks)
    loss = 0.5 * ((img - target) ** 2).sum()
    loss.backward()
    rgba = img.detach().reshape(-1).contiguous()
    dl = (img.detach() - target).reshape(-1).contiguous()
    dtf = torch.zeros(w.tf.size, device="cuda")
    dd = torch.zeros(bricks.numel(), device="cuda")
    plan.backward(view, tf.detach(), rgba, dl, dtf, dd)
    torch.cuda.synchronize()
    assert float(tf.grad.abs().max()) > 0
    assert torch.allclose(tf.grad.reshape(-1), dtf, rtol=1e-5, atol=1e-6 * float(dtf.abs().max()))
    assert torch.allclose(bricks.grad, dd, rtol=1e-5, atol=1e-6 * float(dd.abs().max()))
    plan.close()
