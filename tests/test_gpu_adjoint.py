"""Hand-written adjoint of the batched ray caster on the differentiation configuration (2x2x2 blocks of
depth 6, 512x512): GPU gradient vs the FP64 oracle gradient (relative error < 1e-3) and vs central finite
differences (eps = 1e-3) of the FP64 oracle forward at 64 coordinates, each below 1e-3."""
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


def _keep(ov, w, dense, rects):
    """Pixels where no block-local early-termination test lands within 1e-5 of its threshold (the FP64
    oracle flags the others): there float and FP64 arithmetic keep the same sample sets."""
    _, flags = oracle.render_frame_f64(ov, w, dense, rects, w.tf)
    return flags == 0


def test_adjoint_matches_fp64_gradient(ctx):
    """cfg5 at its full 512x512: the GPU gradients of the loss over the kept pixels against the FP64
    oracle's gradients of the same loss, relative error (2-norm over all coordinates) below 1e-3."""
    w = _setup(512, 512)
    view = host.view_for(w)
    ov = oracle.view_from(view)
    dense = oracle.interp_workload(w)
    rects = _rects(w, view)
    target, _ = oracle.render_frame_f64(ov, w, dense, rects, w.meta["target_tf"])
    keep = _keep(ov, w, dense, rects)
    assert keep.mean() > 0.97
    p = np.arange(w.W * w.H)[keep]
    pixels = np.stack([p % w.W, w.H - 1 - p // w.W], 1)
    loss64, dtf64, dd64 = oracle.render_frame_grad_f64(ov, w, dense, rects, w.tf, target[keep], pixels)
    view, loss, dtf, dd = _gpu_grad(ctx, w, target, keep)
    assert abs(loss - loss64) <= 1e-4 * loss64
    e_tf = np.linalg.norm(dtf - dtf64) / np.linalg.norm(dtf64)
    m = ~np.isnan(dense)
    e_dd = np.linalg.norm(dd[m] - dd64[m]) / np.linalg.norm(dd64[m])
    print(f"adjoint vs FP64 gradient (512x512): transfer function {e_tf:.2e}, dense values {e_dd:.2e}")
    assert e_tf < REL_TOL, e_tf
    assert e_dd < REL_TOL, e_dd


def test_adjoint_vs_central_differences(ctx):
    """cfg5 at its full 512x512, loss over the kept pixels: 32 transfer-function entries and 32 dense
    values, each GPU gradient within 1e-3 relative of the central difference (eps 1e-3) of the FP64
    oracle's loss -- every one of the 64, no median.  Coordinates are drawn at random among those with a
    gradient above 1e-3 of the largest and kept only where the loss is smooth across +-eps: the central
    differences at eps and eps/2 agree to 2e-4 (a kink of the piecewise-linear transfer function or an
    early-termination switch inside the interval shows up as a disagreement).  The selection uses the
    oracle alone."""
    import os
    from oracle import fd
    w = _setup(512, 512)
    view = host.view_for(w)
    ov = oracle.view_from(view)
    dense = oracle.interp_workload(w)
    rects = _rects(w, view)
    target, _ = oracle.render_frame_f64(ov, w, dense, rects, w.meta["target_tf"])
    keep = _keep(ov, w, dense, rects)
    pool = fd.LossPool(ov, w, dense, rects, w.tf, target, keep, processes=min(16, os.cpu_count() or 1))
    _, _, dtf, dd = _gpu_grad(ctx, w, target, keep)
    cam = view.cam
    eps = 1e-3
    rng = np.random.default_rng(64)

    def fd_pairs(kind, base, idx, pix):
        """FD at eps and eps/2 for each index (the actual float32 steps as denominators)."""
        jobs, steps = [], []
        for i, px in zip(idx, pix):
            x = np.float32(base[i])
            row = []
            for e in (eps, eps / 2):
                p, m = np.float32(x + np.float32(e)), np.float32(x - np.float32(e))
                jobs += [(kind, int(i), float(p), px), (kind, int(i), float(m), px)]
                row.append(float(p) - float(m))
            steps.append(row)
        L = pool.losses(jobs)
        out = []
        for k, (s1, s2) in enumerate(steps):
            out.append(((L[4 * k] - L[4 * k + 1]) / s1, (L[4 * k + 2] - L[4 * k + 3]) / s2))
        return out

    def dense_pixels(i):
        b = int(np.searchsorted(w.vertex_off, i, side="right") - 1)
        d = int(w.blocks[b, 3])
        e = (1 << d) + 1
        o = i - int(w.vertex_off[b])
        v = np.array([o % e, (o // e) % e, o // (e * e)], np.float64)
        c, h = host.block_cube(w.level, w.blocks[b, :3])
        texel = 2.0 * float(h) / e
        hh = float(h) + 0.5 * texel
        lo = np.asarray(c, np.float64) - hh + (v - 0.5) * (2 * hh / e)
        hi = np.asarray(c, np.float64) - hh + (v + 1.5) * (2 * hh / e)
        return fd.influence_pixels(cam, w.W, w.H, lo, hi)

    checked = []
    try:
        for kind, grad, base, want in (("tf", dtf.ravel(), w.tf.ravel(), 32), ("dense", dd, dense, 32)):
            cand = np.flatnonzero(np.abs(grad) > 1e-3 * np.abs(grad).max())
            cand = rng.permutation(cand)
            got = 0
            for start in range(0, cand.size, 16):
                idx = cand[start:start + 16]
                pix = [None] * idx.size if kind == "tf" else [dense_pixels(int(i)) for i in idx]
                for i, (f1, f2) in zip(idx, fd_pairs(kind, base, idx, pix)):
                    if abs(f1) <= 1e-3 * np.abs(grad).max() or abs(f1 - f2) > 2e-4 * abs(f1):
                        continue  # negligible, or not smooth across the interval
                    checked.append((kind, int(i), float(grad[i]), f1, abs(grad[i] - f1) / abs(f1)))
                    got += 1
                    if got == want:
                        break
                if got == want:
                    break
            assert got == want, (kind, got)
    finally:
        pool.close()
    errs = np.array([c[4] for c in checked])
    print(f"adjoint vs central differences (512x512, 64 coordinates): max {errs.max():.2e}, "
          f"median {np.median(errs):.2e}")
    assert len(checked) == 64
    assert errs.max() < REL_TOL, sorted(checked, key=lambda c: -c[4])[:5]


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
