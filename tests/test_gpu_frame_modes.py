"""Batched frame in every field mode (s3r_frame_render_mode): the plan's blocks marched per ray
front to back as the per-block renderer marches them, composited in FP32, against the oracle's
restatement of the same composition (both filters)."""
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from revise_gb300 import _lib, host

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import mode_scenes as ms  # noqa: E402

pytestmark = pytest.mark.gpu


def _gpu(ctx, w, view, pres, sparse2):
    import torch
    from revise_gb300.api import FramePlan
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=8)
    plan.interp(torch.from_numpy(w.sparse).cuda())
    plan2 = None
    bricks2 = None
    if sparse2 is not None:
        plan2 = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=8)
        plan2.interp(torch.from_numpy(np.ascontiguousarray(sparse2)).cuda())
        bricks2, _ = plan2.bricks()
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    rgba = torch.full((w.W * w.H * 4,), -1.0, device="cuda")
    argb = torch.zeros(w.W * w.H, dtype=torch.int32, device="cuda")
    plan.render_mode(view, pres, tf, bricks2, rgba, argb)
    torch.cuda.synchronize()
    out = rgba.cpu().numpy().reshape(-1, 4), argb.cpu().numpy().view(np.uint32)
    plan.close()
    if plan2 is not None:
        plan2.close()
    return out


def _oracle(w, view, pres, sparse2):
    dense = oracle.interp_workload(w)
    dense2 = None
    if sparse2 is not None:
        import dataclasses
        dense2 = oracle.interp_workload(dataclasses.replace(w, sparse=sparse2))
    rects = np.array([host.block_view_rect(view, w.blocks[b, :3]) for b in range(w.nblocks)], np.int32)
    return oracle.render_frame_mode(oracle.view_from(view), oracle.presentation_from(pres), w, dense, rects, w.tf,
                                    view.alpha_stop, dense2)


@pytest.mark.parametrize("filt", [_lib.FILTER_EXACT, _lib.FILTER_TEXTURE])
@pytest.mark.parametrize("name", list(ms.MODES))
def test_frame_mode_vs_oracle(ctx, name, filt):
    w, view, pres, sparse2 = ms.scene(name, filt)
    got, argb = _gpu(ctx, w, view, pres, sparse2)
    want = _oracle(w, view, pres, sparse2)
    assert (got >= 0).all()  # every pixel written
    if pres.mode == _lib.MODE_MAX_INTENSITY:
        assert np.array_equal(got[:, 3], want[:, 3])
        m = got[:, 3] > 0
        assert m.mean() > 0.05
        assert np.abs(got[m, 0] - want[m, 0]).max() <= 1e-4
        assert np.array_equal(argb[m].view(np.float32), got[m, 0]) and np.isnan(argb[~m].view(np.float32)).all()
        return
    d = np.abs(got - want).max(1)
    print(f"{name} filter {filt}: {(d > 2e-3).sum()} of {d.size} pixels beyond 2e-3, max {d.max():.3e}, "
          f"median {np.median(d):.2e}")
    assert (want[:, 3] > 0).mean() > 0.03
    # FP32 both sides in the same order: every pixel within the image tolerance (measured: at most 2.8e-5)
    assert d.max() <= 2e-3, d.max()
    assert np.median(d) <= 1e-5


def test_frame_mode_argb_equals_frame_render(ctx):
    """MODE_ARGB through the mode kernel gives the plain batched render's image (same samples,
    the per-block compositing order aside) within FP32 rounding."""
    import torch
    from revise_gb300.api import FramePlan
    w, view, pres, _ = ms.scene("isosurface", _lib.FILTER_EXACT)
    view = host.view_for(w)
    pres = host.presentation(_lib.MODE_ARGB, view)
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=8)
    plan.interp(torch.from_numpy(w.sparse).cuda())
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    a = torch.zeros(w.W * w.H * 4, device="cuda")
    b = torch.zeros(w.W * w.H * 4, device="cuda")
    plan.render_mode(view, pres, tf, None, a, None)
    plan.render(view, tf, b)
    torch.cuda.synchronize()
    assert (a - b).abs().max().item() <= 2e-3
    plan.close()


def test_frame_mode_rejects_missing_secondary_and_16bit(ctx):
    import torch
    from revise_gb300.api import FramePlan
    w, view, pres, sparse2 = ms.scene("value_on_isosurface", _lib.FILTER_EXACT)
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=8)
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    with pytest.raises(_lib.S3RError, match="secondary"):
        plan.render_mode(view, pres, tf, None, torch.zeros(w.W * w.H * 4, device="cuda"))
    plan.close()
    plan = FramePlan(ctx, w, _lib.BRICK_F16, tile_cells=8)
    p2 = host.presentation(_lib.MODE_ISOSURFACE, view)
    with pytest.raises(_lib.S3RError, match="F32"):
        plan.render_mode(view, p2, tf, None, torch.zeros(w.W * w.H * 4, device="cuda"))
    plan.close()
