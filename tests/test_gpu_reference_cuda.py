"""The reference's own CUDA kernels, run on the GPU from cubins compiled from its
sources (oracle/refcu_harness.cpp), against this library's kernels on the same
inputs.  Skipped where the cubins were not built (they need the reference tree)."""
import numpy as np
import pytest

from oracle import refcu
from revise_gb300 import host, workloads

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refcu.available(), reason="reference CUDA cubins not built here")]


def _same_mask(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b))


@pytest.mark.parametrize("seed", [0, 3])
def test_reference_cuda_interpolation_matches(ctx, seed):
    """The reference GPU interpolator sums in its own order: NaN masks agree
    exactly, values within 1e-6 relative (floored at 1e-6 of the field scale)."""
    import torch
    from revise_gb300.api import to_device_n2i
    w = workloads.small(seed=seed, level=1, depths=(2, 4, 6), mask_fraction=0.2)
    for b in range(w.nblocks):
        n2i, sp = w.block_nodes(b)
        d = int(w.blocks[b, 3])
        ref = refcu.interp(n2i, sp, d)
        got = ctx.interp_dense(to_device_n2i(n2i), torch.from_numpy(sp).cuda(), d).cpu().numpy()
        assert _same_mask(got, ref), b
        m = ~np.isnan(ref)
        scale = np.abs(sp[sp != np.float32(1e30)]).max()
        assert np.all(np.abs(got[m] - ref[m]) <= 1e-6 * np.maximum(np.abs(ref[m]), scale)), b


def test_reference_cuda_render_matches_block_by_block(ctx):
    """Whole worker frames, block by block in back-to-front order: the reference's
    renderKernel<Argb> (texture-unit filtering with 8-bit fractions) against the
    exact-FP32-filtering plain kernel; both quantize to ARGB8 after every block."""
    import torch
    from revise_gb300.api import to_device_n2i
    w = workloads.small(seed=2, level=1, depths=(3, 4), W=160, H=120, mask_fraction=0.1)
    view = host.view_for(w)
    w_tf = np.ascontiguousarray(w.tf, dtype=np.float32)
    refcu.set_tf(w_tf)
    order = host.b2f_order([0, 0, 0], [2, 2, 2], [-5.0] * 3, [5.0] * 3, w.eye)
    idx = {tuple(b[:3]): i for i, b in enumerate(w.blocks.tolist())}
    ref = np.zeros(w.W * w.H, np.uint32)
    vp = torch.zeros(w.W * w.H, dtype=torch.int32, device="cuda")
    tf = torch.from_numpy(w_tf).cuda()
    for blk in order.tolist():
        b = idx[tuple(blk)]
        n2i, sp = w.block_nodes(b)
        d = int(w.blocks[b, 3])
        rect = host.block_view_rect(view, blk)
        refcu.render_block(view, n2i, sp, d, blk, rect, ref)
        dense = ctx.interp_dense(to_device_n2i(n2i), torch.from_numpy(sp).cuda(), d)
        ctx.render_block_argb(view, dense, d, blk, rect, tf, vp)
    got = vp.cpu().numpy().view(np.uint32)
    a = got.view(np.uint8).reshape(-1, 4).astype(int)
    r = ref.view(np.uint8).reshape(-1, 4).astype(int)
    diff = np.abs(a - r).max(axis=1)
    assert (ref >> 24).astype(bool).mean() > 0.05
    # texture filtering quantizes interpolation fractions to 1/256: a few LSB where the field is steep
    assert np.mean(diff) < 0.5, np.mean(diff)
    assert np.percentile(diff, 99) <= 4, np.percentile(diff, 99)
