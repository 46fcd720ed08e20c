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


def test_texture_filter_matches_reference_cuda_renderer(ctx):
    """The plain per-block kernel with S3R_FILTER_TEXTURE against the reference's
    own renderKernel<Argb> (hardware tex3D/tex1D), block by block in back-to-front
    order into one ARGB8 viewport, on scenes with masked nodes: equal but for
    isolated 1-2 LSB differences (weighted sums rounded in another order, powf)."""
    import sys
    from pathlib import Path
    import torch
    from revise_gb300 import _lib
    from revise_gb300.api import to_device_n2i
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import texture_variants as tv
    for variant in tv.VARIANTS:
        w = tv.workload(variant)
        view = host.view_for(w, filter=_lib.FILTER_TEXTURE)
        refcu.set_tf(w.tf)
        ref = np.zeros(w.W * w.H, np.uint32)
        vp = torch.zeros(w.W * w.H, dtype=torch.int32, device="cuda")
        tf = torch.from_numpy(w.tf).cuda()
        for b in tv.b2f_blocks(w):
            n2i, sp = w.block_nodes(b)
            d = int(w.blocks[b, 3])
            blk = [int(x) for x in w.blocks[b, :3]]
            rect = host.block_view_rect(view, blk)
            refcu.render_block(view, n2i, sp, d, blk, rect, ref)
            dense = ctx.interp_dense(to_device_n2i(n2i), torch.from_numpy(sp).cuda(), d)
            ctx.render_block_argb(view, dense, d, blk, rect, tf, vp)
        got = vp.cpu().numpy().view(np.uint32)
        diff = np.abs(got.view(np.uint8).reshape(-1, 4).astype(int) - ref.view(np.uint8).reshape(-1, 4).astype(int)).max(1)
        assert (ref >> 24).astype(bool).mean() > 0.05
        assert diff.max() <= 2, (variant, diff.max())
        assert (diff > 0).mean() < 0.01, (variant, (diff > 0).mean())
