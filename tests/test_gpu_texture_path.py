"""The texture-unit per-block path (s3r_texture / s3r_tf_texture / s3r_render_block_texture) against the
reference's own renderKernel<mode> (its kernels compiled from its sources and run from cubins,
oracle/refcu_harness.cpp), block by block in back-to-front order into one ARGB8 viewport.  Both sample
through the texture unit and set up their rays with the same float expressions, so the images are
expected to agree to the last bit; the bound checked is at most 1 LSB per channel, and the number of
pixels that differ at all is printed."""
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import refcu
from revise_gb300 import _lib, host

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import mode_scenes as ms  # noqa: E402
import texture_variants as tv  # noqa: E402

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refcu.available(), reason="reference CUDA cubins not built here")]


def _texture_image(ctx, w, view, pres, sparse2, clear):
    import torch
    from revise_gb300.api import to_device_n2i
    vp = torch.full((w.W * w.H,), clear, dtype=torch.int64, device="cuda").to(torch.int32)
    tft = ctx.tf_texture(torch.from_numpy(np.ascontiguousarray(w.tf)).cuda())
    keep = []
    for b in tv.b2f_blocks(w):
        n2i, sp = w.block_nodes(b)
        d = int(w.blocks[b, 3])
        blk = [int(x) for x in w.blocks[b, :3]]
        dn = to_device_n2i(n2i)
        t1 = ctx.texture(d)
        ctx.interp_dense_texture(dn, torch.from_numpy(sp).cuda(), t1)
        t2 = None
        if sparse2 is not None:
            t2 = ctx.texture(d)
            a, c = int(w.node_off[b]), int(w.node_off[b + 1])
            ctx.interp_dense_texture(dn, torch.from_numpy(np.ascontiguousarray(sparse2[a:c])).cuda(), t2)
        ctx.render_block_texture(view, pres, t1, blk, host.block_view_rect(view, blk), tft, vp, tex2=t2)
        keep += [t1, t2]
    torch.cuda.synchronize()
    return vp.cpu().numpy().view(np.uint32)


def _reference_image(w, view, pres, sparse2, clear):
    refcu.set_tf(w.tf)
    ref = np.full(w.W * w.H, clear, np.uint32)
    for b in tv.b2f_blocks(w):
        n2i, sp = w.block_nodes(b)
        blk = [int(x) for x in w.blocks[b, :3]]
        rect = host.block_view_rect(view, blk)
        if pres is None:
            refcu.render_block(view, n2i, sp, int(w.blocks[b, 3]), blk, rect, ref)
        else:
            s2 = None if sparse2 is None else sparse2[int(w.node_off[b]):int(w.node_off[b + 1])]
            refcu.render_block_mode(view, pres, n2i, sp, int(w.blocks[b, 3]), blk, rect, ref, s2)
    return ref


def _lsb(got, ref):
    return np.abs(got.view(np.uint8).reshape(-1, 4).astype(int) - ref.view(np.uint8).reshape(-1, 4).astype(int)).max(1)


@pytest.mark.parametrize("variant", tv.VARIANTS)
def test_argb_texture_path_vs_reference_kernel(ctx, variant):
    w = tv.workload(variant)
    view = host.view_for(w, filter=_lib.FILTER_TEXTURE)
    got = _texture_image(ctx, w, view, None, None, 0)
    ref = _reference_image(w, view, None, None, 0)
    d = _lsb(got, ref)
    print(f"argb {variant}: {(ref >> 24).astype(bool).sum()} covered, {(d > 0).sum()} differ, max {d.max()} LSB")
    assert (ref >> 24).astype(bool).mean() > 0.05
    assert d.max() <= 1, d.max()


@pytest.mark.parametrize("name", list(ms.MODES))
def test_mode_texture_path_vs_reference_kernel(ctx, name):
    w, view, pres, sparse2 = ms.scene(name, _lib.FILTER_TEXTURE)
    clear = ms.clear_value(pres)
    got = _texture_image(ctx, w, view, pres, sparse2, clear)
    ref = _reference_image(w, view, pres, sparse2, clear)
    if pres.mode == _lib.MODE_MAX_INTENSITY:
        a, b = got.view(np.float32), ref.view(np.float32)
        assert np.array_equal(np.isnan(a), np.isnan(b))
        m = ~np.isnan(a)
        print(f"{name}: {m.sum()} covered, {(a[m] != b[m]).sum()} differ, max {np.abs(a[m] - b[m]).max():.2e}")
        assert m.mean() > 0.05
        assert np.abs(a[m] - b[m]).max() <= 1e-6
        return
    d = _lsb(got, ref)
    print(f"{name}: {(ref >> 24).astype(bool).sum()} covered, {(d > 0).sum()} differ, max {d.max()} LSB")
    assert (ref >> 24).astype(bool).mean() > 0.03
    assert d.max() <= 1, d.max()
