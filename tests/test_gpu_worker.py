"""The native worker loop (s3r_render_scene_part) against the Python worker loop over the same
per-block calls (bit for bit), in the Argb and the field modes, for whole and partial boxes."""
import sys
from pathlib import Path

import numpy as np
import pytest

from revise_gb300 import _lib, host, workloads

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import mode_scenes as ms  # noqa: E402

pytestmark = pytest.mark.gpu


def _img(part, W, H):
    (ox, oy), (w, h), px = part
    out = np.zeros((H, W), np.uint32)
    if w:
        out[oy:oy + h, ox:ox + w] = px.cpu().numpy().view(np.uint32).reshape(h, w)
    return out


@pytest.mark.parametrize("box", [((0, 0, 0), (2, 2, 2)), ((0, 1, 0), (2, 2, 1)), ((1, 0, 1), (2, 2, 2))])
@pytest.mark.parametrize("filt", [_lib.FILTER_EXACT, _lib.FILTER_TEXTURE])
def test_native_argb_equals_python_loop(ctx, box, filt):
    from revise_gb300.api import RenderSharedState, VsWorker
    w = workloads.small(seed=6, level=1, depths=(2, 3, 4), W=96, H=72)
    st = RenderSharedState(w, filter=filt)
    wk = VsWorker(ctx)
    wk.set_render_shared_state(st)
    a = wk.render_scene_part_device(1, *box)
    b = wk.render_scene_part_native(1, *box)
    assert a[0] == b[0] and a[1] == b[1]
    assert np.array_equal(_img(a, w.W, w.H), _img(b, w.W, w.H))
    if box[1] == (2, 2, 2) and box[0] == (0, 0, 0):
        assert a[1][0] > 0


@pytest.mark.parametrize("name", list(ms.MODES))
def test_native_modes_equal_per_block_calls(ctx, name):
    import torch
    from revise_gb300.api import RenderSharedState, VsWorker
    w, view, pres, sparse2 = ms.scene(name, _lib.FILTER_TEXTURE)
    st = RenderSharedState(w, filter=_lib.FILTER_TEXTURE)
    st.view = view
    wk = VsWorker(ctx)
    wk.set_render_shared_state(st)
    s2 = torch.from_numpy(np.ascontiguousarray(sparse2)).cuda() if sparse2 is not None else None
    m = 1 << w.level
    got = wk.render_scene_part_native(w.level, (0, 0, 0), (m, m, m), pres=pres, sparse2_dev=s2)
    # the same calls one by one from Python
    from revise_gb300.api import to_device_n2i
    clear = ms.clear_value(pres)
    vp = torch.full((w.W * w.H,), clear, dtype=torch.int64, device="cuda").to(torch.int32)
    tft = ctx.tf_texture(torch.from_numpy(w.tf).cuda())
    keep = []
    order = host.b2f_order([0, 0, 0], [m, m, m], *host.index_box_world(w.level, [0, 0, 0], [m, m, m]), view.cam.eye[:])
    where = {tuple(b[:3]): i for i, b in enumerate(w.blocks.tolist())}
    for idx in order.tolist():
        b = where[tuple(idx)]
        n2i, sp = w.block_nodes(b)
        d = int(w.blocks[b, 3])
        dn = to_device_n2i(n2i)
        t1 = ctx.texture(d)
        ctx.interp_dense_texture(dn, torch.from_numpy(sp).cuda(), t1)
        t2 = None
        if sparse2 is not None:
            a0, a1 = int(w.node_off[b]), int(w.node_off[b + 1])
            t2 = ctx.texture(d)
            ctx.interp_dense_texture(dn, torch.from_numpy(np.ascontiguousarray(sparse2[a0:a1])).cuda(), t2)
        r = host.block_view_rect(view, idx)
        if r[2] > 0 and r[3] > 0:
            ctx.render_block_texture(view, pres, t1, idx, r, tft, vp, tex2=t2)
        keep += [t1, t2]
    torch.cuda.synchronize()
    want = vp.cpu().numpy().view(np.uint32).reshape(w.H, w.W)
    gimg = _img(got, w.W, w.H)
    if pres.mode == _lib.MODE_MAX_INTENSITY:
        # the native part is cropped to non-transparent pixels (alpha byte != 0), as getBoundRect crops
        (ox, oy), (ww, hh), _ = got
        assert np.array_equal(gimg[oy:oy + hh, ox:ox + ww], want[oy:oy + hh, ox:ox + ww])
    else:
        assert np.array_equal(gimg, want)


@pytest.mark.parametrize("filt", [_lib.FILTER_EXACT, _lib.FILTER_TEXTURE])
def test_scene_part_from_plan_bricks_equals_native_loop(ctx, filt):
    """Rendering from the plan's bricks (interpolated in one launch) gives the image of the same per-block
    render calls on per-block interpolations: the bricks are bit-identical to them.  The plan's bricks are
    linear, so the texture filter is the software restatement of the texture unit there (s3r_render_block);
    the exact filter is also the native worker loop's."""
    import torch
    from revise_gb300.api import FramePlan, RenderSharedState, VsWorker, to_device_n2i
    w = workloads.small(seed=8, level=1, depths=(2, 3, 5), W=96, H=72)
    st = RenderSharedState(w, filter=filt)
    wk = VsWorker(ctx)
    wk.set_render_shared_state(st)
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=8)
    plan.interp(torch.from_numpy(w.sparse).cuda())
    tf = torch.from_numpy(w.tf).cuda()
    for box in [((0, 0, 0), (2, 2, 2)), ((1, 0, 0), (2, 2, 2))]:
        b = wk.render_scene_part_plan(plan, 1, *box)
        if filt == _lib.FILTER_EXACT:
            a = wk.render_scene_part_native(1, *box)
            assert a[0] == b[0] and a[1] == b[1]
            assert np.array_equal(_img(a, w.W, w.H), _img(b, w.W, w.H))
        vp = torch.zeros(w.W * w.H, dtype=torch.int32, device="cuda")
        cmin, cmax = host.index_box_world(1, box[0], box[1])
        where = {tuple(int(x) for x in r[:3]): i for i, r in enumerate(w.blocks)}
        for idx in host.b2f_order(box[0], box[1], cmin, cmax, st.view.cam.eye[:]).tolist():
            k = where.get(tuple(idx))
            if k is None:
                continue
            n2i, sp = w.block_nodes(k)
            d = int(w.blocks[k, 3])
            dense = ctx.interp_dense(to_device_n2i(n2i), torch.from_numpy(sp).cuda(), d)
            r = host.block_view_rect(st.view, idx)
            if r[2] > 0 and r[3] > 0:
                ctx.render_block_argb(st.view, dense, d, idx, r, tf, vp)
        torch.cuda.synchronize()
        want = vp.cpu().numpy().view(np.uint32).reshape(w.H, w.W)
        assert np.array_equal(_img(b, w.W, w.H), want)
        assert (want >> 24).any()
    plan.close()


@pytest.mark.parametrize("render_tile", [0, _lib.RENDER_TILES_WALK + 1])
def test_frame_run_host_pipeline_matches_device_frames(ctx, render_tile):
    """s3r_frame_run_host over several frames with changing sparse values: every image equals the one
    s3r_frame_run makes from device buffers (the two slots alternate and never mix frames), with the
    per-ray walk and with the block-major render (per-slot result buffers, masks and counters)."""
    import torch
    from revise_gb300 import host
    from revise_gb300.api import FramePlan
    w = workloads.small(seed=21, level=1, depths=(2, 3, 4), W=80, H=64)
    view = host.view_for(w)
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=8, render_tile=render_tile)
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    rng = np.random.default_rng(3)
    frames = [(w.sparse * np.float32(1 + 0.1 * k) + np.float32(rng.normal())).astype(np.float32) for k in range(5)]
    frames = [np.where(w.sparse == np.float32(1e30), np.float32(1e30), f).astype(np.float32) for f in frames]
    want = []
    for f in frames:
        argb = torch.zeros(w.W * w.H, dtype=torch.int32, device="cuda")
        plan.run(view, torch.from_numpy(f).cuda(), tf, None, argb)
        want.append(argb.cpu().numpy())
    hosts = [torch.from_numpy(f).pin_memory() for f in frames]
    imgs = [torch.zeros(w.W * w.H, dtype=torch.int32).pin_memory() for _ in frames]
    for f, im in zip(hosts, imgs):
        plan.run_host(view, f, tf, im)
    plan.host_sync()
    for k in range(len(frames)):
        assert np.array_equal(imgs[k].numpy(), want[k]), k
    assert len({x.tobytes() for x in want}) == len(want)  # the frames differ
    plan.close()


@pytest.mark.parametrize("render_tile", [0, _lib.RENDER_TILES_WALK])
@pytest.mark.parametrize("fmt", [_lib.BRICK_F32, _lib.BRICK_F16, _lib.BRICK_BF16])
def test_frame_run_host_view_change_and_tf_reuse(ctx, fmt, render_tile):
    """s3r_frame_run_host with 16-bit bricks in both slots (the second slot's per-brick scales) and a view
    that changes mid-sequence (frames 0-2 one camera, 3-5 another, while the other slot is in flight);
    after every call the caller overwrites its transfer function on the same stream, which the frame
    must not see.  Every image equals s3r_frame_run's from device buffers, bit for bit."""
    import torch
    from revise_gb300 import host
    from revise_gb300.api import FramePlan
    w = workloads.small(seed=23, level=1, depths=(2, 3, 4), W=80, H=64)
    views = [host.view_for(w), host.view_for(w, eye=(3.0, 12.0, 30.0))]
    plan = FramePlan(ctx, w, fmt, tile_cells=8, render_tile=render_tile)
    tf0 = np.ascontiguousarray(w.tf)
    rng = np.random.default_rng(5)
    frames = [(w.sparse * np.float32(1 + 0.1 * k) + np.float32(rng.normal())).astype(np.float32) for k in range(6)]
    frames = [np.where(w.sparse == np.float32(1e30), np.float32(1e30), f).astype(np.float32) for f in frames]
    vsel = [0, 0, 0, 1, 1, 1]
    want = []
    tf_dev = torch.from_numpy(tf0).cuda()
    for f, vi in zip(frames, vsel):
        argb = torch.zeros(w.W * w.H, dtype=torch.int32, device="cuda")
        plan.run(views[vi], torch.from_numpy(f).cuda(), tf_dev, None, argb)
        want.append(argb.cpu().numpy())
    hosts = [torch.from_numpy(f).pin_memory() for f in frames]
    imgs = [torch.zeros(w.W * w.H, dtype=torch.int32).pin_memory() for _ in frames]
    tf_work = torch.from_numpy(tf0).cuda()
    garbage = torch.from_numpy(np.full_like(tf0, 0.5)).cuda()
    for f, im, vi in zip(hosts, imgs, vsel):
        tf_work.copy_(torch.from_numpy(tf0).cuda())
        plan.run_host(views[vi], f, tf_work, im)
        tf_work.copy_(garbage)  # queued on the same stream after the call: the frame keeps the old table
    plan.host_sync()
    for k in range(len(frames)):
        assert np.array_equal(imgs[k].numpy(), want[k]), k
    assert len({x.tobytes() for x in want}) == len(want)
    plan.close()
