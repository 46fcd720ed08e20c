"""Device-side split/compose scheduling: the render graph's assemble tree and final compose on
device image parts (s3r_compose_parts) against the host evaluation, and the progressive level loop
(VsRenderer) over a reference-format dataset against the oracle's worker images pushed through
the same graph."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from revise_gb300 import _lib, host, schedule, workloads
from revise_gb300.dataset import BlockTreeFieldService

pytestmark = pytest.mark.gpu

DATA = Path(__file__).resolve().parent / "golden" / "dataset"


def _rand_parts(rng, n, W, H):
    parts = []
    for _ in range(n):
        if rng.random() < 0.15:
            parts.append(schedule.Part((0, 0), np.zeros((0, 0), np.uint32)))
            continue
        w, h = int(rng.integers(1, 50)), int(rng.integers(1, 40))
        ox, oy = int(rng.integers(0, W - w)), int(rng.integers(0, H - h))
        a = rng.integers(0, 256, (h, w)).astype(np.uint32)
        a[rng.random((h, w)) < 0.25] = 255
        a[rng.random((h, w)) < 0.25] = 0
        parts.append(schedule.Part((ox, oy), (a << 24) | rng.integers(0, 1 << 24, (h, w)).astype(np.uint32)))
    return parts


def _to_device(p):
    import torch
    if not p.pixels.size:
        return schedule.DevicePart((0, 0), (0, 0), torch.zeros(1, dtype=torch.int32, device="cuda"))
    t = torch.from_numpy(np.ascontiguousarray(p.pixels).view(np.int32).ravel()).cuda()
    return schedule.DevicePart(p.origin, p.size, t)


@pytest.mark.parametrize("affinity", [[1], [2], [3], [4], [4, 3], [2, 2, 1], [1, 1, 1, 1, 1]])
def test_device_graph_equals_host_graph(ctx, affinity):
    rng = np.random.default_rng(sum(affinity) * 7 + len(affinity))
    W, H = 120, 90
    g = schedule.render_graph(affinity)
    for _ in range(4):
        parts = _rand_parts(rng, sum(affinity), W, H)
        want = schedule.run_graph(g, parts, W, H, background=0xFF203040)
        got = schedule.run_graph_device(ctx, g, [_to_device(p) for p in parts], W, H, background=0xFF203040)
        assert np.array_equal(got.cpu().numpy().view(np.uint32).reshape(H, W), want), affinity


def _oracle_box_part(state, level, box):
    w = state.w
    sel = [b for b in range(w.nblocks)
           if all(box[a] <= int(w.blocks[b, a]) < box[3 + a] for a in range(3))]
    if not sel:
        return schedule.Part((0, 0), np.zeros((0, 0), np.uint32))
    import dataclasses
    parts = [w.block_nodes(b) for b in sel]
    sub = dataclasses.replace(w, blocks=w.blocks[sel], n2i=np.concatenate([p[0] for p in parts]),
                              sparse=np.concatenate([p[1] for p in parts]),
                              node_off=np.concatenate([[0], np.cumsum([p[0].shape[0] for p in parts])]).astype(np.uint64))
    dense = oracle.interp_workload(sub)
    rects = np.array([host.block_view_rect(state.view, sub.blocks[i, :3]) for i in range(sub.nblocks)], np.int32)
    img = oracle.render_frame_argb8(oracle.view_from(state.view), sub, dense, rects, w.tf).reshape(w.H, w.W)
    ys, xs = np.nonzero(img >> 24)
    if ys.size == 0:
        return schedule.Part((0, 0), np.zeros((0, 0), np.uint32))
    return schedule.Part((int(xs.min()), int(ys.min())), img[ys.min():ys.max() + 1, xs.min():xs.max() + 1].copy())


def _channels(img):
    return np.stack([(img >> s) & 0xFF for s in (0, 8, 16, 24)], -1).astype(np.int32)


def _reference_box_part(state, level, box):
    """The reference's own CUDA worker loop (renderKernel<Argb> from its cubins, texture unit) over the box's
    blocks in back-to-front order, cropped as getBoundRect crops."""
    from oracle import refcu
    w = state.w
    sel = [b for b in range(w.nblocks) if all(box[a] <= int(w.blocks[b, a]) < box[3 + a] for a in range(3))]
    if not sel:
        return schedule.Part((0, 0), np.zeros((0, 0), np.uint32))
    cmin, cmax = host.index_box_world(level, box[:3], box[3:])
    order = host.b2f_order(box[:3], box[3:], cmin, cmax, state.view.cam.eye[:])
    where = {tuple(int(x) for x in w.blocks[b, :3]): b for b in sel}
    oi = np.array([where[tuple(int(x) for x in q)] for q in order.tolist() if tuple(int(x) for x in q) in where])
    rects = np.array([host.block_view_rect(state.view, w.blocks[b, :3]) for b in range(w.nblocks)], np.int32)
    refcu.set_tf(np.ascontiguousarray(w.tf, np.float32))
    img, _, _ = refcu.worker(state.view, w, oi, rects)
    img = img.reshape(w.H, w.W)
    ys, xs = np.nonzero(img >> 24)
    if ys.size == 0:
        return schedule.Part((0, 0), np.zeros((0, 0), np.uint32))
    return schedule.Part((int(xs.min()), int(ys.min())), img[ys.min():ys.max() + 1, xs.min():xs.max() + 1].copy())


@pytest.mark.parametrize("filt", [_lib.FILTER_EXACT, _lib.FILTER_TEXTURE])
@pytest.mark.parametrize("workers,per_node", [(4, 4), (3, 2), (8, 4)])
def test_progressive_levels_over_dataset(ctx, workers, per_node, filt):
    """Exact filter: each worker part against the oracle's image of its box; texture filter (the workers
    sample through the texture unit): against the reference's own CUDA worker loop over the box."""
    from oracle import refcu
    if filt == _lib.FILTER_TEXTURE and not refcu.available():
        pytest.skip("reference CUDA cubins not built here")
    template = workloads.small(seed=2, level=1, W=96, H=72, eye=(4.0, 7.0, 16.0))
    with BlockTreeFieldService(str(DATA / "shell.dat")) as svc:
        levels = list(range(svc.metadata().max_full_level() + 1))
        states = schedule.dataset_level_states(svc, levels, 0, 0, template, filter=filt)
        r = schedule.VsRenderer(ctx, states, node_count=(workers + per_node - 1) // per_node,
                                thread_per_node=per_node, background=0xFF000000)
        r.split.set_split_count(workers)
        frames = list(r.continue_rendering(template.eye))
        assert [lv for lv, _ in frames] == levels
        for lv, frame in frames:
            st = states[lv]
            got = frame.cpu().numpy().view(np.uint32).reshape(template.H, template.W)
            boxes = r.split.get_boxes_sorted(lv)
            g = schedule.render_graph(schedule.affinity_for(boxes.shape[0], per_node))
            # the device tree over the device parts is the host tree over the same parts, bit for bit
            dev_parts = [schedule.Part(p.origin, p.pixels.cpu().numpy().view(np.uint32).reshape(p.size[1], p.size[0])
                                       if p.size[0] else np.zeros((0, 0), np.uint32)) for p in r.last_parts[lv]]
            assert np.array_equal(schedule.run_graph(g, dev_parts, template.W, template.H, 0xFF000000), got)
            # and the checker's worker images through the same graph agree to the render tolerance
            box_part = _oracle_box_part if filt == _lib.FILTER_EXACT else _reference_box_part
            want = schedule.run_graph(g, [box_part(st, lv, b) for b in boxes], template.W, template.H, 0xFF000000)
            d = np.abs(_channels(got) - _channels(want)).max(-1)
            assert d.max() <= 1 and (d > 0).mean() < 0.02, (lv, d.max(), (d > 0).mean())
            assert (_channels(got)[..., :3] > 0).any()


def test_render_level_option_renders_one_level(ctx):
    template = workloads.small(seed=2, level=1, W=64, H=48)
    with BlockTreeFieldService(str(DATA / "shell.dat")) as svc:
        states = schedule.dataset_level_states(svc, [0, 1], 1, 0, template)
        r = schedule.VsRenderer(ctx, states, thread_per_node=2)
        assert [lv for lv, _ in r.continue_rendering(template.eye, render_level=1)] == [1]
        assert [lv for lv, _ in r.continue_rendering(template.eye, render_level=5)] == [1]
