"""Multi-rank sort-last compositing on CPU ranks (gloo, world size 2): each rank
renders its box of the reference's split with the oracle ray caster into a
cropped image part, rank 0 gathers them and evaluates the reference's render
graph back to front; the result equals the same composition done in one
process."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
from revise_gb300 import compose, host, workloads


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _render_box(w, box, view):
    (x0, y0, z0), (x1, y1, z1) = box
    sel = [b for b in range(w.nblocks) if x0 <= w.blocks[b, 0] < x1 and y0 <= w.blocks[b, 1] < y1
           and z0 <= w.blocks[b, 2] < z1]
    sub = workloads.Workload(**{**w.__dict__})
    sub.blocks = w.blocks[sel]
    parts_n2i = [w.block_nodes(b) for b in sel]
    sub.n2i = np.concatenate([p[0] for p in parts_n2i])
    sub.sparse = np.concatenate([p[1] for p in parts_n2i])
    sub.node_off = np.concatenate([[0], np.cumsum([p[0].shape[0] for p in parts_n2i])]).astype(np.uint64)
    dense = oracle.interp_workload(sub)
    rects = np.array([host.block_view_rect(view, sub.blocks[i, :3]) for i in range(sub.nblocks)], np.int32)
    img = oracle.render_frame_argb8(oracle.view_from(view), sub, dense, rects, w.tf).reshape(w.H, w.W)
    ys, xs = np.nonzero(img >> 24)
    if ys.size == 0:
        return ((0, 0), np.zeros((0, 0), np.uint32))
    return ((int(xs.min()), int(ys.min())), img[ys.min():ys.max() + 1, xs.min():xs.max() + 1].copy())


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = workloads.small(seed=4, level=1, depths=(2, 3), W=64, H=48)
    view = host.view_for(w)
    boxes = compose.split_boxes(w.level, world)
    part = _render_box(w, boxes[rank], view)
    img = compose.gather_and_compose(part, boxes, w.level, w.eye, w.W, w.H)
    if rank == 0:
        q.put(img)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gather_and_compose_matches_single_process():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    img = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    w = workloads.small(seed=4, level=1, depths=(2, 3), W=64, H=48)
    view = host.view_for(w)
    boxes = compose.split_boxes(w.level, world)
    parts = [_render_box(w, b, view) for b in boxes]
    want = compose.compose(parts, compose.box_order(w.level, boxes, w.eye), w.W, w.H)
    assert np.array_equal(img, want)
    assert (want >> 24).astype(bool).any()


def test_box_order_puts_far_box_first():
    boxes = compose.split_boxes(2, 2)
    assert boxes == [((0, 0, 0), (2, 4, 4)), ((2, 0, 0), (4, 4, 4))]
    assert compose.box_order(2, boxes, (100.0, 0.0, 0.0)) == [0, 1]
    assert compose.box_order(2, boxes, (-100.0, 0.0, 0.0)) == [1, 0]


def test_compose_is_the_render_graph_of_the_sorted_parts():
    rng = np.random.default_rng(1)
    parts = []
    for _ in range(5):
        h, w = int(rng.integers(1, 9)), int(rng.integers(1, 9))
        px = rng.integers(0, 1 << 32, (h, w), dtype=np.uint64).astype(np.uint32)
        parts.append(((int(rng.integers(0, 20)), int(rng.integers(0, 20))), px))
    order = [3, 0, 4, 1, 2]
    from revise_gb300 import schedule
    g = schedule.render_graph(schedule.affinity_for(5, 2))
    want = schedule.run_graph(g, [schedule.Part(parts[i][0], parts[i][1]) for i in order], 32, 32, 5)
    assert np.array_equal(compose.compose(parts, order, 32, 32, 5, thread_per_node=2), want)
