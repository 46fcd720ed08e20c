"""Sort-last compositing of image parts across ranks.

The reference renders disjoint index boxes of one block-tree level on separate
workers (IndexCubeSplitter, include/IndexCubeSplitter.hpp), orders the boxes
back to front for the eye (IndexCubeSplitStorage::getBoxesSorted,
src/s3vs_lib/IndexCubeSplitStorage.hpp:54-74) and blends the workers' parts
pairwise up the binary tree RenderGraphGenerator builds
(src/s3vs_lib/RenderGraphGenerator.cpp:37-129), ending with FinalComposeFunc
(src/s3vs_lib/VsRenderer.cpp:403-519).  Here each rank renders one box of the
same split into a cropped ARGB32 part; one gather moves the parts to the
destination rank, which evaluates the same tree with the reference's integer
blend, so the pixels are the reference's (the blend is not associative: the
tree's pairing, not just the order, decides them).
"""
from __future__ import annotations

import numpy as np

from . import schedule


def split_boxes(level: int, parts: int):
    """The reference's split of the (2^level)^3 block cube for `parts` workers (IndexCubeSplitter,
    x fastest): index boxes ((min), (max)), max exclusive.  Fewer boxes than parts when the level
    has fewer blocks along the split axes."""
    return [(tuple(int(v) for v in b[:3]), tuple(int(v) for v in b[3:]))
            for b in schedule.split_index_cube(level, parts)]


def box_order(level: int, boxes, eye, split_count: int | None = None) -> list[int]:
    """Indices of `boxes` (a split_boxes result) in back-to-front order for `eye`."""
    n = len(boxes) if split_count is None else split_count
    where = {(tuple(b[0]), tuple(b[1])): i for i, b in enumerate(boxes)}
    return [where[(tuple(int(v) for v in b[:3]), tuple(int(v) for v in b[3:]))]
            for b in schedule.boxes_sorted(level, n, eye)]


def compose(parts, order, W: int, H: int, background: int = 0, thread_per_node: int | None = None) -> np.ndarray:
    """The final W x H ARGB32 frame from parts [(origin, pixels (h, w) uint32)]: the parts taken in
    `order` (back to front) as the render graph's workers for that many threads
    (thread_per_node workers per node; default: all on one node), assembled pairwise up the tree and
    composed onto the background."""
    ordered = [schedule.Part(tuple(int(v) for v in parts[i][0]), np.ascontiguousarray(parts[i][1], dtype=np.uint32))
               for i in order]
    tpn = thread_per_node or max(1, len(ordered))
    graph = schedule.render_graph(schedule.affinity_for(len(ordered), tpn)) if ordered else schedule.render_graph([])
    return schedule.run_graph(graph, ordered, W, H, background)


def gather_and_compose(part, boxes, level: int, eye, W: int, H: int, group=None, dst: int = 0,
                       thread_per_node: int | None = None, background: int = 0):
    """Collective: every rank passes its own (origin, pixels) part of boxes[rank]; rank `dst`
    returns the composed W x H image, the others None."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    gathered = [None] * world if rank == dst else None
    dist.gather_object(part, gathered, dst=dst, group=group)
    if rank != dst:
        return None
    return compose(gathered, box_order(level, boxes, eye), W, H, background, thread_per_node)
