"""Sort-last compositing of image parts across ranks.

The reference renders disjoint index boxes of one block-tree level on separate
workers and blends their image parts pairwise in back-to-front box order
(RenderGraphGenerator.cpp:37-129 builds the binary tree, AssembleFunc /
FinalComposeFunc in VsRenderer.cpp:403-519 run blendImagePart).  Here each
rank renders its box into one cropped ARGB32 part; one gather moves the parts
to the destination rank, which blends them in back-to-front box order on top
of the background with the reference's integer blend.  A binary tree of
pairwise blends in that order gives the same pixels, because every blend is
applied to whole parts in the same sequence per pixel.
"""
from __future__ import annotations

import numpy as np

from . import host


def split_boxes(level: int, parts: int):
    """Splits the (2^level)^3 block cube into `parts` slabs along x (index boxes [min, max))."""
    m = 1 << level
    if parts > m:
        raise ValueError("more parts than block columns")
    cuts = np.linspace(0, m, parts + 1).round().astype(int)
    return [((int(cuts[i]), 0, 0), (int(cuts[i + 1]), m, m)) for i in range(parts)]


def box_order(level: int, boxes, eye) -> list[int]:
    """Back-to-front order of index boxes (IndexCubeSplitStorage::getBoxesSorted,
    src/s3vs_lib/IndexCubeSplitStorage.hpp:66-74): boxes sorted by the
    back-to-front order of their first blocks over the whole cube."""
    m = 1 << level
    cmin, cmax = host.index_box_world(level, (0, 0, 0), (m, m, m))
    order = host.b2f_order((0, 0, 0), (m, m, m), cmin, cmax, eye)
    rank_of = {tuple(int(x) for x in b): i for i, b in enumerate(order.tolist())}
    first = []
    for bmin, bmax in boxes:
        best = min(rank_of[(x, y, z)] for x in range(bmin[0], bmax[0]) for y in range(bmin[1], bmax[1])
                   for z in range(bmin[2], bmax[2]))
        first.append(best)
    return sorted(range(len(boxes)), key=lambda i: first[i])


def compose(parts, order, W: int, H: int, background: int = 0) -> np.ndarray:
    """Blends parts [(origin, pixels (h, w) uint32)] in `order` onto a W x H background."""
    img = np.full((H, W), background, dtype=np.uint32)
    for i in order:
        origin, pix = parts[i]
        if pix.size:
            host.blend_image_part(img, np.ascontiguousarray(pix, dtype=np.uint32), origin)
    return img


def gather_and_compose(part, boxes, level: int, eye, W: int, H: int, group=None, dst: int = 0):
    """Collective: every rank passes its own (origin, pixels) part; rank `dst`
    returns the composed W x H image, the others None."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    gathered = [None] * world if rank == dst else None
    dist.gather_object(part, gathered, dst=dst, group=group)
    if rank != dst:
        return None
    return compose(gathered, box_order(level, boxes, eye), W, H)
