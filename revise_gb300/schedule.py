"""Work split and compose scheduling of one frame, and the progressive level loop.

The reference renders a frame level by level (VsRenderer::continueRendering,
src/s3vs_lib/VsRenderer.cpp:1061-1163): for each level from the coarsest up to
the metadata's max full level it cuts the level's block cube into one index box
per render worker (IndexCubeSplitter, include/IndexCubeSplitter.hpp), sorts the
boxes back to front for the eye (IndexCubeSplitStorage,
src/s3vs_lib/IndexCubeSplitStorage.hpp), lets each worker render its box into a
cropped image part, blends the parts pairwise up a binary tree
(RenderGraphGenerator, src/s3vs_lib/RenderGraphGenerator.cpp:37-129; AssembleFunc,
VsRenderer.cpp:403-469) and finally onto the background (FinalComposeFunc,
:471-519), emitting one frame per level.

Here the split and the order come from the C ABI (s3r_split_index_cube,
s3r_split_b2f), the graph is restated in `render_graph`, and `VsRenderer` runs
the whole loop on one GPU with every image part, assemble and final compose in
device memory (s3r_crop, s3r_compose_parts); only the finished frame of a level
comes back to the host.  The integer blend is not associative, so the tree's
pairing is kept exactly: the parts are blended in the reference's order.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib, host
from ._lib import arr, check


# ------------------------------------------------------------------ split

def split_index_cube(level: int, split_count: int, add_trailing_empty: bool = False) -> np.ndarray:
    """IndexCubeSplitter<3>(level, split_count, [-5,5]^3).all_blocks(...): (n, 6) uint32 boxes
    {min x, y, z, max x, y, z}, max exclusive, empty boxes all zero."""
    lib = _lib.load()
    cap = max(split_count, 1)
    out = np.zeros((cap, 6), dtype=np.uint32)
    n = C.c_uint32()
    check(lib.s3r_split_index_cube(level, split_count, 1 if add_trailing_empty else 0, arr(out, C.c_uint32), cap,
                                   C.byref(n)))
    return out[: n.value]


def boxes_sorted(level: int, split_count: int, eye) -> np.ndarray:
    """The split's boxes back to front for `eye` (IndexCubeSplitStorage::getBoxesSorted)."""
    lib = _lib.load()
    cap = max(split_count, 1)
    out = np.zeros((cap, 6), dtype=np.uint32)
    n = C.c_uint32()
    e = (C.c_double * 3)(*[float(v) for v in eye])
    check(lib.s3r_split_b2f(level, split_count, e, arr(out, C.c_uint32), cap, C.byref(n)))
    return out[: n.value]


class IndexCubeSplitStorage:
    """IndexCubeSplitStorage: the split count and eye the sorted boxes of every level come from."""

    def __init__(self):
        self.split_count = 1
        self.eye = (0.0, 0.0, 10.0)

    def set_split_count(self, n: int):
        self.split_count = int(n)

    def set_eye_position(self, eye):
        self.eye = tuple(float(v) for v in eye)

    def get_boxes_sorted(self, level: int) -> np.ndarray:
        return boxes_sorted(level, self.split_count, self.eye)


# ------------------------------------------------------------------ render graph

RENDER, ASSEMBLE, FINAL_COMPOSE = "Render", "Assemble", "FinalCompose"


@dataclass
class Task:
    kind: str
    node: int
    inputs: list = field(default_factory=list)  # task ids feeding inputs 0, 1


@dataclass
class RenderGraph:
    tasks: list
    worker_tasks: list      # render task ids, in worker (= sorted box) order
    compose_task: int       # the FinalCompose task, -1 when there is no worker


def render_graph(affinity) -> RenderGraph:
    """RenderGraphGenerator::updateGraph: per node `affinity[node]` render tasks, their parts
    assembled pairwise (neighbours (0,1), (2,3), ...; an odd last one passes up) layer by layer
    into one part per node, the nodes' parts assembled the same way, then one FinalCompose."""
    tasks: list = []

    def add(kind, node, inputs=()):
        tasks.append(Task(kind, node, list(inputs)))
        return len(tasks) - 1

    def assemble_layers(layer):
        while len(layer) >= 2:
            nxt = []
            for i in range(1, len(layer), 2):
                nxt.append(add(ASSEMBLE, tasks[layer[i - 1]].node, (layer[i - 1], layer[i])))
            if len(layer) % 2:
                nxt.append(layer[-1])
            layer = nxt
        return layer

    workers, tops = [], []
    for node, count in enumerate(affinity):
        mine = [add(RENDER, node) for _ in range(int(count))]
        top = assemble_layers(mine)
        if mine:
            tops.append(top[0])
        workers.extend(mine)
    top = assemble_layers(tops)
    compose = add(FINAL_COMPOSE, tasks[top[0]].node, (top[0],)) if top else -1
    return RenderGraph(tasks, workers, compose)


# ------------------------------------------------------------------ image parts (host)

@dataclass
class Part:
    """RgbaImagePart: ARGB32 pixels (h, w) at an origin; size (0, 0) when empty."""
    origin: tuple
    pixels: np.ndarray

    @property
    def size(self):
        return (int(self.pixels.shape[1]), int(self.pixels.shape[0])) if self.pixels.size else (0, 0)


def _union(parts):
    lo = hi = None
    for p in parts:  # BoundingBox<2, int> << origin << origin + size, an empty part included
        for pt in (p.origin, (p.origin[0] + p.size[0], p.origin[1] + p.size[1])):
            if lo is None:
                lo, hi = list(pt), list(pt)
            else:
                for a in range(2):
                    if lo[a] > pt[a]:
                        lo[a] = pt[a]
                    elif hi[a] < pt[a]:
                        hi[a] = pt[a]
    return tuple(lo), (hi[0] - lo[0], hi[1] - lo[1])


def assemble(a: Part, b: Part) -> Part:
    """AssembleFunc: the union box of both parts, zeroed; `a` copied in, `b` blended over it."""
    origin, (w, h) = _union([a, b])
    out = np.zeros((h, w), dtype=np.uint32)
    first = True
    for p in (a, b):
        if p.pixels.size:
            host.blend_image_part(out, np.ascontiguousarray(p.pixels, dtype=np.uint32), p.origin, just_copy=first,
                                  offset=origin)
        first = False
    return Part(origin, out)


def final_compose(p: Part, W: int, H: int, background: int = 0) -> np.ndarray:
    """FinalComposeFunc: the W x H viewport filled with the background colour, the part blended over it."""
    img = np.full((H, W), np.uint32(background), dtype=np.uint32)
    if p.pixels.size:
        host.blend_image_part(img, np.ascontiguousarray(p.pixels, dtype=np.uint32), p.origin)
    return img


def run_graph(graph: RenderGraph, parts, W: int, H: int, background: int = 0):
    """Evaluates the graph on host parts given per worker task (in graph.worker_tasks order)."""
    val = {t: p for t, p in zip(graph.worker_tasks, parts)}
    for i, t in enumerate(graph.tasks):
        if t.kind == ASSEMBLE:
            val[i] = assemble(val[t.inputs[0]], val[t.inputs[1]])
    if graph.compose_task < 0:
        return np.full((H, W), np.uint32(background), dtype=np.uint32)
    return final_compose(val[graph.tasks[graph.compose_task].inputs[0]], W, H, background)


# ------------------------------------------------------------------ image parts (device)

@dataclass
class DevicePart:
    """An image part in device memory: pixels (h*w int32 tensor) at an origin."""
    origin: tuple
    size: tuple
    pixels: object


def assemble_device(ctx, a: DevicePart, b: DevicePart, stream=None) -> DevicePart:
    import torch
    origin, (w, h) = _union([Part(a.origin, np.zeros((a.size[1], a.size[0]), np.uint32)),
                             Part(b.origin, np.zeros((b.size[1], b.size[0]), np.uint32))])
    out = torch.zeros(max(1, w * h), dtype=torch.int32, device="cuda")
    parts = [(p.pixels, p.origin, p.size) for p in (a, b) if p.size[0] * p.size[1] > 0]
    # blendImagePart's justCopySrc applies to `a` only; an empty `a` leaves `b` to be blended
    if a.size[0] * a.size[1] > 0:
        ctx.compose_parts(parts[:1], out, w, h, offset=origin, just_copy_first=True, stream=stream)
        parts = parts[1:]
    if parts:
        ctx.compose_parts(parts, out, w, h, offset=origin, just_copy_first=False, stream=stream)
    return DevicePart(origin, (w, h), out)


def final_compose_device(ctx, p: DevicePart, W: int, H: int, background: int = 0, stream=None):
    import torch
    img = torch.full((W * H,), int(np.uint32(background).view(np.int32)), dtype=torch.int32, device="cuda")
    if p.size[0] * p.size[1] > 0:
        ctx.compose_parts([(p.pixels, p.origin, p.size)], img, W, H, stream=stream)
    return img


def run_graph_device(ctx, graph: RenderGraph, parts, W: int, H: int, background: int = 0, stream=None):
    """run_graph on device parts; returns the W*H int32 device frame."""
    import torch
    val = {t: p for t, p in zip(graph.worker_tasks, parts)}
    for i, t in enumerate(graph.tasks):
        if t.kind == ASSEMBLE:
            val[i] = assemble_device(ctx, val[t.inputs[0]], val[t.inputs[1]], stream=stream)
    if graph.compose_task < 0:
        return torch.full((W * H,), int(np.uint32(background).view(np.int32)), dtype=torch.int32, device="cuda")
    return final_compose_device(ctx, val[graph.tasks[graph.compose_task].inputs[0]], W, H, background, stream)


# ------------------------------------------------------------------ progressive frames

def affinity_for(thread_count: int, thread_per_node: int) -> list:
    """RenderGraphGeneratorPool::getAffinity (src/s3vs_lib/RenderGraphGeneratorPool.hpp:51-60): full
    nodes of thread_per_node workers, then the remainder."""
    full, rem = divmod(int(thread_count), int(thread_per_node))
    return [thread_per_node] * full + ([rem] if rem else [])


class VsRenderer:
    """VsRenderer::continueRendering on one GPU: per level from `min_level` to the last full level,
    the level's split boxes back to front, one worker render per box (VsWorker.render_scene_part,
    its part cropped in device memory), the parts assembled up the render graph and composed onto
    the background on the device; yields (level, W*H device ARGB32 frame) per level.

    states: {level: RenderSharedState} for the levels to render (the blocks of a level that are
    subtree roots with their nodes and values; the same camera, viewport and transfer function)."""

    def __init__(self, ctx, states: dict, node_count: int = 1, thread_per_node: int = 4, background: int = 0):
        from .api import VsWorker
        self.ctx = ctx
        self.states = states
        self.node_count = node_count
        self.thread_per_node = thread_per_node
        self.background = background
        self.split = IndexCubeSplitStorage()
        self.split.set_split_count(node_count * thread_per_node)
        self.workers = [VsWorker(ctx) for _ in range(node_count * thread_per_node)]
        self.last_parts = {}

    def continue_rendering(self, eye, min_level: int = 0, level_count: int | None = None, render_level: int = -1,
                           cancelled=lambda: False):
        levels = sorted(self.states)
        level_count = (max(levels) + 1) if level_count is None else level_count
        if render_level >= 0:
            min_level = min(render_level, level_count - 1)
            level_count = min_level + 1
        self.split.set_eye_position(eye)
        for level in range(min_level, level_count):
            if cancelled():
                return
            boxes = self.split.get_boxes_sorted(level)
            if boxes.shape[0] == 0:
                continue
            graph = render_graph(affinity_for(boxes.shape[0], self.thread_per_node))
            st = self.states[level]
            W, H = st.view.W, st.view.H
            parts = []
            for i, box in enumerate(boxes):
                wk = self.workers[i]
                if wk.state is not st:
                    wk.set_render_shared_state(st)
                r = wk.render_scene_part_device(level, box[:3], box[3:], cancelled)
                if r is None:
                    return
                parts.append(DevicePart(*r))
            self.last_parts[level] = parts
            yield level, run_graph_device(self.ctx, graph, parts, W, H, self.background)


def dataset_level_states(svc, levels, field_index: int, time_frame: int, template, filter: int = _lib.FILTER_TEXTURE):
    """RenderSharedState per level from a dataset (revise_gb300.dataset.BlockTreeFieldService): the
    level's subtree roots with their node lists and values, the field's global range, and the camera,
    viewport, quality, threshold and transfer function of `template` (a workloads.Workload)."""
    import dataclasses
    from .api import RenderSharedState
    lo, hi = svc.field_range(field_index)
    out = {}
    for level in levels:
        fr = svc.read_level(svc.level_topology(level), field_index, time_frame)
        w = dataclasses.replace(template, name=f"{template.name}-level{level}", level=level, blocks=fr.blocks,
                                node_off=fr.node_off, n2i=fr.n2i, sparse=fr.sparse, field_min=lo, field_max=hi)
        out[level] = RenderSharedState(w, filter=filter)
    return out
