"""Seeded synthetic block-tree workloads (no dataset ships with the reference).

Each workload is a block set at one block-tree level: per block an octree of
some depth d whose node set (the corners of every octree cell, in dense
vertex coordinates at depth d -- the BlockTreeNodes<3> n2i layout,
include/s3dmm/BlockTreeNodes.hpp:460-601) carries float32 field values, with
S3R_NO_FIELD_VALUE (1e30) at masked nodes.  The node order within a block is
a seeded permutation.  Field values follow the reference's recipe for
function-defined fields: the function evaluated at node positions
(include/s3dmm/BlockTreeFieldFromFunc.hpp:51-87 averages over the blocks
sharing a vertex, which for a continuous function is the value itself).

Configurations (sizes and distributions as specified for the benchmark):
  cfg1  one block, L=5 over the unit cube, refined where |r-0.3| < 2 cell widths,
        f = sin(4 pi x) cos(4 pi y) + z, masked where r >= 0.45; orthographic 512^2
        along +z, quality 2 (one sample per half voxel), 256-entry RGBA ramp over [-1, 2];
  cfg2  4x4x4 blocks, depth 6, a U(0.3, 0.7) fraction of leaves refined per level,
        sum of 8 Gaussian blobs; perspective 1920x1080, fovY 60, eye (0,10,35);
  cfg3  16^3 blocks, depth from {3..7} with p {.3,.3,.2,.15,.05}, node targets
        LogNormal(ln 2000, 1) capped at (2^d+1)^3, 20% of nodes masked; 1920x1080;
  cfg4  cfg2 with FP16 / BF16 bricks (brick format chosen by the caller);
  cfg5  2x2x2 blocks, depth 6, smooth blob field, 512x512; random 256x4 TF (seed 1)
        makes the target image.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

NO_FIELD = np.float32(1e30)

_CORNERS = np.array([[i & 1, (i >> 1) & 1, (i >> 2) & 1] for i in range(8)], dtype=np.int64)


@dataclass
class Workload:
    name: str
    level: int
    blocks: np.ndarray      # (nb, 4) uint32: ix, iy, iz, depth
    node_off: np.ndarray    # (nb + 1,) uint64
    n2i: np.ndarray         # (N, 3) uint16
    sparse: np.ndarray      # (N,) float32
    field_min: float
    field_max: float
    W: int
    H: int
    eye: tuple
    center: tuple
    up: tuple
    fovy: float
    ortho: bool
    ortho_height: float
    quality: float
    threshold_rel: float
    tf: np.ndarray          # (tf_n, 4) float32
    meta: dict = field(default_factory=dict)

    @property
    def nblocks(self) -> int:
        return int(self.blocks.shape[0])

    @property
    def vertex_off(self) -> np.ndarray:
        e = (1 << self.blocks[:, 3].astype(np.int64)) + 1
        return np.concatenate([[0], np.cumsum(e ** 3)]).astype(np.uint64)

    @property
    def vertices(self) -> int:
        return int(self.vertex_off[-1])

    @property
    def nodes(self) -> int:
        return int(self.node_off[-1])

    def block_nodes(self, b: int):
        a, c = int(self.node_off[b]), int(self.node_off[b + 1])
        return self.n2i[a:c], self.sparse[a:c]

    @property
    def threshold(self) -> float:
        return self.field_min + (self.field_max - self.field_min) * self.threshold_rel


def _pack(c: np.ndarray) -> np.ndarray:
    return (c[..., 0] << 40) | (c[..., 1] << 20) | c[..., 2]


def _unpack(k: np.ndarray) -> np.ndarray:
    return np.stack([(k >> 40) & 0xFFFFF, (k >> 20) & 0xFFFFF, k & 0xFFFFF], axis=-1)


def octree_nodes(depth: int, choose, rng: np.random.Generator) -> np.ndarray:
    """Node set of an octree grown level by level.

    choose(level, cells, node_count) returns a boolean mask of the level's cells
    to refine; at least one cell is refined on every level below `depth`, so the
    subtree reaches its full depth.  Returns (n, 3) uint16 vertex coordinates at
    `depth`, in a seeded random order.
    """
    cells = np.zeros((1, 3), dtype=np.int64)
    keys = []
    seen = np.zeros(0, dtype=np.int64)
    for level in range(depth + 1):
        shift = depth - level
        corners = (cells[:, None, :] + _CORNERS[None, :, :]) << shift
        keys.append(_pack(corners).ravel())
        if level == depth:
            break
        seen = np.unique(np.concatenate([seen, keys[-1]]))
        mask = np.asarray(choose(level, cells, seen.size), dtype=bool)
        if not mask.any():
            mask[rng.integers(cells.shape[0])] = True
        ref = cells[mask]
        cells = (ref[:, None, :] * 2 + _CORNERS[None, :, :]).reshape(-1, 3)
    uniq = np.unique(np.concatenate(keys))
    nodes = _unpack(uniq).astype(np.uint16)
    return nodes[rng.permutation(nodes.shape[0])]


def _blob_field(rng: np.random.Generator, count: int = 8):
    centres = rng.uniform(0.0, 1.0, size=(count, 3))
    sigma = rng.uniform(0.05, 0.2, size=count)
    amp = rng.uniform(-1.0, 1.0, size=count)

    def f(u: np.ndarray) -> np.ndarray:
        d2 = ((u[:, None, :] - centres[None, :, :]) ** 2).sum(-1)
        return (amp[None, :] * np.exp(-d2 / (2 * sigma[None, :] ** 2))).sum(-1)

    return f


def _node_unit_coords(level: int, idx, depth: int, n2i: np.ndarray) -> np.ndarray:
    """Node positions in unit-cube coordinates of the whole block cube [-5, 5]^3."""
    m = 1 << level
    return (np.asarray(idx, dtype=np.float64)[None, :] + n2i.astype(np.float64) / (1 << depth)) / m


def ramp_tf(n: int = 256) -> np.ndarray:
    t = np.linspace(0.0, 1.0, n, dtype=np.float64)
    return np.stack([t, 1.0 - np.abs(2 * t - 1), 1.0 - t, t], axis=1).astype(np.float32)


def colormap_points():
    """Control points of the default transfer function (relative field value -> RGBA)."""
    xs = np.array([0.0, 0.25, 0.5, 0.75, 1.0])
    rgba = np.array([[0.05, 0.1, 0.8, 0.0],
                     [0.1, 0.7, 0.9, 0.3],
                     [0.2, 0.9, 0.3, 0.5],
                     [0.95, 0.85, 0.1, 0.8],
                     [0.9, 0.1, 0.05, 1.0]])
    return xs, rgba


def _finish(name, level, blocks, parts, rng, W, H, eye, center, up, fovy, ortho, ortho_height, quality, thr, tf,
            mask_fraction=0.0, meta=None) -> Workload:
    n2i = np.concatenate([p[0] for p in parts]).astype(np.uint16)
    vals = np.concatenate([p[1] for p in parts]).astype(np.float32)
    if mask_fraction > 0:
        m = rng.random(vals.shape[0]) < mask_fraction
        vals = np.where(m, NO_FIELD, vals).astype(np.float32)
    counts = np.array([p[0].shape[0] for p in parts], dtype=np.uint64)
    node_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    valid = vals[(vals != NO_FIELD) & ~np.isnan(vals)]
    fmin, fmax = (float(valid.min()), float(valid.max())) if valid.size else (0.0, 1.0)
    if not fmax > fmin:
        fmax = fmin + 1.0
    return Workload(name, level, np.asarray(blocks, dtype=np.uint32).reshape(-1, 4), node_off, n2i, vals,
                    fmin, fmax, W, H, eye, center, up, fovy, ortho, ortho_height, quality, thr, tf, meta or {})


def cfg1(seed: int = 0) -> Workload:
    rng = np.random.default_rng(seed)
    depth = 5
    c0 = np.array([0.5, 0.5, 0.5])

    def choose(level, cells, _count):
        w = 1.0 / (1 << level)
        centre = (cells + 0.5) * w
        r = np.linalg.norm(centre - c0, axis=1)
        return np.abs(r - 0.3) < 2 * w

    n2i = octree_nodes(depth, choose, rng)
    u = n2i.astype(np.float64) / (1 << depth)
    f = np.sin(4 * np.pi * u[:, 0]) * np.cos(4 * np.pi * u[:, 1]) + u[:, 2]
    r = np.linalg.norm(u - c0, axis=1)
    f = np.where(r >= 0.45, np.float64(NO_FIELD), f).astype(np.float32)
    w = _finish("cfg1", 0, [[0, 0, 0, depth]], [(n2i, f)], rng, 512, 512, (0.0, 0.0, -20.0), (0.0, 0.0, 0.0),
                (0.0, 1.0, 0.0), 60.0, True, 10.0, 2.0, 0.5, ramp_tf(256))
    w.field_min, w.field_max = -1.0, 2.0  # the transfer-function range the config specifies
    return w


def _random_refinement(rng, lo=0.3, hi=0.7):
    def choose(level, cells, _count):
        p = rng.uniform(lo, hi)
        k = cells.shape[0]
        nref = max(1, int(round(p * k)))
        mask = np.zeros(k, dtype=bool)
        mask[rng.choice(k, nref, replace=False)] = True
        return mask

    return choose


def color_table(xs, rgba, n: int) -> np.ndarray:
    """(n, 4) float32 piecewise-linear RGBA table through the control points, in single precision exactly as
    s3r_make_color_transfer (makeColorTransferVector) builds it; kept in numpy so that generating a workload
    loads no native code."""
    xs = np.asarray(xs, np.float64).astype(np.float32)
    rgba = np.asarray(rgba, np.float64).reshape(-1, 4).astype(np.float32)
    out = np.zeros((n, 4), np.float32)
    xmin, xmax = xs[0], xs[-1]
    out[0] = c1 = rgba[0]
    i1 = 0
    one = np.float32(1)
    for ip in range(1, xs.size):
        c2 = rgba[ip]
        i2 = n - 1 if ip + 1 == xs.size else int(np.float32(np.float32(xs[ip] - xmin) / np.float32(xmax - xmin)) * np.float32(n))
        for i in range(i1 + 1, min(i2, n - 1) + 1) if i2 > i1 else ():
            t = np.float32(np.float32(i - i1) / np.float32(i2 - i1))
            out[i] = np.float32(c1 * (one - t)) + np.float32(c2 * t)
        c1 = c2
        i1 = i2
    return out


def _tf_default(n=256):
    xs, rgba = colormap_points()
    return color_table(xs, rgba, n)


def cfg2(seed: int = 0, W: int = 1920, H: int = 1080) -> Workload:
    rng = np.random.default_rng(seed)
    level, depth = 2, 6
    f = _blob_field(rng)
    blocks, parts = [], []
    m = 1 << level
    for iz in range(m):
        for iy in range(m):
            for ix in range(m):
                n2i = octree_nodes(depth, _random_refinement(rng), rng)
                vals = f(_node_unit_coords(level, (ix, iy, iz), depth, n2i))
                blocks.append([ix, iy, iz, depth])
                parts.append((n2i, vals))
    return _finish("cfg2", level, blocks, parts, rng, W, H, (0.0, 10.0, 35.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0),
                   60.0, False, 0.0, 1.0, 0.5, _tf_default())


def cfg3(seed: int = 0, W: int = 1920, H: int = 1080, level: int = 4) -> Workload:
    rng = np.random.default_rng(seed)
    f = _blob_field(rng)
    m = 1 << level
    depths = rng.choice([3, 4, 5, 6, 7], size=m ** 3, p=[0.3, 0.3, 0.2, 0.15, 0.05])
    targets = rng.lognormal(np.log(2000.0), 1.0, size=m ** 3)
    blocks, parts = [], []
    b = 0
    for iz in range(m):
        for iy in range(m):
            for ix in range(m):
                d = int(depths[b])
                cap = ((1 << d) + 1) ** 3
                target = min(float(targets[b]), float(cap))

                def choose(lvl, cells, count, d=d, target=target):
                    k = cells.shape[0]
                    remaining = max(target - count, 0.0)
                    levels_left = d - lvl
                    # spread the remaining node budget over the remaining levels; a refined
                    # cell adds up to 19 vertices (12 edge, 6 face, 1 cell midpoints)
                    want = remaining / (levels_left * 10.0)
                    nref = int(np.clip(round(want), 1, k))
                    mask = np.zeros(k, dtype=bool)
                    mask[rng.choice(k, nref, replace=False)] = True
                    return mask

                n2i = octree_nodes(d, choose, rng)
                vals = f(_node_unit_coords(level, (ix, iy, iz), d, n2i))
                blocks.append([ix, iy, iz, d])
                parts.append((n2i, vals))
                b += 1
    return _finish("cfg3", level, blocks, parts, rng, W, H, (0.0, 10.0, 35.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0),
                   60.0, False, 0.0, 1.0, 0.5, _tf_default(), mask_fraction=0.2)


def cfg5(seed: int = 0, W: int = 512, H: int = 512) -> Workload:
    rng = np.random.default_rng(seed)
    level, depth = 1, 6
    f = _blob_field(rng)
    blocks, parts = [], []
    for iz in range(2):
        for iy in range(2):
            for ix in range(2):
                n2i = octree_nodes(depth, _random_refinement(rng), rng)
                vals = f(_node_unit_coords(level, (ix, iy, iz), depth, n2i))
                blocks.append([ix, iy, iz, depth])
                parts.append((n2i, vals))
    w = _finish("cfg5", level, blocks, parts, rng, W, H, (6.0, 8.0, 20.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0),
                40.0, False, 0.0, 1.0, 0.5, _tf_default())
    w.meta["target_tf"] = np.random.default_rng(1).uniform(0.0, 1.0, size=(256, 4)).astype(np.float32)
    return w


def small(seed: int = 0, level: int = 1, depths=(2, 3, 4), W: int = 96, H: int = 64, mask_fraction: float = 0.15,
          eye=(3.0, 6.0, 14.0)) -> Workload:
    """A small mixed-depth block set for parity tests (oracle-sized)."""
    rng = np.random.default_rng(seed)
    f = _blob_field(rng)
    m = 1 << level
    blocks, parts = [], []
    for iz in range(m):
        for iy in range(m):
            for ix in range(m):
                d = int(rng.choice(depths))
                n2i = octree_nodes(d, _random_refinement(rng), rng)
                vals = f(_node_unit_coords(level, (ix, iy, iz), d, n2i))
                blocks.append([ix, iy, iz, d])
                parts.append((n2i, vals))
    return _finish("small", level, blocks, parts, rng, W, H, eye, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 45.0, False,
                   0.0, 1.5, 0.5, _tf_default(), mask_fraction=mask_fraction)


def tree_blocks(w: Workload) -> np.ndarray:
    """The block tree a workload's node sets define, for writing it as a dataset: every block of
    w.level and, below each, the cells of its octree -- a cell is refined exactly when its centre
    is one of the block's nodes, since only the cell's own children have that point as a corner.
    Returns (n, 4) [level, x, y, z]; the ancestors above w.level are implied."""
    out = [np.concatenate([np.full((w.nblocks, 1), w.level, dtype=np.int64),
                           w.blocks[:, :3].astype(np.int64)], axis=1)]
    # all blocks at once: a node is keyed by (block, x, y, z), 10 bits per coordinate (depth <= 9)
    counts = np.diff(w.node_off.astype(np.int64))
    owner = np.repeat(np.arange(w.nblocks, dtype=np.int64), counts)

    def key(b, xyz):
        return (b << 30) | (xyz[:, 0] << 20) | (xyz[:, 1] << 10) | xyz[:, 2]

    keys = np.sort(key(owner, w.n2i.astype(np.int64)))
    depth = w.blocks[:, 3].astype(np.int64)
    cb = np.arange(w.nblocks, dtype=np.int64)           # block of each cell
    cells = np.zeros((w.nblocks, 3), dtype=np.int64)    # cell coordinates at relative level j
    for j in range(int(depth.max(initial=0))):
        live = depth[cb] > j
        cb, cells = cb[live], cells[live]
        size = (1 << (depth[cb] - j))[:, None]
        ck = key(cb, cells * size + size // 2)
        pos = np.minimum(np.searchsorted(keys, ck), keys.size - 1)
        ref = keys[pos] == ck
        if not ref.any():
            break
        cb = np.repeat(cb[ref], 8)
        cells = (cells[ref][:, None, :] * 2 + _CORNERS[None, :, :]).reshape(-1, 3)
        origin = w.blocks[cb, :3].astype(np.int64) * (2 << j)
        out.append(np.concatenate([np.full((cb.size, 1), w.level + j + 1, dtype=np.int64), origin + cells], axis=1))
    return np.concatenate(out)


def dataset_values(w: Workload):
    """values_fn for revise_gb300.dataset.write_dataset: on w.level's subtrees the workload's values
    in the subtree's node order, on coarser subtrees the no-field value."""
    where = {tuple(int(v) for v in w.blocks[b, :3]): b for b in range(w.nblocks)}

    def fn(_frame, sub, n2i):
        if sub.level != w.level:
            return np.full(n2i.shape[0], NO_FIELD, dtype=np.float32)
        wn, wv = w.block_nodes(where[tuple(sub.index)])
        k = _pack(wn.astype(np.int64))
        o = np.argsort(k)
        pos = np.searchsorted(k[o], _pack(n2i.astype(np.int64)))
        return wv[o[pos]]

    return fn


CONFIGS = {"cfg1": cfg1, "cfg2": cfg2, "cfg3": cfg3, "cfg5": cfg5, "small": small}
