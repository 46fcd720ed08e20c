"""Oracle (TEST INFRASTRUCTURE ONLY): numpy restatement of the reference's field
generation for block-tree datasets, used to check the GPU propagation
(s3r_dataset_propagate) and pinned against field files the reference itself
wrote (tests/golden/dataset).  Nothing in the product imports it.

Restated (paths relative to the reference project root):
  generatePropagatedField   include/s3dmm/BlockTreeFieldProvider.hpp:270-389 -- levels from the deepest up;
                            per subtree the child subtrees' values summed in child order (x fastest) with
                            weights, divided when all 8 children exist, else the generator adds its values
  BlockTreeFieldFromFunc    include/s3dmm/BlockTreeFieldFromFunc.hpp:51-87 -- the function at the 8 corners
                            of every block of the subtree (depth-first pre-order), positions from
                            CompressedBlockTree::blockPos (include/s3dmm/CompressedBlockTree.hpp:50-58)
  computeFieldRange         include/s3dmm/computeFieldRange.hpp:26-45
All arithmetic in float32, operation by operation, as the reference's real_type = float build does it.
"""
from __future__ import annotations

import numpy as np

NO_FIELD = np.float32(1e30)
F = np.float32


def _key(xyz: np.ndarray) -> np.ndarray:
    xyz = xyz.astype(np.int64)
    return (xyz[:, 0] << 42) | (xyz[:, 1] << 21) | xyz[:, 2]


class Tree:
    """A block tree from its blocks per level (the dataset reader's breadth-first lists)."""

    def __init__(self, levels: list[np.ndarray], bc_min, bc_size):
        self.sets = [set(_key(b).tolist()) for b in levels]
        self.bc_min = np.asarray(bc_min, dtype=np.float32)
        self.bc_size = F(bc_size)

    def has(self, level: int, xyz) -> bool:
        if level >= len(self.sets):
            return False
        x, y, z = (int(v) for v in xyz)
        return ((x << 42) | (y << 21) | z) in self.sets[level]

    def walk(self, level: int, xyz, depth: int):
        """Blocks of the subtree in depth-first pre-order, children in local order c = x + 2y + 4z,
        down to `depth` levels below the root: list of (level, (x, y, z))."""
        out, stack = [], [(level, tuple(int(v) for v in xyz), 0)]
        while stack:
            lv, b, r = stack.pop()
            out.append((lv, b))
            if r >= depth:
                continue
            kids = []
            for c in range(8):
                k = (2 * b[0] + (c & 1), 2 * b[1] + ((c >> 1) & 1), 2 * b[2] + (c >> 2))
                if self.has(lv + 1, k):
                    kids.append((lv + 1, k, r + 1))
            stack.extend(reversed(kids))
        return out

    def block_min_size(self, level: int, xyz):
        size = F(self.bc_size / F(1 << level))
        rel = np.asarray(xyz, dtype=np.float32) * size
        return (self.bc_min + rel).astype(np.float32), size


def field_f(p: np.ndarray) -> np.ndarray:
    """Fixture field f: x + 2y - 0.5z, no field inside radius 2 (oracle/ref_dataset_gen.cpp FieldF)."""
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    r2 = (x * x + y * y) + z * z
    v = (x + F(2) * y) - F(0.5) * z
    return np.where(r2 < F(4), np.float32(np.nan), v).astype(np.float32)


def field_g(t: float):
    """Fixture field g: x*y - z + t, no field inside radius 2 (FieldG)."""
    def g(p):
        x, y, z = p[:, 0], p[:, 1], p[:, 2]
        r2 = (x * x + y * y) + z * z
        v = (x * y - z) + F(t)
        return np.where(r2 < F(4), np.float32(np.nan), v).astype(np.float32)
    return g


def add_function(tree: Tree, level: int, xyz, depth: int, n2i: np.ndarray, func, field: np.ndarray,
                 weight: np.ndarray) -> None:
    """BlockTreeFieldFromFunc::generate's accumulation: func at every block corner of the subtree,
    added to field and weight (in place, float32, in the reference's order)."""
    order = np.argsort(_key(n2i))
    keys = _key(n2i)[order]
    mask = (1 << depth) - 1
    blocks = tree.walk(level, xyz, depth)
    pos, nodes = [], []
    for lv, b in blocks:
        shift = depth - (lv - level)
        base = [((v << shift) & mask) for v in b]
        mn, size = tree.block_min_size(lv, b)
        for k in range(8):
            bits = [(k >> d) & 1 for d in range(3)]
            p = mn.copy()
            for d in range(3):
                if bits[d]:
                    p[d] = F(p[d] + size)
            pos.append(p)
            nodes.append([base[d] + (bits[d] << shift) for d in range(3)])
    pos = np.asarray(pos, dtype=np.float32)
    idx = order[np.searchsorted(keys, _key(np.asarray(nodes)))]
    v = func(pos)
    ok = ~np.isnan(v)
    # np.add.at accumulates repeated indices one after another, in index order
    np.add.at(field, idx[ok], v[ok])
    np.add.at(weight, idx[ok], np.float32(1))


def divide(field: np.ndarray, weight: np.ndarray) -> np.ndarray:
    return np.where(weight > 0, field / np.where(weight > 0, weight, F(1)), NO_FIELD).astype(np.float32)


def propagate_into(parent_n2i: np.ndarray, parent_depth: int, children, field: np.ndarray,
                   weight: np.ndarray) -> None:
    """The child loop of generatePropagatedField for one parent: children = [(c, child_depth,
    child_n2i, child_values)] in child order; adds into field / weight in place."""
    order = np.argsort(_key(parent_n2i))
    keys = _key(parent_n2i)[order]
    for c, cd, cn2i, cvals in children:
        shift = cd + 1 - parent_depth
        n = cn2i.astype(np.int64)
        if shift >= 1:
            keep = ~np.any(n & 1, axis=1)
            n, vals = n[keep] >> shift, cvals[keep]
        else:
            vals = cvals
            n = n << (-shift)
        off = np.array([c & 1, (c >> 1) & 1, c >> 2], dtype=np.int64) << (parent_depth - 1)
        idx = order[np.searchsorted(keys, _key(n + off))]
        ok = vals != NO_FIELD
        field[idx[ok]] += vals[ok]
        weight[idx[ok]] += np.float32(1)


def field_range(values: np.ndarray) -> tuple:
    v = values[values != NO_FIELD]
    return (float(v.min()), float(v.max())) if v.size else (0.0, -1.0)


def generate_propagated(svc, func) -> dict:
    """generatePropagatedField over a whole dataset (svc: revise_gb300.dataset.BlockTreeFieldService
    for the tree and node lists): {(level, (x, y, z)): float32 values}."""
    md = svc.metadata()
    levels, lv = [], 0
    while True:
        b = md.tree_blocks(lv)
        if b.shape[0] == 0:
            break
        levels.append(b)
        lv += 1
    bc_min, bc_size = md.bounding_cube()
    tree = Tree(levels, bc_min, bc_size)
    subs = md.levels()
    out = {}
    for level in range(len(subs) - 1, -1, -1):
        for s in subs[level]:
            n2i = md.block_tree_nodes(level, s.index)
            field = np.zeros(n2i.shape[0], dtype=np.float32)
            weight = np.zeros(n2i.shape[0], dtype=np.float32)
            kids = []
            if level + 1 < len(subs):
                for c in range(8):
                    ci = (2 * s.index[0] + (c & 1), 2 * s.index[1] + ((c >> 1) & 1), 2 * s.index[2] + (c >> 2))
                    if (level + 1, ci) in out:
                        cd = md.subtree_depth(level + 1, ci)
                        kids.append((c, cd, md.block_tree_nodes(level + 1, ci), out[(level + 1, ci)]))
            propagate_into(n2i, s.depth, kids, field, weight)
            if len(kids) < 8:
                add_function(tree, level, s.index, s.depth, n2i, func, field, weight)
            out[(level, s.index)] = divide(field, weight)
    return out
