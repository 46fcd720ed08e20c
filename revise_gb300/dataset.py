"""Host mirror of the reference's dataset services over the s3r_dataset_* C ABI.

BlockTreeFieldService (include/s3dmm/BlockTreeFieldService.hpp:31-262) opens a
preprocessed dataset by its base name: the field info file, the metadata with
the block tree (Metadata<3>, include/s3dmm/Metadata.hpp:119-499) and the field
files (BlockTreeFieldProvider<3>, include/s3dmm/BlockTreeFieldProvider.hpp).
The method names follow the reference's in snake case.  Parsing, node lists and
file reads run in libs3r.so (host C++); the device side is the batched upload of
a level (`upload`) and the GPU dense-field generator (`interpolate`).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import DatasetInfo, SubtreeInfo, arr, check, ptr


@dataclass
class Subtree:
    """One subtree root of the metadata (Metadata<3>::MetadataBlock + its node count)."""
    level: int
    index: tuple
    depth: int
    tree_index: int
    values_offset: int
    node_count: int


def _subtree(s: SubtreeInfo) -> Subtree:
    return Subtree(int(s.level), (int(s.x), int(s.y), int(s.z)), int(s.depth), int(s.tree_index),
                   int(s.values_offset), int(s.node_count))


def _idx(index) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(index, dtype=np.uint32).reshape(3))


@dataclass
class LevelFrame:
    """A block set of one level in the form FramePlan takes (blocks, node_off, n2i),
    with the sparse values of one field and time frame when read."""
    level: int
    index: np.ndarray       # (nb, 3) uint32 block indices
    blocks: np.ndarray      # (nb, 4) uint32: ix, iy, iz, depth
    node_off: np.ndarray    # (nb + 1,) uint64
    n2i: np.ndarray         # (N, 3) uint16
    sparse: np.ndarray | None = None   # (N,) float32
    ranges: np.ndarray | None = None   # (nb, 2) float32: each subtree's stored [min, max]

    @property
    def nblocks(self) -> int:
        return int(self.blocks.shape[0])

    @property
    def nodes(self) -> int:
        return int(self.node_off[-1])

    @property
    def vertex_off(self) -> np.ndarray:
        e = (1 << self.blocks[:, 3].astype(np.int64)) + 1
        return np.concatenate([[0], np.cumsum(e ** 3)]).astype(np.uint64)

    def block_nodes(self, b: int):
        a, c = int(self.node_off[b]), int(self.node_off[b + 1])
        return self.n2i[a:c], (None if self.sparse is None else self.sparse[a:c])


class Metadata:
    """Read side of Metadata<3> for an open dataset."""

    def __init__(self, svc: "BlockTreeFieldService"):
        self._svc = svc

    @property
    def _info(self) -> DatasetInfo:
        return self._svc._info

    def max_subtree_depth(self) -> int:
        return int(self._info.max_subtree_depth)

    def max_full_level(self) -> int:
        return int(self._info.max_full_level)

    def field_file_size(self) -> int:
        return int(self._info.field_file_size)

    def metadata_block_count(self) -> int:
        return int(self._info.subtree_count)

    def format_version(self) -> int:
        return int(self._info.format_version)

    def bounding_cube(self):
        return tuple(float(v) for v in self._info.bc_min), float(self._info.bc_size)

    def level_count(self) -> int:
        return int(self._info.level_count)

    def levels(self) -> list[list[Subtree]]:
        """Per level its subtree roots, sorted by z, then y, then x."""
        return [self.level_blocks(lv) for lv in range(self.level_count())]

    def level_blocks(self, level: int) -> list[Subtree]:
        lib, h = self._svc._lib, self._svc._h
        n = C.c_uint32()
        check(lib.s3r_dataset_subtrees(h, level, None, 0, C.byref(n)))
        out = (SubtreeInfo * max(1, n.value))()
        check(lib.s3r_dataset_subtrees(h, level, out, n.value, C.byref(n)))
        return [_subtree(out[i]) for i in range(n.value)]

    def tree_blocks(self, level: int) -> np.ndarray:
        """(n, 3) uint32 indices of the whole block tree's blocks at `level`, breadth-first order."""
        lib, h = self._svc._lib, self._svc._h
        n = C.c_uint64()
        check(lib.s3r_dataset_tree_blocks(h, level, None, 0, C.byref(n)))
        out = np.empty((n.value, 3), dtype=np.uint32)
        check(lib.s3r_dataset_tree_blocks(h, level, arr(out, C.c_uint32), n.value, C.byref(n)))
        return out

    def subtree_data(self, level: int, index) -> Subtree:
        s = SubtreeInfo()
        check(self._svc._lib.s3r_dataset_subtree(self._svc._h, level, arr(_idx(index), C.c_uint32), C.byref(s)))
        return _subtree(s)

    def subtree_depth(self, level: int, index) -> int:
        return self.subtree_data(level, index).depth

    def block_tree_nodes(self, level: int, index) -> np.ndarray:
        """BlockTreeNodes<3>(tree, root, depth).data().n2i: (n, 3) uint16."""
        lib, h = self._svc._lib, self._svc._h
        ix = arr(_idx(index), C.c_uint32)
        n = C.c_uint64()
        check(lib.s3r_dataset_subtree_nodes(h, level, ix, None, 0, C.byref(n)))
        out = np.empty((n.value, 3), dtype=np.uint16)
        check(lib.s3r_dataset_subtree_nodes(h, level, ix, ptr(out), n.value, C.byref(n)))
        return out


class BlockTreeFieldService:
    """BlockTreeFieldService<3>: a dataset opened by its base name."""

    def __init__(self, base_name: str):
        self._lib = _lib.load()
        h = C.c_void_p()
        check(self._lib.s3r_dataset_open(str(base_name).encode(), C.byref(h)))
        self._h = h
        self._info = DatasetInfo()
        check(self._lib.s3r_dataset_info_get(h, C.byref(self._info)))
        self._metadata = Metadata(self)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.s3r_dataset_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- field info (BlockTreeFieldService.hpp:42-88)
    def field_count(self) -> int:
        return int(self._info.field_count)

    def field_name(self, field_index: int) -> str:
        buf = C.create_string_buffer(256)
        check(self._lib.s3r_dataset_field(self._h, field_index, buf, 256, None, None))
        return buf.value.decode()

    def field_names(self) -> list[str]:
        return [self.field_name(i) for i in range(self.field_count())]

    def maybe_field_index(self, name: str) -> int:
        i = C.c_uint32()
        rc = self._lib.s3r_dataset_field_index(self._h, name.encode(), C.byref(i))
        return int(i.value) if rc == _lib.S3R_OK else 0xFFFFFFFF

    def field_index(self, name: str) -> int:
        i = C.c_uint32()
        check(self._lib.s3r_dataset_field_index(self._h, name.encode(), C.byref(i)))
        return int(i.value)

    def field_range(self, field_index: int) -> tuple:
        r = (C.c_float * 2)()
        check(self._lib.s3r_dataset_field(self._h, field_index, None, 0, r, None))
        return float(r[0]), float(r[1])

    def field_animated(self, field_index: int) -> bool:
        a = C.c_int32()
        check(self._lib.s3r_dataset_field(self._h, field_index, None, 0, None, C.byref(a)))
        return bool(a.value)

    def time_frame_count(self) -> int:
        return int(self._info.time_steps)

    def has_time_steps(self) -> bool:
        return bool(self._info.has_time_steps)

    def metadata(self) -> Metadata:
        return self._metadata

    # -- one subtree (BlockTreeFieldProvider<3>::fieldValues)
    def field_values(self, field_index: int, time_frame: int, level: int, index):
        """(range, values) of one subtree: its stored [min, max] and one float per node, in n2i order."""
        ix = arr(_idx(index), C.c_uint32)
        n = C.c_uint64()
        r = (C.c_float * 2)()
        check(self._lib.s3r_dataset_subtree_values(self._h, field_index, time_frame, level, ix, None, None, 0,
                                                   C.byref(n)))
        vals = np.empty(n.value, dtype=np.float32)
        check(self._lib.s3r_dataset_subtree_values(self._h, field_index, time_frame, level, ix, r, ptr(vals),
                                                   n.value, C.byref(n)))
        return (float(r[0]), float(r[1])), vals

    def interpolate(self, ctx, field_index: int, time_frame: int, level: int, index, stream=None):
        """BlockTreeFieldService::interpolateWith with the GPU generator: the subtree's dense
        (2^d+1)^3 grid on the device (NaN outside the domain) and the field's global range."""
        import torch
        from .api import to_device_n2i
        n2i = self._metadata.block_tree_nodes(level, index)
        _, vals = self.field_values(field_index, time_frame, level, index)
        depth = self._metadata.subtree_depth(level, index)
        sparse = torch.from_numpy(vals).cuda()
        dense = ctx.interp_dense(to_device_n2i(n2i), sparse, depth, stream=stream)
        return self.field_range(field_index), dense

    # -- a whole level (batched)
    def level_topology(self, level: int, index=None, threads: int = 0) -> LevelFrame:
        """The blocks `index` ((nb, 3); default: every subtree root of the level) with their depths,
        node offsets and concatenated node lists, ready for FramePlan."""
        if index is None:
            index = np.array([s.index for s in self._metadata.level_blocks(level)], dtype=np.uint32).reshape(-1, 3)
        index = np.ascontiguousarray(np.asarray(index, dtype=np.uint32).reshape(-1, 3))
        nb = index.shape[0]
        blocks = np.empty((nb, 4), dtype=np.uint32)
        node_off = np.empty(nb + 1, dtype=np.uint64)
        ix = arr(index, C.c_uint32)
        check(self._lib.s3r_dataset_frame_topology(self._h, level, ix, nb, arr(blocks, C.c_uint32),
                                                   arr(node_off, C.c_uint64), None, 0, threads))
        n2i = np.empty((int(node_off[-1]), 3), dtype=np.uint16)
        check(self._lib.s3r_dataset_frame_topology(self._h, level, ix, nb, arr(blocks, C.c_uint32),
                                                   arr(node_off, C.c_uint64), ptr(n2i), n2i.shape[0], threads))
        return LevelFrame(level, index, blocks, node_off, n2i)

    def read_level(self, frame: LevelFrame, field_index: int, time_frame: int, threads: int = 0) -> LevelFrame:
        """Reads the level's values of one field and time frame into frame.sparse (host)."""
        vals = np.empty(frame.nodes, dtype=np.float32)
        ranges = np.empty((frame.nblocks, 2), dtype=np.float32)
        check(self._lib.s3r_dataset_frame_values(self._h, field_index, time_frame, frame.level,
                                                 arr(frame.index, C.c_uint32), frame.nblocks,
                                                 arr(frame.node_off, C.c_uint64), ptr(vals), ptr(ranges), threads))
        frame.sparse, frame.ranges = vals, ranges
        return frame

    def upload(self, ctx, frame: LevelFrame, field_index: int, time_frame: int, sparse_dev, ranges=None,
               threads: int = 0, stream=None):
        """Reads the level's values through the dataset's pinned staging buffers and copies them to
        sparse_dev (device, frame.nodes floats) in one asynchronous copy on `stream`."""
        from .api import _stream
        rc = self._lib.s3r_dataset_frame_upload(ctx.h, self._h, field_index, time_frame, frame.level,
                                                arr(frame.index, C.c_uint32), frame.nblocks,
                                                arr(frame.node_off, C.c_uint64), ptr(sparse_dev), ptr(ranges),
                                                threads, _stream(stream))
        ctx._check(rc)


# ------------------------------------------------------------------ writing

def _key(xyz: np.ndarray) -> np.ndarray:
    xyz = xyz.astype(np.uint64)
    return xyz[:, 0] | (xyz[:, 1] << np.uint64(21)) | (xyz[:, 2] << np.uint64(42))


def _sorted_unique(k: np.ndarray) -> np.ndarray:
    k = np.sort(k)
    return k[np.concatenate([[True], k[1:] != k[:-1]])] if k.size else k


def _unkey(k: np.ndarray) -> np.ndarray:
    m = np.uint64((1 << 21) - 1)
    return np.stack([k & m, (k >> np.uint64(21)) & m, k >> np.uint64(42)], axis=1).astype(np.uint32)


class BlockTreeLayout:
    """A block tree as the compressed format stores it: per level its blocks in breadth-first
    order (children of one parent consecutive, in local index order c = x + 2y + 4z), each
    block's children bits (bit 7-c), and each block's depth (levels below it).

    The order is what BlockTree<3>::makeCompressible (include/s3dmm/BlockTree.hpp:306-326)
    produces and BlockTreeCompressor<3>::compressBlockTree packs (BlockTreeCompressor.hpp:52-65)."""

    def __init__(self, blocks: np.ndarray):
        blocks = np.asarray(blocks, dtype=np.int64).reshape(-1, 4)
        top = int(blocks[:, 0].max()) if blocks.size else 0
        per = [_sorted_unique(_key(blocks[blocks[:, 0] == lv, 1:4])) for lv in range(top + 1)]
        # close under ancestors, deepest level first
        for lv in range(top, 0, -1):
            parents = _key(_unkey(per[lv]) >> 1)
            per[lv - 1] = _sorted_unique(np.concatenate([per[lv - 1], parents]))
        per[0] = np.array([0], dtype=np.uint64)
        self.xyz = [np.zeros((1, 3), dtype=np.uint32)]
        self.masks = []
        for lv in range(top):
            child = _unkey(per[lv + 1])
            pkey = _key(child >> 1)
            pk_sorted = _key(self.xyz[lv])
            order_p = np.argsort(pk_sorted)
            rank = order_p[np.searchsorted(pk_sorted[order_p], pkey)]
            c = (child[:, 0] & 1) + 2 * (child[:, 1] & 1) + 4 * (child[:, 2] & 1)
            o = np.lexsort((c, rank))
            self.xyz.append(child[o])
            m = np.zeros(self.xyz[lv].shape[0], dtype=np.uint8)
            np.bitwise_or.at(m, rank[o], (0x80 >> c[o]).astype(np.uint8))
            self.masks.append(m)
        self.masks.append(np.zeros(self.xyz[top].shape[0], dtype=np.uint8))
        self.base = np.concatenate([[0], np.cumsum([x.shape[0] for x in self.xyz])]).astype(np.int64)
        # first child rank of each block on the next level
        self.first = [np.concatenate([[0], np.cumsum(_popcount8(m))[:-1]]).astype(np.int64) for m in self.masks]
        self.depth = [np.zeros(x.shape[0], dtype=np.int64) for x in self.xyz]
        for lv in range(top - 1, -1, -1):
            cnt = _popcount8(self.masks[lv])
            parent = np.repeat(np.arange(cnt.size), cnt)
            np.maximum.at(self.depth[lv], parent, self.depth[lv + 1] + 1)

    @property
    def levels(self) -> int:
        return len(self.xyz)

    def children(self, lv: int, r: int):
        m = int(self.masks[lv][r])
        f = int(self.first[lv][r])
        out = []
        for c in range(8):
            if m & (0x80 >> c):
                out.append((c, f))
                f += 1
        return out

    def subtree_roots(self, max_subtree_depth: int, max_full_level: int):
        """Metadata's subtree roots as CompressedBlockTree<3>::walkSubtrees(minDepth = max full level,
        maxDepth = max subtree depth) visits them (include/s3dmm/CompressedBlockTree.hpp:191-228): a
        block's children are roots while the minimum depth is not reached or the block's subtree is
        deeper than the maximum; among them only children themselves deeper than maximum - 1 (the
        reference builds with S3DMM_BLOCKTREE_COUNT_EACH_SUBTREE_DEPTH).  Yields (level, rank) in
        visiting order."""
        out = []
        stack = [(0, 0, max_full_level)]
        while stack:
            lv, r, md = stack.pop()
            out.append((lv, r))
            if md > 0 or self.depth[lv][r] > max_subtree_depth:
                kids = [(lv + 1, f) for c, f in self.children(lv, r)
                        if md > 0 or self.depth[lv + 1][f] > max_subtree_depth - 1]
                stack.extend((kl, kr, max(md - 1, 0)) for kl, kr in reversed(kids))
        return out


def _popcount8(m: np.ndarray) -> np.ndarray:
    return np.unpackbits(m.reshape(-1, 1), axis=1).sum(axis=1).astype(np.int64)


def field_range(values: np.ndarray) -> tuple:
    """computeFieldRange (include/s3dmm/computeFieldRange.hpp:26-45): min and max over the
    values other than the no-field value; (0, -1) when there are none."""
    v = values[values != np.float32(_lib.NO_FIELD_VALUE)]
    return (float(v.min()), float(v.max())) if v.size else (0.0, -1.0)


def _frame_file(base: str, frame: int, has_time_steps: bool) -> str:
    if not has_time_steps:
        return base
    from pathlib import Path
    p = Path(base)
    return str(p.parent / p.stem / f"{p.stem}_t{frame:06d}{p.suffix}")


def write_dataset(base: str, blocks, max_subtree_depth: int, max_full_level: int, fields, time_steps: int = 1,
                  bc_min=(-5.0, -5.0, -5.0), bc_size: float = 10.0) -> None:
    """Writes a dataset in the reference's format (what its preprocessing tools produce).

    blocks: (n, 4) [level, x, y, z] blocks of the tree (their ancestors are added).
    fields: list of (name, values_fn); values_fn(frame, subtree: Subtree, n2i) returns the subtree's
    float32 values in n2i order (S3R_NO_FIELD_VALUE where masked).
    time_steps > 1 writes the per-frame layout <dir>/<stem>/<stem>_tNNNNNN<ext>.  The info file gets
    each field's range over all subtrees and frames, as processMesh.cpp:326-371 computes it."""
    import struct
    from pathlib import Path
    tree = BlockTreeLayout(blocks)
    roots = tree.subtree_roots(max_subtree_depth, max_full_level)
    has_ts = time_steps > 1
    p = Path(base)
    if has_ts:
        (p.parent / p.stem).mkdir(parents=True, exist_ok=True)
        info_path = p.parent / p.stem / f"{p.stem}{p.suffix}.s3dmm-fields"
    else:
        p.parent.mkdir(parents=True, exist_ok=True)
        if not p.exists():
            p.write_text("")
        info_path = Path(base + ".s3dmm-fields")

    def meta_bytes(offsets, file_size):
        hdr = b"s3dmm-metadata" + struct.pack("<IQ", 1, 12) + struct.pack("<III", 3, max_subtree_depth,
                                                                           max_full_level)
        masks = np.concatenate(tree.masks).tobytes()
        nblk = len(masks)
        body = bytearray(struct.pack("<ffff", *bc_min, bc_size) + struct.pack("<QQ", nblk << 3, nblk) + masks)
        nlev = max(lv for lv, _ in roots) + 1
        body += struct.pack("<Q", nlev)
        for lv in range(nlev):
            items = sorted((tuple(int(v) for v in tree.xyz[lv][r][::-1]), r, k)
                           for k, (l2, r) in enumerate(roots) if l2 == lv)
            body += struct.pack("<Q", len(items))
            for _, r, k in items:
                x, y, z = (int(v) for v in tree.xyz[lv][r])
                depth = min(int(tree.depth[lv][r]), max_subtree_depth)
                body += struct.pack("<IIIIQQ", x, y, z, int(tree.base[lv] + r), offsets[k], depth)
        body += struct.pack("<Q", file_size)
        return hdr + struct.pack("<Q", len(hdr) + 8) + bytes(body)

    # metadata with placeholder offsets, then node counts from the reader, then the final file
    info_path.write_text("time_steps\n%d\n\nfield\tmin\tmax\tanimated\n" % time_steps +
                         "".join(f"{name}\t-\t-\t{int(has_ts)}\n" for name, _ in fields))
    frames = [_frame_file(base, t, has_ts) for t in range(time_steps)]
    for f in frames:
        Path(f + ".s3dmm-meta").write_bytes(meta_bytes([0] * len(roots), 0))
    with BlockTreeFieldService(base) as svc:
        md = svc.metadata()
        counts = []
        for lv, r in roots:
            counts.append(md.subtree_data(lv, tuple(int(v) for v in tree.xyz[lv][r])).node_count)
        offsets = np.concatenate([[0], np.cumsum([(2 + n) * 4 for n in counts])]).astype(np.int64)
        for f in frames:
            Path(f + ".s3dmm-meta").write_bytes(meta_bytes([int(o) for o in offsets[:-1]], int(offsets[-1])))
        ranges = []
        for name, fn in fields:
            lo, hi = np.inf, -np.inf
            for t, f in enumerate(frames):
                buf = bytearray(int(offsets[-1]))
                for k, (lv, r) in enumerate(roots):
                    ix = tuple(int(v) for v in tree.xyz[lv][r])
                    sub = Subtree(lv, ix, min(int(tree.depth[lv][r]), max_subtree_depth),
                                  int(tree.base[lv] + r), int(offsets[k]), counts[k])
                    vals = np.ascontiguousarray(fn(t, sub, md.block_tree_nodes(lv, ix)), dtype=np.float32)
                    assert vals.shape == (counts[k],), (lv, ix, vals.shape, counts[k])
                    rng = field_range(vals)
                    if rng[0] <= rng[1]:
                        lo, hi = min(lo, rng[0]), max(hi, rng[1])
                    o = int(offsets[k])
                    buf[o:o + 8] = np.array(rng, dtype=np.float32).tobytes()
                    buf[o + 8:o + 8 + 4 * counts[k]] = vals.tobytes()
                Path(f + ".s3dmm-field#" + name).write_bytes(bytes(buf))
            ranges.append((lo, hi))
    info_path.write_text("time_steps\n%d\n\nfield\tmin\tmax\tanimated\n" % time_steps +
                         "".join((f"{name}\t{lo:.9g}\t{hi:.9g}\t{int(has_ts)}\n" if lo <= hi else
                                  f"{name}\t-\t-\t{int(has_ts)}\n") for (name, _), (lo, hi) in zip(fields, ranges)))


# ------------------------------------------------------------------ upstream field generation

def _propagate(svc: BlockTreeFieldService, ctx, level: int, child_values, sums, weights, stream=None) -> np.ndarray:
    from .api import _stream
    n = len(svc.metadata().level_blocks(level))
    counts = np.zeros(max(1, n), dtype=np.uint8)
    ctx._check(svc._lib.s3r_dataset_propagate(ctx.h, svc._h, level, ptr(child_values), ptr(sums), ptr(weights),
                                              arr(counts, C.c_uint8), _stream(stream)))
    return counts[:n]


def _field_divide(ctx, sums, weights, values, stream=None) -> None:
    from .api import _stream
    n = int(values.numel())
    ctx._check(ctx.lib.s3r_field_divide(ctx.h, ptr(sums), ptr(weights), n, ptr(values), _stream(stream)))


BlockTreeFieldService.propagate = _propagate
BlockTreeFieldService.propagate.__doc__ = """The child -> parent step of generatePropagatedField for `level` on
the GPU: child_values (device, the field on every subtree of level+1 in level_blocks order) -> sums and
weights (device, one float per node of every subtree of `level`).  Returns per parent subtree its number
of child subtrees (8: divide; fewer: add the generator's contributions first)."""
field_divide = _field_divide
