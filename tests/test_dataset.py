"""On-disk dataset reader (s3r_dataset_*), host side, against datasets written
and read back by the reference's own code (tests/golden/make_dataset.py):
metadata records, BlockTreeNodes n2i order and field values, bit for bit."""
import hashlib
import json
import shutil
from pathlib import Path

import numpy as np
import pytest

from revise_gb300 import _lib
from revise_gb300.dataset import BlockTreeFieldService

DATA = Path(__file__).resolve().parent / "golden" / "dataset"
EXPECTED = json.loads((DATA / "expected.json").read_text())


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def shell():
    with BlockTreeFieldService(str(DATA / "shell.dat")) as s:
        yield s


@pytest.fixture(scope="module")
def series():
    with BlockTreeFieldService(str(DATA / "series.dat")) as s:
        yield s


def test_field_info(shell, series):
    assert shell.field_names() == ["f", "g"]
    assert shell.time_frame_count() == 1 and not shell.has_time_steps()
    assert shell.field_index("g") == 1 and shell.maybe_field_index("h") == 0xFFFFFFFF
    assert shell.field_range(0) == (-17.5, 17.5)
    with pytest.raises(_lib.S3RError):
        shell.field_index("h")
    assert series.field_names() == ["g"] and series.time_frame_count() == 2 and series.has_time_steps()
    assert series.field_animated(0)


def test_metadata_header(shell):
    md = shell.metadata()
    assert md.format_version() == 1
    assert md.max_subtree_depth() == 3 and md.max_full_level() == 1
    assert md.bounding_cube() == ((-5.0, -5.0, -5.0), 10.0)
    recs = EXPECTED["shell.dat"]["frames"][0]
    assert md.metadata_block_count() == len(recs)
    assert md.field_file_size() == (DATA / "shell.dat.s3dmm-field#f").stat().st_size


@pytest.mark.parametrize("name", ["shell.dat", "series.dat"])
def test_subtrees_nodes_and_values_match_reference(name, shell, series):
    svc = shell if name == "shell.dat" else series
    exp = EXPECTED[name]
    md = svc.metadata()
    for frame, recs in enumerate(exp["frames"]):
        got = [s for lv in md.levels() for s in lv]
        assert [(s.level, list(s.index)) for s in got] == [(r["level"], r["idx"]) for r in recs]
        for s, r in zip(got, recs):
            assert (s.depth, s.tree_index, s.values_offset, s.node_count) == \
                (r["depth"], r["tree_index"], r["values_offset"], r["node_count"]), r
            n2i = md.block_tree_nodes(s.level, s.index)
            assert n2i.shape == (r["node_count"], 3)
            assert sha(n2i.astype("<u2")) == r["n2i_sha256"], (s.level, s.index)
            for k in range(len(exp["fields"])):
                rng, vals = svc.field_values(k, frame, s.level, s.index)
                stored = np.concatenate([np.array(rng, dtype=np.float32), vals]).astype("<f4")
                assert sha(stored) == r["values_sha256"][k], (frame, k, s.level, s.index)


def test_level_frame_matches_per_subtree_reads(shell):
    md = shell.metadata()
    for level in range(md.level_count()):
        blocks = md.level_blocks(level)
        fr = shell.level_topology(level, threads=3)
        assert fr.nblocks == len(blocks)
        shell.read_level(fr, 1, 0, threads=3)
        for b, s in enumerate(blocks):
            a, c = int(fr.node_off[b]), int(fr.node_off[b + 1])
            assert list(fr.blocks[b]) == [*s.index, s.depth]
            assert np.array_equal(fr.n2i[a:c], md.block_tree_nodes(level, s.index))
            rng, vals = shell.field_values(1, 0, level, s.index)
            assert np.array_equal(fr.sparse[a:c].view(np.uint32), vals.view(np.uint32))
            assert tuple(fr.ranges[b]) == rng


def test_level_frame_subset_in_caller_order(shell):
    blocks = shell.metadata().level_blocks(3)
    pick = np.array([blocks[i].index for i in (7, 0, 30, 2)], dtype=np.uint32)
    fr = shell.read_level(shell.level_topology(3, pick), 0, 0)
    for b, ix in enumerate(pick):
        _, vals = shell.field_values(0, 0, 3, ix)
        assert np.array_equal(fr.sparse[int(fr.node_off[b]):int(fr.node_off[b + 1])], vals)


def test_nodes_are_octree_corners_within_the_subtree(shell):
    md = shell.metadata()
    for s in md.level_blocks(2)[:8]:
        n2i = md.block_tree_nodes(2, s.index).astype(np.int64)
        assert n2i.max() <= (1 << s.depth) and len(np.unique(n2i @ [1, 1 << 12, 1 << 24])) == len(n2i)
        # the root block's 8 corners come first, in x-fastest order
        e = 1 << s.depth
        assert n2i[:8].tolist() == [[(k & 1) * e, ((k >> 1) & 1) * e, (k >> 2) * e] for k in range(8)]


def test_errors(shell, tmp_path):
    with pytest.raises(_lib.S3RError, match="no dataset files"):
        BlockTreeFieldService(str(tmp_path / "nothing.dat"))
    with pytest.raises(_lib.S3RError, match="no subtree root"):
        shell.metadata().subtree_data(3, (0, 0, 0))
    with pytest.raises(_lib.S3RError, match="field index"):
        shell.field_values(5, 0, 0, (0, 0, 0))
    with pytest.raises(_lib.S3RError, match="time frame"):
        shell.field_values(0, 3, 0, (0, 0, 0))
    # truncated metadata and a missing field file
    d = tmp_path / "cut"
    d.mkdir()
    for f in DATA.glob("shell.dat*"):
        shutil.copy(f, d / f.name)
    meta = (d / "shell.dat.s3dmm-meta")
    meta.write_bytes(meta.read_bytes()[:-20])
    with pytest.raises(_lib.S3RError, match="truncated|bad subtree record"):
        BlockTreeFieldService(str(d / "shell.dat"))
    shutil.copy(DATA / "shell.dat.s3dmm-meta", meta)
    (d / "shell.dat.s3dmm-field#g").unlink()
    with BlockTreeFieldService(str(d / "shell.dat")) as s:
        s.field_values(0, 0, 0, (0, 0, 0))
        with pytest.raises(_lib.S3RError, match="cannot open the field file"):
            s.field_values(1, 0, 0, (0, 0, 0))


def test_version0_metadata(tmp_path):
    """A v1 file rewritten in the v0 layout (no header; max subtree depth after the tree;
    subtree records without depth) reads the same subtrees with the file-wide depth."""
    src = (DATA / "shell.dat.s3dmm-meta").read_bytes()
    import struct
    id_len = len(b"s3dmm-metadata")
    hdr = id_len + 4 + 8 + 12
    (max_depth,) = struct.unpack_from("<I", src, id_len + 12 + 4)
    tree_pos = struct.unpack_from("<Q", src, hdr)[0]
    pos = tree_pos + 16
    nbits, nbytes = struct.unpack_from("<QQ", src, pos)
    pos += 16 + nbytes
    tree = src[tree_pos:pos]
    (nlevels,) = struct.unpack_from("<Q", src, pos)
    pos += 8
    levels = []
    for _ in range(nlevels):
        (n,) = struct.unpack_from("<Q", src, pos)
        pos += 8
        items = []
        for _ in range(n):
            x, y, z, t, vp, dep = struct.unpack_from("<IIIIQQ", src, pos)
            pos += 32
            items.append((x, y, z, t, vp, dep))
        levels.append(items)
    (ffs,) = struct.unpack_from("<Q", src, pos)
    body = bytearray(tree) + struct.pack("<I", max_depth) + struct.pack("<Q", nlevels)
    for items in levels:
        body += struct.pack("<Q", len(items))
        for x, y, z, t, vp, dep in items:
            body += struct.pack("<IIIIQ", x, y, z, t, vp)
    body += struct.pack("<Q", ffs)
    out = struct.pack("<Q", 8) + bytes(body)
    d = tmp_path / "v0"
    d.mkdir()
    for f in DATA.glob("shell.dat*"):
        shutil.copy(f, d / f.name)
    (d / "shell.dat.s3dmm-meta").write_bytes(out)
    with BlockTreeFieldService(str(d / "shell.dat")) as s, BlockTreeFieldService(str(DATA / "shell.dat")) as ref:
        assert s.metadata().format_version() == 0 and s.metadata().max_full_level() == 0
        a = [x for lv in s.metadata().levels() for x in lv]
        b = [x for lv in ref.metadata().levels() for x in lv]
        assert [(x.level, x.index, x.values_offset) for x in a] == [(x.level, x.index, x.values_offset) for x in b]
        assert all(x.depth == max_depth for x in a)


def _all_tree_blocks(svc):
    md = svc.metadata()
    out, lv = [], 0
    while True:
        b = md.tree_blocks(lv)
        if b.shape[0] == 0:
            break
        out.append(np.concatenate([np.full((b.shape[0], 1), lv, dtype=np.uint32), b], axis=1))
        lv += 1
    return np.concatenate(out), lv


def test_tree_blocks_breadth_first(shell):
    md = shell.metadata()
    assert md.tree_blocks(0).tolist() == [[0, 0, 0]]
    lv1 = md.tree_blocks(1)
    assert lv1.tolist() == [[c & 1, (c >> 1) & 1, c >> 2] for c in range(8)]
    assert md.tree_blocks(2).shape[0] == 64
    blocks, nlev = _all_tree_blocks(shell)
    assert nlev == 7  # full to level 2, refined to level 6


@pytest.mark.parametrize("name", ["shell.dat", "series.dat"])
def test_writer_round_trip_matches_reference_files(name, tmp_path):
    """Rewrite a reference-written dataset from its blocks and values with write_dataset:
    the same subtree roots, tree positions, depths, field file offsets, node lists and values."""
    from revise_gb300.dataset import write_dataset
    with BlockTreeFieldService(str(DATA / name)) as src:
        blocks, _ = _all_tree_blocks(src)
        md = src.metadata()
        names = src.field_names()

        def values_of(k):
            return lambda t, sub, n2i: src.field_values(k, t, sub.level, sub.index)[1]

        out = str(tmp_path / name)
        write_dataset(out, blocks, md.max_subtree_depth(), md.max_full_level(),
                      [(nm, values_of(k)) for k, nm in enumerate(names)], time_steps=src.time_frame_count(),
                      bc_min=md.bounding_cube()[0], bc_size=md.bounding_cube()[1])
        with BlockTreeFieldService(out) as dst:
            assert dst.field_names() == names and dst.time_frame_count() == src.time_frame_count()
            a = [x for lv in md.levels() for x in lv]
            b = [x for lv in dst.metadata().levels() for x in lv]
            assert a == b
            assert dst.metadata().field_file_size() == md.field_file_size()
            for t in range(src.time_frame_count()):
                for x in a:
                    assert np.array_equal(dst.metadata().block_tree_nodes(x.level, x.index),
                                          md.block_tree_nodes(x.level, x.index))
                    for k in range(len(names)):
                        r1, v1 = src.field_values(k, t, x.level, x.index)
                        r2, v2 = dst.field_values(k, t, x.level, x.index)
                        assert r1 == r2 and np.array_equal(v1, v2)


def test_written_dataset_read_by_reference_reader(tmp_path):
    """The reference's own Metadata<3> / BlockTreeNodes / fieldValues read a write_dataset file
    with the reference-written fixture's digests (oracle/_ref/ref_dataset_gen, built with the
    reference tree present)."""
    import subprocess
    gen = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "ref_dataset_gen"
    if not gen.exists():
        pytest.skip("oracle/_ref/ref_dataset_gen not built (needs the reference tree)")
    from revise_gb300.dataset import write_dataset
    with BlockTreeFieldService(str(DATA / "shell.dat")) as src:
        blocks, _ = _all_tree_blocks(src)
        md = src.metadata()
        out = str(tmp_path / "shell.dat")
        write_dataset(out, blocks, md.max_subtree_depth(), md.max_full_level(),
                      [(nm, (lambda k: lambda t, sub, n2i: src.field_values(k, t, sub.level, sub.index)[1])(k))
                       for k, nm in enumerate(src.field_names())])
    d = tmp_path / "dump"
    d.mkdir()
    subprocess.run([str(gen), "dump", out + ".s3dmm-meta", str(d), out + ".s3dmm-field#f", out + ".s3dmm-field#g"],
                   check=True, stdout=subprocess.DEVNULL)
    rows = [list(map(int, ln.split())) for ln in (d / "subtrees.txt").read_text().splitlines()]
    recs = EXPECTED["shell.dat"]["frames"][0]
    assert [[r["level"], *r["idx"], r["depth"], r["tree_index"], r["values_offset"], r["node_count"]]
            for r in recs] == rows
    n2i = np.fromfile(d / "n2i.bin", dtype="<u2")
    vals = [np.fromfile(d / f"values_{k}.bin", dtype="<f4") for k in range(2)]
    pn = pv = 0
    for r in recs:
        n = r["node_count"]
        assert sha(n2i[3 * pn:3 * (pn + n)]) == r["n2i_sha256"]
        assert [sha(v[pv:pv + 2 + n]) for v in vals] == r["values_sha256"]
        pn += n
        pv += 2 + n


def test_workload_written_as_dataset_keeps_blocks_and_values(tmp_path):
    """A synthetic workload written in the reference format (its octree cells recovered from the
    node sets) reads back with the same blocks, depths, node counts and node -> value pairs."""
    from revise_gb300 import workloads
    from revise_gb300.dataset import write_dataset
    w = workloads.small(seed=3, level=2, depths=(1, 2, 3, 4, 5))
    write_dataset(str(tmp_path / "w.dat"), workloads.tree_blocks(w), 5, w.level,
                  [("f", workloads.dataset_values(w))])
    with BlockTreeFieldService(str(tmp_path / "w.dat")) as s:
        assert [len(lv) for lv in s.metadata().levels()] == [1, 8, 64]
        fr = s.read_level(s.level_topology(w.level, w.blocks[:, :3]), 0, 0)
        assert np.array_equal(fr.blocks, w.blocks) and np.array_equal(fr.node_off, w.node_off)
        for b in range(w.nblocks):
            a, c = int(w.node_off[b]), int(w.node_off[b + 1])
            key = lambda n: n[:, 0].astype(np.int64) << 20 | n[:, 1].astype(np.int64) << 10 | n[:, 2]  # noqa: E731
            oa, ob = np.argsort(key(w.n2i[a:c])), np.argsort(key(fr.n2i[a:c]))
            assert np.array_equal(w.n2i[a:c][oa], fr.n2i[a:c][ob])
            assert np.array_equal(w.sparse[a:c][oa].view(np.uint32), fr.sparse[a:c][ob].view(np.uint32))
        # coarser subtrees carry no field; their stored range is computeFieldRange's empty (0, -1)
        rng, vals = s.field_values(0, 0, 0, (0, 0, 0))
        assert rng == (0.0, -1.0) and np.all(vals == np.float32(1e30))
