"""Work split, back-to-front box order and render graph vs the reference (its own
IndexCubeSplitter / BackToFrontOrder compiled in place: tests/golden/splits.json, and live when
oracle/_ref is built), and the host assemble tree's semantics."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from revise_gb300 import host, schedule

SPLITS = json.loads((Path(__file__).resolve().parent / "golden" / "splits.json").read_text())


@pytest.mark.parametrize("case", SPLITS, ids=lambda c: f"L{c['level']}n{c['count']}")
def test_split_and_b2f_match_reference_fixture(case):
    lv, n = case["level"], case["count"]
    assert schedule.split_index_cube(lv, n).tolist() == case["boxes"]
    assert schedule.split_index_cube(lv, n, add_trailing_empty=True).tolist() == case["boxes_trailing"]
    for e in case["b2f"]:
        assert schedule.boxes_sorted(lv, n, e["eye"]).tolist() == e["boxes"], e["eye"]


def test_split_and_b2f_match_reference_live_random_eyes():
    if not oracle.ref_available():
        pytest.skip("oracle/_ref not built (needs the reference tree)")
    rng = np.random.default_rng(7)
    for _ in range(300):
        lv = int(rng.integers(0, 5))
        n = int(rng.integers(1, 70))
        # eyes on boundaries (multiples of 10/2^k), inside and outside the cube
        e = np.where(rng.random(3) < 0.4, np.round(rng.uniform(-6, 6, 3) * 1.6) / 1.6, rng.uniform(-40, 40, 3))
        assert schedule.boxes_sorted(lv, n, e).tolist() == oracle.ref_split_b2f(lv, n, e).tolist(), (lv, n, e)
        assert schedule.split_index_cube(lv, n, True).tolist() == oracle.ref_split_cube(lv, n, True).tolist()


def test_split_covers_the_cube_once():
    for lv, n in [(2, 5), (3, 37), (2, 100), (4, 300)]:
        boxes = schedule.split_index_cube(lv, n).astype(np.int64)
        m = 1 << lv
        cover = np.zeros((m, m, m), dtype=np.int32)
        for b in boxes:
            cover[b[2]:b[5], b[1]:b[4], b[0]:b[3]] += 1
        assert (cover == 1).all()


def test_b2f_boxes_are_a_visibility_order():
    """No box is drawn before one it hides: for boxes in one row along an axis (same ranges on the
    other two), the one on the eye's side of their separation comes later."""
    for eye in [(1.3, -0.2, 20.0), (0.1, 0.2, 0.3), (-30.0, 7.0, 2.0), (2.5, 2.5, -2.5)]:
        for lv, n in [(3, 64), (3, 20), (2, 9)]:
            boxes = schedule.boxes_sorted(lv, n, eye).astype(np.float64)
            h = 10.0 / (1 << lv)
            lo, hi = boxes[:, :3] * h - 5, boxes[:, 3:] * h - 5
            e = np.asarray(eye)
            for i in range(len(boxes)):
                for j in range(i + 1, len(boxes)):
                    for a in range(3):
                        o = [k for k in range(3) if k != a]
                        if not (np.array_equal(lo[i, o], lo[j, o]) and np.array_equal(hi[i, o], hi[j, o])):
                            continue
                        assert not (hi[j, a] <= lo[i, a] and e[a] > lo[i, a]), (eye, lv, n, i, j, a)
                        assert not (hi[i, a] <= lo[j, a] and e[a] < hi[i, a]), (eye, lv, n, i, j, a)


@pytest.mark.parametrize("affinity,expected", [
    ([1], [("Render", []), ("FinalCompose", [0])]),
    ([2], [("Render", []), ("Render", []), ("Assemble", [0, 1]), ("FinalCompose", [2])]),
    ([3], [("Render", []), ("Render", []), ("Render", []), ("Assemble", [0, 1]), ("Assemble", [3, 2]),
           ("FinalCompose", [4])]),
    ([2, 1], [("Render", []), ("Render", []), ("Assemble", [0, 1]), ("Render", []), ("Assemble", [2, 3]),
              ("FinalCompose", [4])]),
])
def test_render_graph_structure(affinity, expected):
    g = schedule.render_graph(affinity)
    assert [(t.kind, t.inputs) for t in g.tasks] == expected
    assert len(g.worker_tasks) == sum(affinity)


def test_affinity_for():
    assert schedule.affinity_for(7, 4) == [4, 3]
    assert schedule.affinity_for(8, 4) == [4, 4]
    assert schedule.affinity_for(3, 4) == [3]


def _rand_part(rng, W, H):
    w, h = int(rng.integers(1, 40)), int(rng.integers(1, 30))
    ox, oy = int(rng.integers(0, W - w)), int(rng.integers(0, H - h))
    a = rng.integers(0, 256, (h, w)).astype(np.uint32)
    a[rng.random((h, w)) < 0.3] = 255
    a[rng.random((h, w)) < 0.3] = 0
    px = (a << 24) | rng.integers(0, 1 << 24, (h, w)).astype(np.uint32)
    return schedule.Part((ox, oy), px)


def test_assemble_tree_follows_the_reference_pairing():
    """The tree result equals the reference's pairwise evaluation written out by hand, and differs
    from blending the parts one after another (the integer blend is not associative)."""
    rng = np.random.default_rng(3)
    W, H = 80, 60
    differs = False
    for _ in range(20):
        parts = [_rand_part(rng, W, H) for _ in range(4)]
        g = schedule.render_graph([4])
        got = schedule.run_graph(g, parts, W, H, background=0xFF102030)
        a01 = schedule.assemble(parts[0], parts[1])
        a23 = schedule.assemble(parts[2], parts[3])
        want = schedule.final_compose(schedule.assemble(a01, a23), W, H, 0xFF102030)
        assert np.array_equal(got, want)
        seq = np.full((H, W), 0xFF102030, dtype=np.uint32)
        for p in parts:
            host.blend_image_part(seq, p.pixels, p.origin)
        differs |= not np.array_equal(seq, got)
    assert differs


def test_assemble_with_empty_parts():
    empty = schedule.Part((0, 0), np.zeros((0, 0), dtype=np.uint32))
    p = schedule.Part((10, 5), np.full((3, 4), 0xFF00FF00, dtype=np.uint32))
    a = schedule.assemble(empty, p)
    assert a.origin == (0, 0) and a.size == (14, 8)   # the empty part's origin joins the box
    assert (a.pixels[5:8, 10:14] == 0xFF00FF00).all() and a.pixels[:5].max() == 0
    img = schedule.run_graph(schedule.render_graph([2]), [empty, empty], 16, 16, background=7)
    assert (img == 7).all()
