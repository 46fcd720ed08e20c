"""The seeded workload generator: node sets are valid octree node sets."""
import numpy as np

from revise_gb300 import workloads


def _check_block(n2i, d):
    assert n2i.dtype == np.uint16
    assert n2i.max() <= (1 << d)
    keys = n2i[:, 0].astype(np.int64) << 40 | n2i[:, 1].astype(np.int64) << 20 | n2i[:, 2].astype(np.int64)
    assert np.unique(keys).size == keys.size
    corners = {((i & 1) << d, ((i >> 1) & 1) << d, ((i >> 2) & 1) << d) for i in range(8)}
    assert corners <= {tuple(x) for x in n2i.tolist()}
    # the deepest level is reached: some node has an odd coordinate
    assert (n2i % 2 == 1).any()


def test_small_and_cfg1_are_valid_and_deterministic():
    for w in (workloads.small(), workloads.cfg1(), workloads.small(seed=5, depths=(1, 5))):
        for b in range(w.nblocks):
            n2i, v = w.block_nodes(b)
            _check_block(n2i, int(w.blocks[b, 3]))
            assert v.dtype == np.float32
    a, b = workloads.small(seed=7), workloads.small(seed=7)
    assert np.array_equal(a.n2i, b.n2i) and np.array_equal(a.sparse, b.sparse)


def test_cfg1_matches_its_specification():
    w = workloads.cfg1()
    assert (w.nblocks, int(w.blocks[0, 3]), w.W, w.H, w.ortho, w.quality) == (1, 5, 512, 512, True, 2.0)
    n2i, v = w.block_nodes(0)
    u = n2i / 32.0
    r = np.linalg.norm(u - 0.5, axis=1)
    assert np.all((v == np.float32(1e30)) == (r >= 0.45))
    f = np.sin(4 * np.pi * u[:, 0]) * np.cos(4 * np.pi * u[:, 1]) + u[:, 2]
    np.testing.assert_allclose(v[r < 0.45], f[r < 0.45], rtol=1e-6, atol=1e-6)
    assert w.tf.shape == (256, 4) and (w.field_min, w.field_max) == (-1.0, 2.0)


def test_workload_color_table_equals_the_library_table():
    """Workloads build their transfer-function tables in numpy (no native code loads while generating
    inputs): bit-identical to s3r_make_color_transfer on the default and on random control points."""
    from revise_gb300 import host
    xs, rgba = workloads.colormap_points()
    cases = [(xs, rgba, n) for n in (2, 5, 256, 512, 1000)]
    rng = np.random.default_rng(0)
    for _ in range(100):
        x = np.unique(np.sort(rng.uniform(-3, 3, int(rng.integers(2, 8)))))
        cases.append((x, rng.uniform(0, 1, (x.size, 4)), int(rng.integers(2, 600))))
    for x, c, n in cases:
        a = workloads.color_table(x, c, n)
        b = np.asarray(host.make_color_transfer(x, c, n), np.float32)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), n
