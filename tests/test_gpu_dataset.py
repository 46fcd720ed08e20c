"""Dataset -> GPU: the reference-format fixtures read by s3r_dataset_*, uploaded
through the pinned staging path and interpolated by the batched plan and the
per-block generator, bit-exact against the oracle's CPU interpolation."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from revise_gb300 import _lib
from revise_gb300.dataset import BlockTreeFieldService

pytestmark = pytest.mark.gpu

DATA = Path(__file__).resolve().parent / "golden" / "dataset"


def _same(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


@pytest.fixture(scope="module")
def shell():
    with BlockTreeFieldService(str(DATA / "shell.dat")) as s:
        yield s


def test_upload_level_equals_host_read(ctx, shell):
    import torch
    for level in range(shell.metadata().level_count()):
        fr = shell.level_topology(level)
        shell.read_level(fr, 0, 0)
        dev = torch.full((fr.nodes,), float("nan"), device="cuda")
        ranges = np.empty((fr.nblocks, 2), dtype=np.float32)
        s = torch.cuda.Stream()
        shell.upload(ctx, fr, 0, 0, dev, ranges, stream=s)
        s.synchronize()
        assert np.array_equal(dev.cpu().numpy().view(np.uint32), fr.sparse.view(np.uint32))
        assert np.array_equal(ranges, fr.ranges)


def test_upload_double_buffered_frames(ctx):
    """Frames alternate between the two staging buffers; every copy lands intact."""
    import torch
    with BlockTreeFieldService(str(DATA / "series.dat")) as svc:
        fr = svc.level_topology(2)
        outs = [torch.empty(fr.nodes, device="cuda") for _ in range(4)]
        for k, o in enumerate(outs):
            svc.upload(ctx, fr, 0, k % 2, o)
        torch.cuda.synchronize()
        for k, o in enumerate(outs):
            svc.read_level(fr, 0, k % 2)
            assert np.array_equal(o.cpu().numpy(), fr.sparse), k
        assert not np.array_equal(outs[0].cpu().numpy(), outs[1].cpu().numpy())


def test_level_plan_interp_matches_oracle(ctx, shell):
    import torch
    from revise_gb300.api import FramePlan
    for level in (2, 3):
        fr = shell.read_level(shell.level_topology(level), 1, 0)
        dev = torch.empty(fr.nodes, device="cuda")
        shell.upload(ctx, fr, 1, 0, dev)
        for tile in (8, 16):
            plan = FramePlan(ctx, fr, _lib.BRICK_F32, tile_cells=tile)
            plan.interp(dev)
            torch.cuda.synchronize()
            assert _same(plan.dense().cpu().numpy(), oracle.interp_workload(fr)), (level, tile)
            plan.close()


def test_service_interpolate_per_block(ctx, shell):
    md = shell.metadata()
    for s in md.level_blocks(3)[:6] + md.level_blocks(0):
        rng, dense = shell.interpolate(ctx, 0, 0, s.level, s.index)
        assert rng == shell.field_range(0)
        _, vals = shell.field_values(0, 0, s.level, s.index)
        ref = oracle.interp_f32(md.block_tree_nodes(s.level, s.index), vals, s.depth)
        assert _same(dense.cpu().numpy(), ref), (s.level, s.index)
