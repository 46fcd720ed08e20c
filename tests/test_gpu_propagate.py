"""GPU propagation (s3r_dataset_propagate + s3r_field_divide) against the field files the
reference's generatePropagatedField wrote: averaged parents straight from the GPU, parents with
missing children after the oracle's BlockTreeFieldFromFunc contributions; bit for bit."""
from pathlib import Path

import numpy as np
import pytest

from oracle import fieldgen
from revise_gb300 import _lib
from revise_gb300.dataset import BlockTreeFieldService, field_divide

pytestmark = pytest.mark.gpu

DATA = Path(__file__).resolve().parent / "golden" / "dataset"


def _level_values(svc, field, frame, level):
    subs = svc.metadata().level_blocks(level)
    vals = [svc.field_values(field, frame, level, s.index)[1] for s in subs]
    return subs, (np.concatenate(vals) if vals else np.zeros(0, np.float32))


@pytest.mark.parametrize("name,field,func,frame", [
    ("shell.dat", 0, fieldgen.field_f, 0),
    ("shell.dat", 1, fieldgen.field_g(0.0), 0),
    ("series.dat", 0, fieldgen.field_g(1.0), 1),
])
def test_propagation_matches_reference_files(ctx, name, field, func, frame):
    import torch
    with BlockTreeFieldService(str(DATA / name)) as svc:
        md = svc.metadata()
        levels, lv = [], 0
        while md.tree_blocks(lv).shape[0]:
            levels.append(md.tree_blocks(lv))
            lv += 1
        tree = fieldgen.Tree(levels, *md.bounding_cube())
        for level in range(md.level_count() - 2, -1, -1):
            _, child = _level_values(svc, field, frame, level + 1)
            subs, want = _level_values(svc, field, frame, level)
            child_dev = torch.from_numpy(child).cuda()
            sums = torch.empty(want.size, device="cuda")
            weights = torch.empty(want.size, device="cuda")
            counts = svc.propagate(ctx, level, child_dev, sums, weights)
            assert counts.shape == (len(subs),) and counts.max() <= 8
            s_h, w_h = sums.cpu().numpy(), weights.cpu().numpy()
            off = 0
            for s, n_kids in zip(subs, counts):
                n = s.node_count
                if n_kids < 8:  # the reference's generator adds the function at every block corner
                    n2i = md.block_tree_nodes(level, s.index)
                    fieldgen.add_function(tree, level, s.index, s.depth, n2i, func, s_h[off:off + n], w_h[off:off + n])
                off += n
            out = torch.empty_like(sums)
            field_divide(ctx, torch.from_numpy(s_h).cuda(), torch.from_numpy(w_h).cuda(), out)
            got = out.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (name, level)


def test_propagation_of_synthetic_children_matches_oracle(ctx):
    """Arbitrary child values (masked ones included) through the GPU step and the oracle's child loop."""
    import torch
    rng = np.random.default_rng(5)
    with BlockTreeFieldService(str(DATA / "shell.dat")) as svc:
        md = svc.metadata()
        for level in (2, 1, 0):
            csubs = md.level_blocks(level + 1)
            cvals = {tuple(s.index): np.where(rng.random(s.node_count) < 0.25, np.float32(1e30),
                                              rng.standard_normal(s.node_count).astype(np.float32))
                     for s in csubs}
            child = np.concatenate([cvals[tuple(s.index)] for s in csubs])
            subs = md.level_blocks(level)
            total = sum(s.node_count for s in subs)
            sums = torch.empty(total, device="cuda")
            weights = torch.empty(total, device="cuda")
            svc.propagate(ctx, level, torch.from_numpy(child).cuda(), sums, weights)
            s_h, w_h = sums.cpu().numpy(), weights.cpu().numpy()
            off = 0
            for s in subs:
                n2i = md.block_tree_nodes(level, s.index)
                f = np.zeros(s.node_count, np.float32)
                w = np.zeros(s.node_count, np.float32)
                kids = []
                for c in range(8):
                    ci = (2 * s.index[0] + (c & 1), 2 * s.index[1] + ((c >> 1) & 1), 2 * s.index[2] + (c >> 2))
                    if ci in cvals:
                        kids.append((c, md.subtree_depth(level + 1, ci), md.block_tree_nodes(level + 1, ci), cvals[ci]))
                fieldgen.propagate_into(n2i, s.depth, kids, f, w)
                assert np.array_equal(s_h[off:off + s.node_count].view(np.uint32), f.view(np.uint32)), (level, s.index)
                assert np.array_equal(w_h[off:off + s.node_count], w)
                off += s.node_count


def test_deepest_level_has_no_children(ctx):
    import torch
    with BlockTreeFieldService(str(DATA / "shell.dat")) as svc:
        md = svc.metadata()
        top = md.level_count() - 1
        n = sum(s.node_count for s in md.level_blocks(top))
        sums = torch.full((n,), 7.0, device="cuda")
        weights = torch.full((n,), 7.0, device="cuda")
        counts = svc.propagate(ctx, top, None, sums, weights)
        assert counts.max() == 0
        assert float(sums.abs().max()) == 0.0 and float(weights.abs().max()) == 0.0
        vals = torch.empty(n, device="cuda")
        field_divide(ctx, sums, weights, vals)
        assert bool((vals == 1e30).all())
