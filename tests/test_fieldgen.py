"""The oracle's restatement of the reference's field generation (generatePropagatedField with
BlockTreeFieldFromFunc) against the field files the reference itself wrote for the dataset
fixtures: every subtree's values and stored range, bit for bit."""
from pathlib import Path

import numpy as np
import pytest

from oracle import fieldgen
from revise_gb300.dataset import BlockTreeFieldService

DATA = Path(__file__).resolve().parent / "golden" / "dataset"


@pytest.mark.parametrize("name,field,func,frame", [
    ("shell.dat", 0, fieldgen.field_f, 0),
    ("shell.dat", 1, fieldgen.field_g(0.0), 0),
    ("series.dat", 0, fieldgen.field_g(0.0), 0),
    ("series.dat", 0, fieldgen.field_g(1.0), 1),
])
def test_oracle_generate_propagated_matches_reference_files(name, field, func, frame):
    with BlockTreeFieldService(str(DATA / name)) as svc:
        out = fieldgen.generate_propagated(svc, func)
        assert len(out) == svc.metadata().metadata_block_count()
        for (lv, ix), vals in out.items():
            rng, ref = svc.field_values(field, frame, lv, ix)
            assert np.array_equal(vals.view(np.uint32), ref.view(np.uint32)), (lv, ix)
            assert fieldgen.field_range(vals) == rng, (lv, ix)


def test_fixture_exercises_both_propagation_cases():
    """Some parents have all 8 child subtrees (averaged), some fewer (function added); the
    deepest level's subtrees have none (function only)."""
    with BlockTreeFieldService(str(DATA / "shell.dat")) as svc:
        md = svc.metadata()
        kinds = set()
        for level in range(md.level_count() - 1):
            kids = {tuple(s.index) for s in md.level_blocks(level + 1)}
            for s in md.level_blocks(level):
                n = sum((2 * s.index[0] + (c & 1), 2 * s.index[1] + ((c >> 1) & 1), 2 * s.index[2] + (c >> 2))
                        in kids for c in range(8))
                kinds.add("all" if n == 8 else ("some" if n else "none"))
        assert {"all", "some"} <= kinds
