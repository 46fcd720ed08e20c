"""Makes tests/golden/splits.json from the reference's own IndexCubeSplitter and BackToFrontOrder
(oracle/_ref/libs3r_ref.so, oracle/Makefile target `ref`): the split boxes for (level, count) pairs
and their back-to-front order for eyes inside, outside and exactly on box boundaries.

Run from the repository root:  python tests/golden/make_splits.py
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402

CASES = [(0, 1), (0, 3), (1, 1), (1, 2), (1, 5), (1, 8), (1, 9), (2, 2), (2, 3), (2, 5), (2, 9), (2, 16),
         (2, 20), (2, 64), (2, 100), (3, 7), (3, 32), (3, 100), (3, 512), (4, 24), (4, 1024)]
EYES = [(0.1, 0.1, 0.1), (0.0, 10.0, 35.0), (-7.0, 3.0, -2.5), (2.5, 0.0, -5.0), (5.0, 5.0, 5.0),
        (-1.25, 1.25, 3.75), (30.0, -40.0, 12.0), (0.0, 0.0, 0.0), (4.9, -4.9, 0.6)]


def main():
    out = []
    for level, count in CASES:
        rec = {"level": level, "count": count,
               "boxes": oracle.ref_split_cube(level, count, False).tolist(),
               "boxes_trailing": oracle.ref_split_cube(level, count, True).tolist(),
               "b2f": [{"eye": list(e), "boxes": oracle.ref_split_b2f(level, count, e).tolist()}
                       for e in (EYES if count < 500 else EYES[:3])]}
        out.append(rec)
    (ROOT / "tests" / "golden" / "splits.json").write_text(json.dumps(out, separators=(",", ":")) + "\n")
    print("wrote", len(out), "cases")


if __name__ == "__main__":
    main()
