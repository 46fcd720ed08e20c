"""Makes the dataset fixtures under tests/golden/dataset/ with the reference's own code.

Builds oracle/_ref/ref_dataset_gen (oracle/Makefile, target `ref`: the
reference's Metadata, MetadataProvider, BlockTreeFieldProvider and
BlockTreeFieldFromFunc compiled in place from the reference tree), lets it
write two small datasets in the reference's on-disk format:

  shell.dat          one time frame, fields f and g; a block tree full to level 2
                     of [-5, 5]^3 and refined to level 6 on a sphere shell;
                     subtree roots on levels 0-3 (max subtree depth 3); values
                     written with the Propagate policy (child subtrees averaged
                     into their parents, the function where children are missing)
  series.dat         two time frames in series/ (per-frame metadata and field g)

and then dumps what the reference's own readers return for them (Metadata<3>
levels, blockTreeNodes n2i, BlockTreeFieldProvider::fieldValues).  The dataset
files are copied here; expected.json keeps per subtree its record and SHA-256
digests of its n2i list (uint16 x, y, z) and of its {min, max, values} per field
and frame.

Run from the repository root:  python tests/golden/make_dataset.py
"""
from __future__ import annotations

import hashlib
import json
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "dataset"
GEN = ROOT / "oracle" / "_ref" / "ref_dataset_gen"


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def dump(meta: Path, field_files: list[Path], tmp: Path) -> list[dict]:
    d = tmp / ("dump_" + meta.name)
    d.mkdir()
    subprocess.run([str(GEN), "dump", str(meta), str(d), *map(str, field_files)], check=True,
                   stdout=subprocess.DEVNULL)
    rows = [list(map(int, ln.split())) for ln in (d / "subtrees.txt").read_text().splitlines()]
    n2i = np.fromfile(d / "n2i.bin", dtype="<u2")
    vals = [np.fromfile(d / f"values_{k}.bin", dtype="<f4") for k in range(len(field_files))]
    out, pn, pv = [], 0, 0
    for level, x, y, z, depth, tree, pos, count in rows:
        rec = {"level": level, "idx": [x, y, z], "depth": depth, "tree_index": tree, "values_offset": pos,
               "node_count": count, "n2i_sha256": sha(n2i[3 * pn:3 * (pn + count)].tobytes()),
               "values_sha256": [sha(v[pv:pv + 2 + count].tobytes()) for v in vals],
               "range": [[float(v[pv]), float(v[pv + 1])] for v in vals],
               "values_sum": [float(np.where(v[pv + 2:pv + 2 + count] < 1e29, v[pv + 2:pv + 2 + count], 0)
                                    .astype(np.float64).sum()) for v in vals]}
        out.append(rec)
        pn += count
        pv += 2 + count
    assert pn * 3 == n2i.size and all(pv == v.size for v in vals)
    return out


def main() -> int:
    # the reference's writer, compiled from the staged reference files (make -C oracle stage REFERENCE=<root>)
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "_ref/ref_dataset_gen"], check=True)
    with tempfile.TemporaryDirectory() as t:
        tmp = Path(t)
        data = tmp / "data"
        data.mkdir()
        for name, variant in (("shell.dat", "shell"), ("series.dat", "frames")):
            subprocess.run([str(GEN), "write", str(data / name), variant], check=True, stdout=subprocess.DEVNULL)
        expected = {
            "shell.dat": {
                "time_steps": 1, "fields": ["f", "g"],
                "frames": [dump(data / "shell.dat.s3dmm-meta",
                                [data / "shell.dat.s3dmm-field#f", data / "shell.dat.s3dmm-field#g"], tmp)],
            },
            "series.dat": {
                "time_steps": 2, "fields": ["g"],
                "frames": [dump(data / "series" / f"series_t{t:06d}.dat.s3dmm-meta",
                                [data / "series" / f"series_t{t:06d}.dat.s3dmm-field#g"], tmp) for t in range(2)],
            },
        }
        if OUT.exists():
            shutil.rmtree(OUT)
        shutil.copytree(data, OUT)
        (OUT / "expected.json").write_text(json.dumps(expected, separators=(",", ":")) + "\n")
    print("wrote", OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main())
