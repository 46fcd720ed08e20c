"""Generates tests/golden/golden.npz from the reference's own code.

Run where the reference's code has been staged and compiled into oracle/_ref
(`make -C oracle stage ref REFERENCE=<reference root>`):

    python tests/golden/make_golden.py

Contents (all produced by the reference implementation, never by this repo's code):
  interp_*   DenseFieldInterpolator<3>::interpolate on seeded node sets
             (include/s3dmm/DenseFieldInterpolator.hpp:198-419)
  b2f_*      BackToFrontOrder<MacroBlock<3>> orders (include/BackToFrontOrder.hpp:61-359):
             the eye positions and grids of the reference's own known-answer tests
             (tests/test_BackToFrontOrder.cpp:346-684, 1D/2D cases embedded in 3D with
             singleton extra axes) plus seeded random boxes and eyes
  blend_*    blendImagePart on seeded ARGB32 images (src/s3vs_lib/BlendImagePart.hpp:61-145)
  ctf_*      makeColorTransferVector on seeded control points (include/s3vs/ColorTransferFunction.hpp:27-69)
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from revise_gb300 import workloads as wl  # noqa: E402

TREE = ROOT / "oracle" / "_ref" / "tree"  # the staged reference files


def interp_cases(rng):
    cases = []
    w = wl.small(seed=3, level=1, depths=(1, 2, 3, 4, 5))
    for b in range(w.nblocks):
        n2i, v = w.block_nodes(b)
        cases.append((f"small_b{b}", n2i, v, int(w.blocks[b, 3])))
    w1 = wl.cfg1()
    n2i, v = w1.block_nodes(0)
    cases.append(("cfg1", n2i, v, 5))
    # root corners only
    for d in (1, 3):
        n2i = np.array([[(i & 1) << d, ((i >> 1) & 1) << d, ((i >> 2) & 1) << d] for i in range(8)], np.uint16)
        cases.append((f"corners_d{d}", n2i, rng.normal(size=8).astype(np.float32), d))
    # one masked root corner: the sentinel spreads through the whole block
    n2i = np.array([[(i & 1) << 3, ((i >> 1) & 1) << 3, ((i >> 2) & 1) << 3] for i in range(8)], np.uint16)
    vals = rng.normal(size=8).astype(np.float32)
    vals[5] = np.float32(1e30)
    cases.append(("masked_corner_d3", n2i, vals, 3))
    # full refinement at depth 4 with 30% masked nodes
    d = 4
    g = np.stack(np.meshgrid(*[np.arange((1 << d) + 1)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(np.uint16)
    vals = rng.normal(size=g.shape[0]).astype(np.float32)
    vals[rng.random(g.shape[0]) < 0.3] = np.float32(1e30)
    perm = rng.permutation(g.shape[0])
    cases.append(("full_d4_masked", g[perm], vals[perm], d))
    # deep sparse chain: one refined cell per level down to depth 6
    d = 6

    def one(level, cells, count):
        m = np.zeros(cells.shape[0], bool)
        m[0] = True
        return m

    n2i = wl.octree_nodes(d, one, rng)
    cases.append(("chain_d6", n2i, rng.uniform(-2, 2, n2i.shape[0]).astype(np.float32), d))
    return cases


def b2f_cases(rng):
    src = (TREE / "tests" / "test_BackToFrontOrder.cpp").read_text()
    cases = []
    for m in re.finditer(r"format_b2fo_result<(\d)>\((\d+),\s*([^)]*?)\)\s*,", src):
        dim, size, eye = int(m.group(1)), int(m.group(2)), m.group(3)
        vals = [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?", eye)]
        e3 = vals + [0.5] * (3 - len(vals))
        bmax = [size] * dim + [1] * (3 - dim)
        cases.append(([0, 0, 0], bmax, [0.0] * 3, [1.0] * 3, e3))
    for _ in range(40):
        bmin = rng.integers(0, 4, size=3)
        ext = rng.integers(1, 7, size=3)
        bmax = bmin + ext
        cmin = rng.uniform(-5, 0, size=3)
        cmax = cmin + rng.uniform(1, 8, size=3)
        eye = np.where(rng.random(3) < 0.5, rng.uniform(cmin - 3, cmax + 3), rng.uniform(cmin, cmax))
        cases.append((bmin.tolist(), bmax.tolist(), cmin.tolist(), cmax.tolist(), eye.tolist()))
    # the worker's use: a level-4 block cube seen from the reference example camera
    cases.append(([0, 0, 0], [16, 16, 16], [-5.0] * 3, [5.0] * 3, [0.0, 10.0, 35.0]))
    cases.append(([2, 0, 5], [9, 16, 11], [-5.0 + 0.625 * 2, -5.0, -5.0 + 0.625 * 5],
                  [-5.0 + 0.625 * 9, 5.0, -5.0 + 0.625 * 11], [0.3, -1.2, 0.7]))
    return cases


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libs3r_ref.so missing: make -C oracle ref")
    rng = np.random.default_rng(20261203)
    out = {}
    names = []
    for name, n2i, vals, d in interp_cases(rng):
        out[f"interp_{name}_n2i"] = np.asarray(n2i, np.uint16)
        out[f"interp_{name}_sparse"] = np.asarray(vals, np.float32)
        out[f"interp_{name}_depth"] = np.array(d)
        out[f"interp_{name}_dense"] = oracle.ref_interp(n2i, vals, d)
        names.append(name)
    out["interp_names"] = np.array(names)
    bc = b2f_cases(rng)
    for i, (bmin, bmax, cmin, cmax, eye) in enumerate(bc):
        out[f"b2f_{i}_args"] = np.array(bmin + bmax + cmin + cmax + eye, np.float64)
        out[f"b2f_{i}_order"] = oracle.ref_b2f_order(bmin, bmax, cmin, cmax, eye)
    out["b2f_count"] = np.array(len(bc))
    nb = 0
    for i in range(24):
        dw, dh = rng.integers(8, 40, size=2)
        sw, sh = rng.integers(1, 8, size=2)
        off = rng.integers(-5, 5, size=2)
        ox = int(off[0] + rng.integers(0, dw - sw + 1))
        oy = int(off[1] + rng.integers(0, dh - sh + 1))
        dst = rng.integers(0, 2 ** 32, size=(dh, dw), dtype=np.uint64).astype(np.uint32)
        src = rng.integers(0, 2 ** 32, size=(sh, sw), dtype=np.uint64).astype(np.uint32)
        # exercise the alpha special cases
        a_src = rng.choice([0, 255, 1, 128, 254], size=src.shape)
        a_dst = rng.choice([0, 255, 3, 200], size=dst.shape)
        src = (src & 0x00FFFFFF) | (np.where(rng.random(src.shape) < 0.5, a_src, src >> 24).astype(np.uint32) << 24)
        dst = (dst & 0x00FFFFFF) | (np.where(rng.random(dst.shape) < 0.5, a_dst, dst >> 24).astype(np.uint32) << 24)
        just = bool(i % 6 == 5)
        res = dst.copy()
        oracle.blend_image_part(res, src, (ox, oy), just, (int(off[0]), int(off[1])), use_ref=True)
        out[f"blend_{i}_dst"] = dst
        out[f"blend_{i}_src"] = src
        out[f"blend_{i}_args"] = np.array([ox, oy, int(just), int(off[0]), int(off[1])], np.int64)
        out[f"blend_{i}_out"] = res
        nb += 1
    out["blend_count"] = np.array(nb)
    nc = 0
    for i, (npts, count) in enumerate([(0, 16), (1, 16), (2, 256), (3, 512), (5, 256), (7, 100), (4, 7)]):
        xs = np.sort(rng.uniform(-1, 3, size=npts))
        xs = np.unique(xs.astype(np.float32)).astype(np.float64)
        rgba = rng.uniform(0, 1, size=(xs.shape[0], 4))
        out[f"ctf_{i}_xs"] = xs
        out[f"ctf_{i}_rgba"] = rgba
        out[f"ctf_{i}_count"] = np.array(count)
        out[f"ctf_{i}_out"] = oracle.make_ctf(xs, rgba, count, use_ref=True)
        nc += 1
    xs, rgba = wl.colormap_points()
    out[f"ctf_{nc}_xs"], out[f"ctf_{nc}_rgba"], out[f"ctf_{nc}_count"] = xs, rgba, np.array(256)
    out[f"ctf_{nc}_out"] = oracle.make_ctf(xs, rgba, 256, use_ref=True)
    out["ctf_count"] = np.array(nc + 1)
    path = Path(__file__).resolve().parent / "golden.npz"
    np.savez_compressed(path, **out)
    print(path, path.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
