"""Generates the GPU-measured fixtures (run on a host with the GPU):

    python tests/golden/make_gpu_golden.py [out_dir]      (default: tests/golden)

texture_weights.npz  the texture unit's linear-filter weights, measured by
                     tests/golden/texture_probe.cu (compiled here with nvcc):
                     A (fractions, units of 1/256), W[8, na, na, na] (per texel,
                     k slowest), ramp[4096], nan_case[na, na, na].
refcu_render.npz     the reference's own renderer -- renderKernel<Argb> from its
                     sources (src/s3dmm_cuda/DenseFieldRenderer_cu.cu), fed by its
                     own GPU interpolator (DenseFieldInterpolatorArr_cu_3.cu), both
                     compiled to cubins by `make -C oracle refcu` and launched by
                     oracle/refcu_harness.cpp -- on the scenes of
                     tests/golden/texture_variants.py, block by block in
                     back-to-front order into one ARGB32 viewport: <variant> images.
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def texture_weights(out: Path):
    with tempfile.TemporaryDirectory() as d:
        exe = Path(d) / "texture_probe"
        binf = Path(d) / "probe.bin"
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-o", str(exe),
                        str(Path(__file__).resolve().parent / "texture_probe.cu")], check=True)
        subprocess.run([str(exe), str(binf)], check=True)
        raw = binf.read_bytes()
    na = int(np.frombuffer(raw[:4], np.int32)[0])
    A = np.frombuffer(raw[4:4 + 4 * na], np.int32).copy()
    rest = np.frombuffer(raw[4 + 4 * na:], np.float32)
    n3 = na ** 3
    W = rest[:8 * n3].reshape(8, na, na, na)
    ramp = rest[8 * n3:8 * n3 + 4096]
    nan_case = rest[8 * n3 + 4096:].reshape(na, na, na)
    Wi = np.round(W * 256)
    assert np.array_equal(Wi, W * 256), "weights are not multiples of 1/256"
    np.savez_compressed(out / "texture_weights.npz", A=A, W=Wi.astype(np.uint16), ramp=ramp, nan_case=nan_case)


def refcu_render(out: Path):
    from oracle import refcu
    import texture_variants as tv
    from revise_gb300 import host
    images = {}
    for variant in tv.VARIANTS:
        w = tv.workload(variant)
        view = host.view_for(w)
        refcu.set_tf(w.tf)
        img = np.zeros(w.W * w.H, np.uint32)
        for b in tv.b2f_blocks(w):
            n2i, sp = w.block_nodes(b)
            blk = [int(x) for x in w.blocks[b, :3]]
            refcu.render_block(view, n2i, sp, int(w.blocks[b, 3]), blk, host.block_view_rect(view, blk), img)
        images[variant] = img
    np.savez_compressed(out / "refcu_render.npz", **images)


if __name__ == "__main__":
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent
    out.mkdir(parents=True, exist_ok=True)
    texture_weights(out)
    refcu_render(out)
    print("wrote", out / "texture_weights.npz", out / "refcu_render.npz")
