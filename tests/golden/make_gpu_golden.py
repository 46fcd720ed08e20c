"""Generates the GPU-measured fixtures (run on a host with the GPU):

    python tests/golden/make_gpu_golden.py [out_dir]      (default: tests/golden)

texture_weights.npz  the texture unit's linear-filter weights, measured by
                     tests/golden/texture_probe.cu (compiled here with nvcc):
                     A (fractions, units of 1/256), W[8, na, na, na] (per texel,
                     k slowest), ramp[4096], nan_case[na, na, na], and the ramp
                     at off-lattice coordinates xs -> ramp_off.
refcu_render.npz     the reference's own renderer -- renderKernel<Argb> from its
                     sources (src/s3dmm_cuda/DenseFieldRenderer_cu.cu), fed by its
                     own GPU interpolator (DenseFieldInterpolatorArr_cu_3.cu), both
                     compiled to cubins by `make -C oracle refcu` and launched by
                     oracle/refcu_harness.cpp -- on the scenes of
                     tests/golden/texture_variants.py, block by block in
                     back-to-front order into one ARGB32 viewport: <variant> images.
refcu_modes.npz      the same for every other field mode (renderKernel<mode>) on
                     the scenes of tests/golden/mode_scenes.py: <mode name> images.
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
    nan_case = rest[8 * n3 + 4096:8 * n3 + 4096 + n3].reshape(na, na, na)
    tail = raw[4 + 4 * na + 4 * (9 * n3 + 4096):]
    m = int(np.frombuffer(tail[:4], np.int32)[0])
    xs = np.frombuffer(tail[4:4 + 4 * m], np.float32).copy()
    ramp_off = np.frombuffer(tail[4 + 4 * m:4 + 8 * m], np.float32).copy()
    Wi = np.round(W * 256)
    assert np.array_equal(Wi, W * 256), "weights are not multiples of 1/256"
    np.savez_compressed(out / "texture_weights.npz", A=A, W=Wi.astype(np.uint16), ramp=ramp, nan_case=nan_case,
                        xs=xs, ramp_off=ramp_off)


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


def refcu_modes(out: Path):
    """The reference's renderKernel<mode> for every other field mode on the scenes of
    tests/golden/mode_scenes.py: refcu_modes.npz, one image per mode name."""
    from oracle import refcu
    import mode_scenes as ms
    import texture_variants as tv
    from revise_gb300 import host
    images = {}
    for name in ms.MODES:
        w, view, pres, sparse2 = ms.scene(name)
        refcu.set_tf(w.tf)
        img = np.full(w.W * w.H, ms.clear_value(pres), np.uint32)
        for b in tv.b2f_blocks(w):
            n2i, sp = w.block_nodes(b)
            blk = [int(x) for x in w.blocks[b, :3]]
            s2 = None if sparse2 is None else sparse2[int(w.node_off[b]):int(w.node_off[b + 1])]
            refcu.render_block_mode(view, pres, n2i, sp, int(w.blocks[b, 3]), blk, host.block_view_rect(view, blk),
                                    img, s2)
        images[name] = img
    np.savez_compressed(out / "refcu_modes.npz", **images)


if __name__ == "__main__":
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent
    out.mkdir(parents=True, exist_ok=True)
    texture_weights(out)
    refcu_render(out)
    refcu_modes(out)
    print("wrote", out / "texture_weights.npz", out / "refcu_render.npz", out / "refcu_modes.npz")
