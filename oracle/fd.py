"""TEST INFRASTRUCTURE ONLY: central finite differences of the FP64 oracle's image loss
L = 1/2 sum over the kept pixels of |I - target|^2, for checking the GPU adjoint.

Evaluations run in a process pool started with `spawn` (the calling test process holds a CUDA
context): each worker receives the frame once (pool initializer) and then evaluates the loss for
one perturbed transfer-function entry or dense value per task, on all kept pixels or on the pixels
a dense value can reach.
"""
from __future__ import annotations

import multiprocessing as mp
from types import SimpleNamespace

import numpy as np

_S = {}


def _init(view_bytes, blocks, vertex_off, dense, rects, tf, target, keep):
    import oracle
    _S.update(view=oracle.OrcView.from_buffer_copy(view_bytes), w=SimpleNamespace(blocks=blocks, vertex_off=vertex_off),
              dense=dense, rects=rects, tf=tf, target=target, keep=keep)


def _loss(job):
    """job = (kind, index, value, pixel ordinals or None): the loss with tf.ravel()[index] (kind 'tf')
    or dense[index] (kind 'dense') set to value, over those of the pixels that are kept."""
    import oracle
    kind, index, value, pix = job
    tf, dense = _S["tf"], _S["dense"]
    if kind == "tf":
        tf = tf.copy()
        tf.reshape(-1)[index] = value
    else:
        dense = dense.copy()
        dense[index] = value
    v = _S["view"]
    W, H = v.W, v.H
    o = np.flatnonzero(_S["keep"]) if pix is None else pix[_S["keep"][pix]]
    pixels = np.stack([o % W, H - 1 - o // W], 1).astype(np.uint32)
    img, _ = oracle.render_frame_f64(v, _S["w"], dense, _S["rects"], tf, pixels, f64=True)
    return 0.5 * float(((img - _S["target"][o]) ** 2).sum())


class LossPool:
    """The frame's loss under single-coordinate perturbations, evaluated by `processes` workers."""

    def __init__(self, view, w, dense, rects, tf, target, keep, processes: int):
        args = (bytes(view), np.ascontiguousarray(w.blocks), np.ascontiguousarray(w.vertex_off),
                np.ascontiguousarray(dense, np.float32), np.ascontiguousarray(rects, np.int32),
                np.ascontiguousarray(tf, np.float32), np.ascontiguousarray(target, np.float64), np.asarray(keep, bool))
        self.pool = mp.get_context("spawn").Pool(processes, initializer=_init, initargs=args)

    def losses(self, jobs):
        return self.pool.map(_loss, jobs)

    def close(self):
        self.pool.close()
        self.pool.join()


def influence_pixels(cam, W: int, H: int, lo, hi) -> np.ndarray:
    """Image ordinals ((H-1-vy)*W + vx) of the pixels whose perspective rays can pass through the world box
    [lo, hi] (camera: eye, e1, e2, n, w, h as s3r_camera holds them), with a 2-pixel margin."""
    eye, e1, e2, n = (np.asarray(x, np.float64) for x in (cam.eye, cam.e1, cam.e2, cam.n))
    xs, ys = [], []
    for c in range(8):
        p = np.array([hi[a] if (c >> a) & 1 else lo[a] for a in range(3)], np.float64)
        q = p - eye
        tau = q @ n / (n @ n)
        if tau <= 0:
            return np.arange(W * H)
        xs.append((q @ e1) / (e1 @ e1) / tau)
        ys.append((q @ e2) / (e2 @ e2) / tau)
    vx = (np.array(xs) / cam.w + 0.5) * W - 0.5
    vy = (np.array(ys) / cam.h + 0.5) * H - 0.5
    x0, x1 = max(int(np.floor(vx.min())) - 2, 0), min(int(np.ceil(vx.max())) + 2, W - 1)
    y0, y1 = max(int(np.floor(vy.min())) - 2, 0), min(int(np.ceil(vy.max())) + 2, H - 1)
    if x1 < x0 or y1 < y0:
        return np.zeros(0, np.int64)
    gx, gy = np.meshgrid(np.arange(x0, x1 + 1), np.arange(y0, y1 + 1))
    return ((H - 1 - gy) * W + gx).ravel()
