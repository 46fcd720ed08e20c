"""TEST INFRASTRUCTURE ONLY: ctypes access to oracle/_build/libs3r_refcu.so, which
runs the reference's own CUDA kernels (compiled from the reference sources into
oracle/_ref/*.cubin) with the reference's host orchestration restated
(oracle/refcu_harness.cpp).  Used by tests/ and bench.py as a checker and as
the reference-CUDA timing leg; available only where the cubins were built."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libs3r_refcu.so"
INTERP_CUBIN = HERE / "_ref" / "ref_interp.cubin"
RENDER_CUBIN = HERE / "_ref" / "ref_render.cubin"

_lib = None


class HarnessView(C.Structure):
    """The harness's view parameters (the field layout of the s3r_view the library's tests pass)."""
    _fields_ = [("eye", C.c_float * 3), ("e1", C.c_float * 3), ("e2", C.c_float * 3), ("n", C.c_float * 3),
                ("w", C.c_float), ("h", C.c_float), ("ortho", C.c_int32), ("reserved", C.c_int32),
                ("view_r", C.c_float * 9), ("view_t", C.c_float * 3), ("W", C.c_uint32), ("H", C.c_uint32),
                ("level", C.c_uint32), ("field_min", C.c_float), ("field_max", C.c_float), ("threshold", C.c_float),
                ("quality", C.c_float), ("tf_n", C.c_uint32), ("alpha_stop", C.c_float), ("filter", C.c_uint32),
                ("reserved2", C.c_uint32 * 2)]


def harness_view(cam: dict, W: int, H: int, level: int, field_min, field_max, threshold, quality, tf_n: int,
                 filter: int = 1) -> HarnessView:
    """HarnessView from an oracle.look_at_camera() camera and the frame parameters."""
    v = HarnessView()
    for f in ("eye", "e1", "e2", "n", "view_r", "view_t"):
        getattr(v, f)[:] = [float(x) for x in cam[f]]
    v.w, v.h = float(cam["w"]), float(cam["h"])
    v.W, v.H, v.level = W, H, level
    v.field_min, v.field_max, v.threshold, v.quality, v.tf_n = field_min, field_max, threshold, quality, tf_n
    v.alpha_stop, v.filter = 2.0, filter
    return v


def available() -> bool:
    return LIB.exists() and INTERP_CUBIN.exists() and RENDER_CUBIN.exists()


def load():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference CUDA harness not built (oracle/_ref cubins + make -C oracle refcu-harness)")
        import torch
        torch.zeros(1, device="cuda")  # primary context current
        lib = C.CDLL(str(LIB))
        lib.ref_cuda_error.restype = C.c_char_p
        if lib.ref_cuda_init(str(INTERP_CUBIN).encode(), str(RENDER_CUBIN).encode()):
            raise RuntimeError(lib.ref_cuda_error().decode())
        _lib = lib
    return _lib


def _check(rc):
    if rc:
        raise RuntimeError(_lib.ref_cuda_error().decode())


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def interp(n2i, sparse, depth):
    lib = load()
    n2i = np.ascontiguousarray(n2i, dtype=np.uint16)
    sparse = np.ascontiguousarray(sparse, dtype=np.float32)
    out = np.empty(((1 << depth) + 1) ** 3, dtype=np.float32)
    _check(lib.ref_cuda_interp(_p(n2i, C.c_uint16), _p(sparse, C.c_float), C.c_uint32(sparse.shape[0]),
                               C.c_uint32(depth), _p(out, C.c_float)))
    return out


def set_tf(tf):
    lib = load()
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    _check(lib.ref_cuda_set_tf(_p(tf, C.c_float), C.c_uint32(tf.shape[0])))


def render_block(view, n2i, sparse, depth, idx, rect, viewport):
    """renderKernel<Argb> for one block into a host ARGB32 viewport (in place)."""
    lib = load()
    n2i = np.ascontiguousarray(n2i, dtype=np.uint16)
    sparse = np.ascontiguousarray(sparse, dtype=np.float32)
    i = (C.c_uint32 * 3)(*[int(x) for x in idx])
    r = (C.c_int32 * 4)(*[int(x) for x in rect])
    _check(lib.ref_cuda_render_block(C.byref(view), _p(n2i, C.c_uint16), _p(sparse, C.c_float),
                                     C.c_uint32(sparse.shape[0]), C.c_uint32(depth), i, r, _p(viewport, C.c_uint32)))


def worker(view, w, order_idx, rects):
    """The reference worker loop over w's blocks in the given order; returns (viewport, crop, ms)."""
    lib = load()
    blocks = np.ascontiguousarray(w.blocks[order_idx], dtype=np.uint32)
    counts = np.diff(w.node_off.astype(np.int64))[order_idx]
    node_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    n2i = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[0] for b in order_idx]), dtype=np.uint16)
    sparse = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[1] for b in order_idx]), dtype=np.float32)
    rects = np.ascontiguousarray(rects[order_idx], dtype=np.int32)
    vp = np.zeros(view.W * view.H, dtype=np.uint32)
    crop = (C.c_int32 * 4)()
    ms = C.c_double()
    _check(lib.ref_cuda_worker(C.byref(view), C.c_uint32(blocks.shape[0]), _p(blocks, C.c_uint32),
                               _p(node_off, C.c_uint64), _p(n2i, C.c_uint16), _p(sparse, C.c_float),
                               _p(rects, C.c_int32), _p(vp, C.c_uint32), crop, C.byref(ms)))
    return vp, tuple(crop[:]), ms.value


def worker_kernel_ms(view, w, order_idx, rects):
    """The reference worker loop with each kernel launch timed by CUDA events: (interpolation kernels ms,
    renderKernel<Argb> ms) summed over the blocks, host copies excluded."""
    lib = load()
    blocks = np.ascontiguousarray(w.blocks[order_idx], dtype=np.uint32)
    counts = np.diff(w.node_off.astype(np.int64))[order_idx]
    node_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    n2i = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[0] for b in order_idx]), dtype=np.uint16)
    sparse = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[1] for b in order_idx]), dtype=np.float32)
    rects = np.ascontiguousarray(rects[order_idx], dtype=np.int32)
    im, rm = C.c_double(), C.c_double()
    _check(lib.ref_cuda_worker_kernel_ms(C.byref(view), C.c_uint32(blocks.shape[0]), _p(blocks, C.c_uint32),
                                        _p(node_off, C.c_uint64), _p(n2i, C.c_uint16), _p(sparse, C.c_float),
                                        _p(rects, C.c_int32), C.byref(im), C.byref(rm)))
    return im.value, rm.value


def render_block_mode(view, pres, n2i, sparse, depth, idx, rect, viewport, sparse2=None):
    """renderKernel<pres.mode> for one block into a host ARGB32 viewport (in place);
    pres: a revise_gb300._lib.Presentation; sparse2: the secondary field's node values."""
    lib = load()
    n2i = np.ascontiguousarray(n2i, dtype=np.uint16)
    sparse = np.ascontiguousarray(sparse, dtype=np.float32)
    s2 = None if sparse2 is None else np.ascontiguousarray(sparse2, dtype=np.float32)
    i = (C.c_uint32 * 3)(*[int(x) for x in idx])
    r = (C.c_int32 * 4)(*[int(x) for x in rect])
    _check(lib.ref_cuda_render_block_mode(C.byref(view), C.byref(pres), _p(n2i, C.c_uint16), _p(sparse, C.c_float),
                                          _p(s2, C.c_float) if s2 is not None else None,
                                          C.c_uint32(sparse.shape[0]), C.c_uint32(depth), i, r,
                                          _p(viewport, C.c_uint32)))


def time_render(view, pres, w, order_idx, rects, sparse2=None, clear=0):
    """Kernel time (ms, summed CUDA-event times of the render launches) of the reference's
    renderKernel<pres.mode> over w's blocks in the given order, each block's field interpolated
    first (not timed); returns (ms, viewport)."""
    lib = load()
    blocks = np.ascontiguousarray(w.blocks[order_idx], dtype=np.uint32)
    counts = np.diff(w.node_off.astype(np.int64))[order_idx]
    node_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    n2i = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[0] for b in order_idx]), dtype=np.uint16)
    sparse = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[1] for b in order_idx]), dtype=np.float32)
    s2 = None
    if sparse2 is not None:
        s2 = np.ascontiguousarray(np.concatenate([sparse2[int(w.node_off[b]):int(w.node_off[b + 1])]
                                                  for b in order_idx]), dtype=np.float32)
    rects = np.ascontiguousarray(rects[order_idx], dtype=np.int32)
    vp = np.full(view.W * view.H, clear, dtype=np.uint32)
    ms = C.c_double()
    _check(lib.ref_cuda_time_render(C.byref(view), C.byref(pres), C.c_uint32(blocks.shape[0]), _p(blocks, C.c_uint32),
                                    _p(node_off, C.c_uint64), _p(n2i, C.c_uint16), _p(sparse, C.c_float),
                                    _p(s2, C.c_float) if s2 is not None else None, _p(rects, C.c_int32),
                                    _p(vp, C.c_uint32), C.byref(ms)))
    return ms.value, vp


def time_render_graph(view, pres, w, order_idx, rects, sparse2=None, reps: int = 5):
    """GPU time (ms) of the reference's renderKernel<pres.mode> over w's blocks in the given order, back to
    back: each block's field interpolated into a texture of its own first (not timed), the launches
    captured into one CUDA graph and replayed; ms per replay."""
    lib = load()
    blocks = np.ascontiguousarray(w.blocks[order_idx], dtype=np.uint32)
    counts = np.diff(w.node_off.astype(np.int64))[order_idx]
    node_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    n2i = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[0] for b in order_idx]), dtype=np.uint16)
    sparse = np.ascontiguousarray(np.concatenate([w.block_nodes(int(b))[1] for b in order_idx]), dtype=np.float32)
    s2 = None
    if sparse2 is not None:
        s2 = np.ascontiguousarray(np.concatenate([sparse2[int(w.node_off[b]):int(w.node_off[b + 1])]
                                                  for b in order_idx]), dtype=np.float32)
    rects = np.ascontiguousarray(rects[order_idx], dtype=np.int32)
    ms = C.c_double()
    _check(lib.ref_cuda_time_render_graph(C.byref(view), C.byref(pres), C.c_uint32(blocks.shape[0]),
                                          _p(blocks, C.c_uint32), _p(node_off, C.c_uint64), _p(n2i, C.c_uint16),
                                          _p(sparse, C.c_float), _p(s2, C.c_float) if s2 is not None else None,
                                          _p(rects, C.c_int32), C.c_uint32(reps), C.byref(ms)))
    return ms.value
