"""Oracle (TEST INFRASTRUCTURE ONLY): ctypes access to the C restatement of the
reference's hot path (oracle/s3r_oracle.c -> oracle/_build/libs3r_oracle.so)
and, where it was built, to the reference's own code compiled in place
(oracle/ref_harness.cpp -> oracle/_ref/libs3r_ref.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs use this package, and only as the checker or the CPU baseline; the
product (revise_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libs3r_oracle.so"
REF_LIB = HERE / "_ref" / "libs3r_ref.so"

_port = None
_ref = None


class OrcCamera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("e1", C.c_float * 3), ("e2", C.c_float * 3), ("n", C.c_float * 3),
                ("w", C.c_float), ("h", C.c_float), ("ortho", C.c_int32), ("pad_", C.c_int32)]


class OrcView(C.Structure):
    _fields_ = [("cam", OrcCamera), ("W", C.c_uint32), ("H", C.c_uint32), ("level", C.c_uint32),
                ("field_min", C.c_float), ("field_max", C.c_float), ("threshold", C.c_float),
                ("quality", C.c_float), ("tf_n", C.c_uint32), ("filter", C.c_uint32)]


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def build_port() -> None:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)


def port():
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            build_port()
        _port = C.CDLL(str(PORT_LIB))
        _port.orc_render_frame_grad_f64.restype = C.c_double
    return _port


def ref_available() -> bool:
    return REF_LIB.exists()


def ref():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise RuntimeError("oracle/_ref/libs3r_ref.so is not built (make -C oracle ref, needs the reference tree)")
        _ref = C.CDLL(str(REF_LIB))
    return _ref


def view_from(v) -> OrcView:
    """OrcView from a revise_gb300._lib.View (same camera and frame parameters)."""
    o = OrcView()
    for f in ("eye", "e1", "e2", "n"):
        getattr(o.cam, f)[:] = getattr(v.cam, f)[:]
    o.cam.w, o.cam.h, o.cam.ortho = v.cam.w, v.cam.h, v.cam.ortho
    o.W, o.H, o.level = v.W, v.H, v.level
    o.field_min, o.field_max, o.threshold, o.quality, o.tf_n = v.field_min, v.field_max, v.threshold, v.quality, v.tf_n
    o.filter = v.filter
    return o


# ---------------------------------------------------------------- interpolation

def interp_f32(n2i: np.ndarray, sparse: np.ndarray, depth: int) -> np.ndarray:
    n2i = np.ascontiguousarray(n2i, dtype=np.uint16)
    sparse = np.ascontiguousarray(sparse, dtype=np.float32)
    e = (1 << depth) + 1
    out = np.empty(e ** 3, dtype=np.float32)
    port().orc_interp_dense_f32(_p(n2i, C.c_uint16), _p(sparse, C.c_float), C.c_uint32(sparse.shape[0]),
                                C.c_uint32(depth), _p(out, C.c_float))
    return out


def interp_f64(n2i: np.ndarray, sparse: np.ndarray, depth: int) -> np.ndarray:
    n2i = np.ascontiguousarray(n2i, dtype=np.uint16)
    sparse = np.ascontiguousarray(sparse, dtype=np.float32)
    e = (1 << depth) + 1
    out = np.empty(e ** 3, dtype=np.float64)
    port().orc_interp_dense_f64(_p(n2i, C.c_uint16), _p(sparse, C.c_float), C.c_uint32(sparse.shape[0]),
                                C.c_uint32(depth), _p(out, C.c_double))
    return out


def ref_interp(n2i: np.ndarray, sparse: np.ndarray, depth: int) -> np.ndarray:
    """The reference's own DenseFieldInterpolator<3>::interpolate."""
    n2i = np.ascontiguousarray(n2i, dtype=np.uint16)
    sparse = np.ascontiguousarray(sparse, dtype=np.float32)
    e = (1 << depth) + 1
    out = np.empty(e ** 3, dtype=np.float32)
    ref().ref_interp_dense(_p(n2i, C.c_uint16), _p(sparse, C.c_float), C.c_uint32(sparse.shape[0]),
                           C.c_uint32(depth), _p(out, C.c_float))
    return out


def interp_workload(w, blocks=None, f64: bool = False) -> np.ndarray:
    """Concatenated dense grids of a workload's blocks (all or the listed ones)."""
    vo = w.vertex_off
    out = np.full(int(vo[-1]), np.nan, dtype=np.float64 if f64 else np.float32)
    for b in (range(w.nblocks) if blocks is None else blocks):
        n2i, vals = w.block_nodes(b)
        d = int(w.blocks[b, 3])
        out[int(vo[b]):int(vo[b + 1])] = (interp_f64 if f64 else interp_f32)(n2i, vals, d)
    return out


# ---------------------------------------------------------------- geometry / render

def look_at_camera(eye, center, up, fovy_deg: float, W: int, H: int) -> dict:
    """The perspective camera of a look-at view, restated for the oracle side: the view matrix of the
    OpenGL convention (camera looking along -Z: z = normalize(eye - center), x = normalize(up x z),
    y = z x x, in double), then the eye set-up of DenseFieldRenderer_cu.cu:353-372 (n = -Lcam z with
    Lcam = 0.1, h = 2 Lcam tan(fovY/2), pixel = h / H, w = pixel W) in float.  Keys: eye, e1, e2, n, w, h,
    view_r (rows of the world -> eye rotation), view_t (its translation)."""
    eye = np.asarray(eye, np.float64)
    z = eye - np.asarray(center, np.float64)
    z /= np.sqrt((z * z).sum())
    u = np.asarray(up, np.float64)
    x = np.array([u[1] * z[2] - u[2] * z[1], u[2] * z[0] - u[0] * z[2], u[0] * z[1] - u[1] * z[0]])
    x /= np.sqrt((x * x).sum())
    y = np.array([z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]])
    lcam = np.float32(np.float32(np.float32(0.01) * np.float32(2)) * np.float32(5))
    h = np.float32(2 * np.float64(lcam) * np.tan(0.5 * fovy_deg * np.pi / 180))
    pixel = np.float32(h / np.float32(H))
    rows = np.stack([x, y, z])
    return {"eye": eye.astype(np.float32), "e1": x.astype(np.float32), "e2": y.astype(np.float32),
            "n": (z.astype(np.float32) * -lcam).astype(np.float32), "h": h, "w": np.float32(pixel * np.float32(W)),
            "view_r": rows.astype(np.float32).ravel(),
            "view_t": np.array([-(r[0] * eye[0] + r[1] * eye[1] + r[2] * eye[2]) for r in rows], np.float32)}


def orc_view(cam: dict, W: int, H: int, level: int, field_min, field_max, threshold, quality, tf_n: int,
             filter: int = 0) -> OrcView:
    """OrcView from a look_at_camera() camera and the frame parameters."""
    o = OrcView()
    for f in ("eye", "e1", "e2", "n"):
        getattr(o.cam, f)[:] = [float(v) for v in cam[f]]
    o.cam.w, o.cam.h, o.cam.ortho = float(cam["w"]), float(cam["h"]), 0
    o.W, o.H, o.level = W, H, level
    o.field_min, o.field_max, o.threshold, o.quality, o.tf_n = field_min, field_max, threshold, quality, tf_n
    o.filter = filter
    return o


def block_view_rect(view: OrcView, r9, t3, idx) -> np.ndarray:
    rr = np.ascontiguousarray(r9, dtype=np.float32)
    tt = np.ascontiguousarray(t3, dtype=np.float32)
    i = (C.c_uint32 * 3)(*idx)
    out = (C.c_int32 * 4)()
    port().orc_block_view_rect(C.byref(view), _p(rr, C.c_float), _p(tt, C.c_float), i, out)
    return np.array(out[:], dtype=np.int32)


def render_block_argb8(view: OrcView, brick: np.ndarray, depth: int, idx, rect, tf: np.ndarray,
                       viewport: np.ndarray) -> None:
    brick = np.ascontiguousarray(brick, dtype=np.float32)
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    i = (C.c_uint32 * 3)(*idx)
    r = (C.c_int32 * 4)(*[int(x) for x in rect])
    port().orc_render_block_argb8(C.byref(view), _p(brick, C.c_float), C.c_uint32(depth), i, r,
                                  _p(tf, C.c_float), _p(viewport, C.c_uint32))


def tex3d_weights(tc, n: int):
    """Texture-unit weights (int, units of 1/256), NaN-footprint flags and texel indices
    of the 8 texels around texel coordinate tc = (x, y, z) in an n^3 clamped texture."""
    t = (C.c_float * 3)(*[float(x) for x in tc])
    w = (C.c_int32 * 8)()
    f = (C.c_uint8 * 8)()
    i = (C.c_uint32 * 8)()
    port().orc_tex3d_weights(t, C.c_uint32(n), w, f, i)
    return np.array(w[:]), np.array(f[:], dtype=bool), np.array(i[:])


class OrcLight(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("ambient", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3)]


class OrcPresentation(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("isosurface_opacity", C.c_float), ("level_count", C.c_uint32),
                ("levels", C.c_float * 50), ("light_count", C.c_uint32), ("lights", OrcLight * 10),
                ("secondary_min", C.c_float), ("secondary_max", C.c_float)]


def presentation_from(p) -> OrcPresentation:
    """OrcPresentation from a revise_gb300._lib.Presentation (same fields)."""
    o = OrcPresentation()
    C.memmove(C.byref(o), C.byref(p), C.sizeof(o))
    return o


def render_block_mode(view: OrcView, pres: OrcPresentation, brick: np.ndarray, depth: int, idx, rect,
                      tf: np.ndarray, viewport: np.ndarray, brick2: np.ndarray = None) -> None:
    brick = np.ascontiguousarray(brick, dtype=np.float32)
    b2 = None if brick2 is None else np.ascontiguousarray(brick2, dtype=np.float32)
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    i = (C.c_uint32 * 3)(*idx)
    r = (C.c_int32 * 4)(*[int(x) for x in rect])
    port().orc_render_block_mode(C.byref(view), C.byref(pres), _p(brick, C.c_float),
                                 _p(b2, C.c_float) if b2 is not None else None, C.c_uint32(depth), i, r,
                                 _p(tf, C.c_float), _p(viewport, C.c_uint32))


def _frame_args(w, dense, rects):
    blocks = np.ascontiguousarray(w.blocks, dtype=np.uint32)
    off = np.ascontiguousarray(w.vertex_off[:-1], dtype=np.uint64)
    dense = np.ascontiguousarray(dense, dtype=np.float32)
    rp = None
    if rects is not None:
        rects = np.ascontiguousarray(rects, dtype=np.int32)
        rp = _p(rects, C.c_int32)
    return blocks, off, dense, rects, rp


def render_frame_f64(view: OrcView, w, dense: np.ndarray, rects, tf: np.ndarray, pixels=None, f64: bool = False):
    """FP64 frame render: (np, 4) RGBA (float32, or float64 with f64) and (np,) near-threshold flags."""
    blocks, off, dense, rects, rp = _frame_args(w, dense, rects)
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    if pixels is None:
        npx = view.W * view.H
        pp = None
    else:
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        npx = pixels.shape[0]
        pp = _p(pixels, C.c_uint32)
    out = np.zeros((npx, 4), dtype=np.float64 if f64 else np.float32)
    flags = np.zeros(npx, dtype=np.uint8)
    fn = port().orc_render_frame_f64d if f64 else port().orc_render_frame_f64
    fn(C.byref(view), C.c_uint32(blocks.shape[0]), _p(blocks, C.c_uint32), _p(off, C.c_uint64), _p(dense, C.c_float),
       rp, _p(tf, C.c_float), C.c_uint32(npx), pp, _p(out, C.c_double if f64 else C.c_float), _p(flags, C.c_uint8))
    return out, flags


def render_frame_argb8(view: OrcView, w, dense: np.ndarray, rects, tf: np.ndarray) -> np.ndarray:
    blocks, off, dense, rects, rp = _frame_args(w, dense, rects)
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    vp = np.zeros(view.W * view.H, dtype=np.uint32)
    port().orc_render_frame_argb8(C.byref(view), C.c_uint32(blocks.shape[0]), _p(blocks, C.c_uint32),
                                  _p(off, C.c_uint64), _p(dense, C.c_float), rp, _p(tf, C.c_float),
                                  _p(vp, C.c_uint32))
    return vp


def render_frame_grad_f64(view: OrcView, w, dense, rects, tf, target, pixels=None):
    """Loss and FP64 gradients (dtf (tf_n, 4), ddense (V,)) of 1/2 |I - target|^2."""
    blocks, off, dense, rects, rp = _frame_args(w, dense, rects)
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    target = np.ascontiguousarray(target, dtype=np.float32)
    if pixels is None:
        npx, pp = view.W * view.H, None
    else:
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        npx, pp = pixels.shape[0], _p(pixels, C.c_uint32)
    dtf = np.zeros(tf.shape, dtype=np.float64)
    dd = np.zeros(dense.shape[0], dtype=np.float64)
    loss = port().orc_render_frame_grad_f64(C.byref(view), C.c_uint32(blocks.shape[0]), _p(blocks, C.c_uint32),
                                            _p(off, C.c_uint64), _p(dense, C.c_float), rp, _p(tf, C.c_float),
                                            C.c_uint32(npx), pp, _p(target, C.c_float), _p(dtf, C.c_double),
                                            _p(dd, C.c_double))
    return loss, dtf, dd


# ---------------------------------------------------------------- blend / ctf / order

def blend_image_part(dst, src, origin, just_copy=False, offset=(0, 0), use_ref=False) -> None:
    lib = ref() if use_ref else port()
    fn = lib.ref_blend_image_part if use_ref else lib.orc_blend_image_part
    fn(_p(dst, C.c_uint32), C.c_int32(dst.shape[1]), C.c_int32(dst.shape[0]), _p(src, C.c_uint32),
       C.c_int32(src.shape[1]), C.c_int32(src.shape[0]), C.c_int32(int(origin[0])), C.c_int32(int(origin[1])),
       C.c_int32(1 if just_copy else 0), C.c_int32(int(offset[0])), C.c_int32(int(offset[1])))


def make_ctf(xs, rgba, count: int, use_ref=False) -> np.ndarray:
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    rgba = np.ascontiguousarray(rgba, dtype=np.float64).reshape(-1, 4)
    out = np.zeros((count, 4), dtype=np.float32)
    lib = ref() if use_ref else port()
    fn = lib.ref_make_ctf if use_ref else lib.orc_make_ctf
    fn(_p(xs, C.c_double), _p(rgba, C.c_double), C.c_uint32(xs.shape[0]), C.c_uint32(count), _p(out, C.c_float))
    return out


def ref_b2f_order(bmin, bmax, cmin, cmax, eye) -> np.ndarray:
    a = (C.c_uint32 * 3)(*bmin)
    b = (C.c_uint32 * 3)(*bmax)
    c0 = (C.c_double * 3)(*cmin)
    c1 = (C.c_double * 3)(*cmax)
    e = (C.c_double * 3)(*eye)
    cap = int(np.prod(np.asarray(bmax, dtype=np.int64) - np.asarray(bmin, dtype=np.int64)))
    out = np.zeros((max(cap, 1), 3), dtype=np.uint32)
    n = ref().ref_b2f_order(a, b, c0, c1, e, _p(out, C.c_uint32), C.c_uint32(cap))
    return out[:n]


def read_blocks_per_call(path: str, offsets, counts):
    """The reference worker's per-block field read (open, seek, read, close per block): values
    concatenated in block order and the (nb, 2) stored ranges."""
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    counts = np.ascontiguousarray(counts, dtype=np.uint64)
    out = np.empty(int(counts.sum()), dtype=np.float32)
    ranges = np.empty((counts.size, 2), dtype=np.float32)
    lib = port()
    lib.orc_read_blocks_per_call.restype = C.c_int
    rc = lib.orc_read_blocks_per_call(str(path).encode(), _p(offsets, C.c_uint64), _p(counts, C.c_uint64),
                                      C.c_uint32(counts.size), _p(out, C.c_float), _p(ranges, C.c_float))
    if rc != 0:
        raise IOError(f"per-block read of {path} failed")
    return out, ranges


def ref_split_cube(level: int, count: int, trailing: bool) -> np.ndarray:
    """The reference's IndexCubeSplitter<3>(level, count, [-5,5]^3).all_blocks(trailing): (n, 6) boxes."""
    lib = ref()
    cap = max(count, 1) + 8
    out = np.zeros((cap, 6), dtype=np.uint32)
    n = lib.ref_split_cube(C.c_uint32(level), C.c_uint32(count), C.c_int(int(trailing)), _p(out, C.c_uint32),
                           C.c_uint32(cap))
    return out[:n].copy()


def ref_split_b2f(level: int, count: int, eye) -> np.ndarray:
    """The reference's BackToFrontOrder over that splitter for `eye`: (n, 6) boxes."""
    lib = ref()
    cap = max(count, 1) + 8
    out = np.zeros((cap, 6), dtype=np.uint32)
    e = np.ascontiguousarray(eye, dtype=np.float64)
    n = lib.ref_split_b2f(C.c_uint32(level), C.c_uint32(count), _p(e, C.c_double), _p(out, C.c_uint32),
                          C.c_uint32(cap))
    return out[:n].copy()


def render_frame_mode(view: OrcView, pres: OrcPresentation, w, dense: np.ndarray, rects, tf: np.ndarray,
                      alpha_stop: float, dense2=None) -> np.ndarray:
    """Batched field-mode frame in FP32: (W*H, 4) float RGBA (see orc_render_frame_mode)."""
    blocks, off, dense, rects, rp = _frame_args(w, dense, rects)
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    d2 = None if dense2 is None else np.ascontiguousarray(dense2, dtype=np.float32)
    out = np.zeros((view.W * view.H, 4), dtype=np.float32)
    port().orc_render_frame_mode(C.byref(view), C.byref(pres), C.c_uint32(blocks.shape[0]), _p(blocks, C.c_uint32),
                                 _p(off, C.c_uint64), _p(dense, C.c_float),
                                 _p(d2, C.c_float) if d2 is not None else None, rp, _p(tf, C.c_float),
                                 C.c_float(alpha_stop), _p(out, C.c_float))
    return out
