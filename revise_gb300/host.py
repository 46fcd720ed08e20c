"""Host-only entry points of the s3r C ABI (no GPU needed): camera and view set-up,
block geometry, back-to-front ordering, the transfer-function table and the
host image-part blend."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import Camera, Light, Presentation, View, arr, check


def camera_look_at(eye, center, up, fovy_deg: float, W: int, H: int, ortho: bool = False,
                   ortho_height: float = 0.0) -> Camera:
    lib = _lib.load()
    cam = Camera()
    e = (C.c_double * 3)(*eye)
    c = (C.c_double * 3)(*center)
    u = (C.c_double * 3)(*up)
    check(lib.s3r_camera_look_at(e, c, u, float(fovy_deg), W, H, 1 if ortho else 0, float(ortho_height),
                                 C.byref(cam)))
    return cam


def camera_from_view(view_matrix, fovy_deg: float, W: int, H: int) -> Camera:
    """s3r_camera_from_view: the renderer's camera from a world -> eye transform (4x4, column-major floats,
    the reference's VsRenderSharedState::cameraTransform)."""
    lib = _lib.load()
    m = np.ascontiguousarray(view_matrix, dtype=np.float32).reshape(16)
    cam = Camera()
    check(lib.s3r_camera_from_view(m.ctypes.data_as(C.POINTER(C.c_float)), float(fovy_deg), W, H, C.byref(cam)))
    return cam


def view_matrix_look_at(eye, center, up) -> np.ndarray:
    """The world -> eye transform of s3r_camera_look_at's camera as 16 column-major floats (the rotation rows
    and translation it keeps in view_r / view_t)."""
    cam = camera_look_at(eye, center, up, 60.0, 2, 2)
    m = np.zeros(16, np.float32)
    r = np.array(cam.view_r[:], np.float32).reshape(3, 3)
    for c in range(3):
        m[4 * c:4 * c + 3] = r[:, c]
    m[12:15] = np.array(cam.view_t[:], np.float32)
    m[15] = 1.0
    return m


def relative_to_absolute(field_min: float, field_max: float, rel: float) -> float:
    """The absolute field value of a relative one in float arithmetic, min + (max - min) rel
    (relToAbsFieldValue, DenseFieldRenderer_cu.cu:591-595)."""
    lo, hi, r = np.float32(field_min), np.float32(field_max), np.float32(rel)
    return float(np.float32(lo + np.float32(np.float32(hi - lo) * r)))


def make_view(cam: Camera, W: int, H: int, level: int, field_min: float, field_max: float, threshold: float,
              quality: float, tf_n: int, alpha_stop: float = 2.0, filter: int = _lib.FILTER_EXACT) -> View:
    """filter: _lib.FILTER_EXACT (exact FP32 filtering) or _lib.FILTER_TEXTURE (the texture
    unit's filtering of the reference's textures, giving the reference's images)."""
    v = View()
    v.cam = cam
    v.W, v.H, v.level = W, H, level
    v.field_min, v.field_max = field_min, field_max
    v.threshold, v.quality = threshold, quality
    v.tf_n = tf_n
    v.alpha_stop = alpha_stop
    v.filter = filter
    return v


def view_for(w, alpha_stop: float = 2.0, filter: int = _lib.FILTER_EXACT, eye=None) -> View:
    """The view of a revise_gb300.workloads.Workload (eye: another camera position, same target)."""
    cam = camera_look_at(w.eye if eye is None else eye, w.center, w.up, w.fovy, w.W, w.H, w.ortho, w.ortho_height)
    return make_view(cam, w.W, w.H, w.level, w.field_min, w.field_max, w.threshold, w.quality, w.tf.shape[0],
                     alpha_stop, filter)


def block_cube(level: int, idx):
    lib = _lib.load()
    i = (C.c_uint32 * 3)(*idx)
    c = (C.c_float * 3)()
    h = C.c_float()
    check(lib.s3r_block_cube(level, i, c, C.byref(h)))
    return np.array(c[:], dtype=np.float32), np.float32(h.value)


def block_view_rect(view: View, idx) -> np.ndarray:
    lib = _lib.load()
    i = (C.c_uint32 * 3)(*idx)
    r = (C.c_int32 * 4)()
    check(lib.s3r_block_view_rect(C.byref(view), i, r))
    return np.array(r[:], dtype=np.int32)


def b2f_order(bmin, bmax, cmin, cmax, eye) -> np.ndarray:
    """BackToFrontOrder<MacroBlock<3>>::range(eye) over index box [bmin, bmax): (n, 3) uint32."""
    lib = _lib.load()
    a = (C.c_uint32 * 3)(*bmin)
    b = (C.c_uint32 * 3)(*bmax)
    c0 = (C.c_double * 3)(*cmin)
    c1 = (C.c_double * 3)(*cmax)
    e = (C.c_double * 3)(*eye)
    cap = int(np.prod(np.asarray(bmax, dtype=np.int64) - np.asarray(bmin, dtype=np.int64)))
    out = np.zeros((max(cap, 1), 3), dtype=np.uint32)
    cnt = C.c_uint32()
    check(lib.s3r_b2f_order(a, b, c0, c1, e, arr(out, C.c_uint32), cap, C.byref(cnt)))
    return out[: cnt.value]


def index_box_world(level: int, bmin, bmax):
    lib = _lib.load()
    a = (C.c_uint32 * 3)(*bmin)
    b = (C.c_uint32 * 3)(*bmax)
    c0 = (C.c_double * 3)()
    c1 = (C.c_double * 3)()
    check(lib.s3r_index_box_world(level, a, b, c0, c1))
    return np.array(c0[:]), np.array(c1[:])


def make_color_transfer(xs, rgba, color_count: int) -> np.ndarray:
    lib = _lib.load()
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    rgba = np.ascontiguousarray(rgba, dtype=np.float64).reshape(-1, 4)
    out = np.zeros((color_count, 4), dtype=np.float32)
    check(lib.s3r_make_color_transfer(arr(xs, C.c_double), arr(rgba, C.c_double), xs.shape[0], color_count,
                                      arr(out, C.c_float)))
    return out


def blend_image_part(dst: np.ndarray, src: np.ndarray, origin, just_copy: bool = False, offset=(0, 0)) -> None:
    """blendImagePart on host ARGB32 images (uint32 arrays of shape (h, w)), in place on dst."""
    lib = _lib.load()
    assert dst.dtype == np.uint32 and src.dtype == np.uint32 and dst.flags.c_contiguous and src.flags.c_contiguous
    check(lib.s3r_blend_image_part_host(arr(dst, C.c_uint32), dst.shape[1], dst.shape[0], arr(src, C.c_uint32),
                                        src.shape[1], src.shape[0], int(origin[0]), int(origin[1]),
                                        1 if just_copy else 0, int(offset[0]), int(offset[1])))


def default_light(view: View) -> Light:
    """The reference renderer's single light source for this view."""
    lib = _lib.load()
    out = Light()
    check(lib.s3r_default_light(C.byref(view), C.byref(out)))
    return out


def presentation(mode: int, view: View = None, isosurface_opacity: float = 1.0, levels=(), lights=None,
                 secondary_range=(0.0, 1.0)) -> Presentation:
    """s3r_presentation for a field mode.  levels: absolute isosurface values (sorted and
    de-duplicated here, as the reference's makeLevels does); lights default to the
    renderer's single light for view."""
    p = Presentation()
    p.mode = mode
    p.isosurface_opacity = isosurface_opacity
    lv = sorted(set(float(np.float32(x)) for x in levels))[:_lib.MAX_LEVELS]
    p.level_count = len(lv)
    for i, x in enumerate(lv):
        p.levels[i] = x
    if lights is None:
        lights = [default_light(view)] if view is not None else []
    p.light_count = len(lights)
    for i, L in enumerate(lights):
        p.lights[i] = L
    p.secondary_min, p.secondary_max = secondary_range
    return p


def blend_image_part_mip(dst: np.ndarray, src: np.ndarray, origin, just_copy: bool = False, offset=(0, 0)) -> None:
    """blendImagePartMaxIntensity on host float images (float32 arrays of shape (h, w)), in place on dst."""
    lib = _lib.load()
    assert dst.dtype == np.float32 and src.dtype == np.float32 and dst.flags.c_contiguous and src.flags.c_contiguous
    check(lib.s3r_blend_image_part_mip_host(arr(dst, C.c_float), dst.shape[1], dst.shape[0], arr(src, C.c_float),
                                            src.shape[1], src.shape[0], int(origin[0]), int(origin[1]),
                                            1 if just_copy else 0, int(offset[0]), int(offset[1])))
