"""ctypes binding of the s3r C ABI (include/s3r.h).

The shared library is built in-tree by revise_gb300.build; loading fails loudly
when it is missing -- there is no CPU fallback for any entry point here.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libs3r.so"

S3R_OK = 0
S3R_ERR_INVALID = 1
S3R_ERR_CUDA = 2
S3R_ERR_NOMEM = 3
S3R_ERR_CANCELLED = 4
S3R_ERR_UNSUPPORTED = 5
NO_FIELD_VALUE = 1e30
MAX_DEPTH = 9

BRICK_F32, BRICK_F16, BRICK_BF16 = 0, 1, 2
FILTER_EXACT, FILTER_TEXTURE = 0, 1
RENDER_TILES_WALK, RENDER_TILES = 16, 19  # render forms: per-ray walk ids, then block-major ids
ABI_VERSION = 7

u8p = C.POINTER(C.c_uint8)
u16p = C.POINTER(C.c_uint16)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
vp = C.c_void_p


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("e1", C.c_float * 3), ("e2", C.c_float * 3), ("n", C.c_float * 3),
                ("w", C.c_float), ("h", C.c_float), ("ortho", C.c_int32), ("reserved", C.c_int32),
                ("view_r", C.c_float * 9), ("view_t", C.c_float * 3)]


class View(C.Structure):
    _fields_ = [("cam", Camera), ("W", C.c_uint32), ("H", C.c_uint32), ("level", C.c_uint32),
                ("field_min", C.c_float), ("field_max", C.c_float), ("threshold", C.c_float),
                ("quality", C.c_float), ("tf_n", C.c_uint32), ("alpha_stop", C.c_float),
                ("filter", C.c_uint32), ("reserved", C.c_uint32 * 2)]


MODE_ISOSURFACE, MODE_ISOSURFACES, MODE_MAX_INTENSITY, MODE_ARGB = 0, 1, 2, 3
MODE_ARGB_LIGHT, MODE_DOMAIN_VOXELS, MODE_VALUE_ON_ISOSURFACE, MODE_VALUE_ON_ISOSURFACES = 4, 5, 6, 7
MAX_LEVELS, MAX_LIGHTS = 50, 10


class Light(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("ambient", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3)]


class Presentation(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("isosurface_opacity", C.c_float), ("level_count", C.c_uint32),
                ("levels", C.c_float * MAX_LEVELS), ("light_count", C.c_uint32), ("lights", Light * MAX_LIGHTS),
                ("secondary_min", C.c_float), ("secondary_max", C.c_float)]


class FrameDesc(C.Structure):
    _fields_ = [("level", C.c_uint32), ("nblocks", C.c_uint32), ("blocks", u32p), ("node_off", u64p),
                ("n2i", u16p), ("brick_format", C.c_uint32), ("tile_cells", C.c_uint32),
                ("render_tile", C.c_uint32), ("reserved", C.c_uint32)]


class PlanInfo(C.Structure):
    _fields_ = [("nodes", C.c_uint64), ("vertices", C.c_uint64), ("brick_bytes", C.c_uint64),
                ("tiles", C.c_uint64), ("tile_entries", C.c_uint64), ("tile_cells", C.c_uint32),
                ("render_tile", C.c_uint32), ("brick_format", C.c_uint32), ("nblocks", C.c_uint32)]


class ImagePart(C.Structure):
    _fields_ = [("pixels", vp), ("origin", C.c_int32 * 2), ("size", C.c_int32 * 2)]


class WorkerBlocks(C.Structure):
    _fields_ = [("nblocks", C.c_uint32), ("blocks", u32p), ("node_off", u64p), ("n2i", vp), ("sparse", vp),
                ("sparse2", vp)]


class DatasetInfo(C.Structure):
    _fields_ = [("format_version", C.c_uint32), ("time_steps", C.c_uint32), ("field_count", C.c_uint32),
                ("max_subtree_depth", C.c_uint32), ("max_full_level", C.c_uint32), ("level_count", C.c_uint32),
                ("subtree_count", C.c_uint32), ("has_time_steps", C.c_uint32), ("tree_blocks", C.c_uint64),
                ("field_file_size", C.c_uint64), ("bc_min", C.c_float * 3), ("bc_size", C.c_float)]


class SubtreeInfo(C.Structure):
    _fields_ = [("level", C.c_uint32), ("x", C.c_uint32), ("y", C.c_uint32), ("z", C.c_uint32),
                ("depth", C.c_uint32), ("tree_index", C.c_uint32), ("values_offset", C.c_uint64),
                ("node_count", C.c_uint64)]


# name -> (restype, argtypes)
_SIGS = {
    "s3r_abi_version": (C.c_int, []),
    "s3r_ctx_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
    "s3r_ctx_destroy": (C.c_int, [vp]),
    "s3r_last_error": (C.c_char_p, [vp]),
    "s3r_ctx_launch_count": (C.c_uint64, [vp]),
    "s3r_interp_dense": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, vp, vp]),
    "s3r_interp_dense_noalloc": (C.c_int, [vp, vp, C.c_uint32, C.c_uint32, vp, vp]),
    "s3r_camera_look_at": (C.c_int, [f64p, f64p, f64p, C.c_double, C.c_uint32, C.c_uint32, C.c_int32,
                                     C.c_double, C.POINTER(Camera)]),
    "s3r_block_cube": (C.c_int, [C.c_uint32, u32p, f32p, f32p]),
    "s3r_block_view_rect": (C.c_int, [C.POINTER(View), u32p, i32p]),
    "s3r_clear_viewport": (C.c_int, [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, vp]),
    "s3r_render_block_argb": (C.c_int, [vp, C.POINTER(View), vp, C.c_uint32, u32p, i32p, vp, vp, vp]),
    "s3r_camera_from_view": (C.c_int, [C.POINTER(C.c_float), C.c_float, C.c_uint32, C.c_uint32, C.POINTER(Camera)]),
    "s3r_texture_create": (C.c_int, [vp, C.c_uint32, C.POINTER(vp)]),
    "s3r_texture_destroy": (C.c_int, [vp]),
    "s3r_texture_fill": (C.c_int, [vp, vp, vp, vp]),
    "s3r_interp_dense_texture": (C.c_int, [vp, vp, vp, C.c_uint32, vp, vp]),
    "s3r_tf_texture_create": (C.c_int, [vp, C.c_uint32, C.POINTER(vp)]),
    "s3r_tf_texture_set": (C.c_int, [vp, vp, vp, vp]),
    "s3r_tf_texture_destroy": (C.c_int, [vp]),
    "s3r_render_block_texture": (C.c_int, [vp, C.POINTER(View), C.POINTER(Presentation), vp, vp, u32p, i32p, vp, vp,
                                           vp]),
    "s3r_render_block": (C.c_int, [vp, C.POINTER(View), C.POINTER(Presentation), vp, vp, C.c_uint32, u32p, i32p, vp,
                                   vp, vp]),
    "s3r_default_light": (C.c_int, [C.POINTER(View), C.POINTER(Light)]),
    "s3r_blend_image_part_mip_host": (C.c_int, [f32p, C.c_int32, C.c_int32, f32p, C.c_int32, C.c_int32, C.c_int32,
                                                C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "s3r_b2f_order": (C.c_int, [u32p, u32p, f64p, f64p, f64p, u32p, C.c_uint32, u32p]),
    "s3r_split_index_cube": (C.c_int, [C.c_uint32, C.c_uint32, C.c_int32, u32p, C.c_uint32, u32p]),
    "s3r_split_b2f": (C.c_int, [C.c_uint32, C.c_uint32, f64p, u32p, C.c_uint32, u32p]),
    "s3r_index_box_world": (C.c_int, [C.c_uint32, u32p, u32p, f64p, f64p]),
    "s3r_bound_rect": (C.c_int, [vp, vp, C.c_uint32, C.c_uint32, i32p, vp]),
    "s3r_crop": (C.c_int, [vp, vp, C.c_uint32, i32p, vp, vp]),
    "s3r_blend_image_part_host": (C.c_int, [u32p, C.c_int32, C.c_int32, u32p, C.c_int32, C.c_int32, C.c_int32,
                                            C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "s3r_compose_parts": (C.c_int, [vp, C.POINTER(ImagePart), C.c_uint32, C.c_int32, vp, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_int32, vp]),
    "s3r_render_scene_part": (C.c_int, [vp, C.POINTER(View), C.POINTER(Presentation), C.POINTER(WorkerBlocks), u32p,
                                        u32p, vp, vp, i32p, vp]),
    "s3r_render_scene_part_bricks": (C.c_int, [vp, vp, C.POINTER(View), C.POINTER(Presentation), vp, u32p, u32p,
                                               vp, vp, i32p, vp]),
    "s3r_make_color_transfer": (C.c_int, [f64p, f64p, C.c_uint32, C.c_uint32, f32p]),
    "s3r_frame_plan": (C.c_int, [vp, C.POINTER(FrameDesc), C.POINTER(vp)]),
    "s3r_plan_destroy": (C.c_int, [vp]),
    "s3r_plan_info_get": (C.c_int, [vp, C.POINTER(PlanInfo)]),
    "s3r_plan_bricks": (C.c_int, [vp, C.POINTER(vp), C.POINTER(u64p)]),
    "s3r_plan_tile_cells": (C.c_int, [vp, C.c_uint32, u32p]),
    "s3r_plan_brick_pitches": (C.c_int, [vp, C.POINTER(u32p)]),
    "s3r_frame_run_host": (C.c_int, [vp, vp, C.POINTER(View), vp, vp, vp, vp]),
    "s3r_frame_host_sync": (C.c_int, [vp, vp]),
    "s3r_plan_brick_scales": (C.c_int, [vp, C.POINTER(vp)]),
    "s3r_plan_autotune": (C.c_int, [vp, vp, C.POINTER(View), vp, vp, C.c_uint32, vp]),
    "s3r_frame_interp": (C.c_int, [vp, vp, vp, vp]),
    "s3r_frame_render": (C.c_int, [vp, vp, C.POINTER(View), vp, vp, vp, vp, vp]),
    "s3r_frame_render_mode": (C.c_int, [vp, vp, C.POINTER(View), C.POINTER(Presentation), vp, vp, vp, vp, vp]),
    "s3r_frame_run": (C.c_int, [vp, vp, C.POINTER(View), vp, vp, vp, vp, vp, vp]),
    "s3r_render_argb_backward": (C.c_int, [vp, vp, C.POINTER(View), vp, vp, vp, vp, vp, vp]),
    "s3r_dataset_open": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "s3r_dataset_close": (C.c_int, [vp]),
    "s3r_dataset_info_get": (C.c_int, [vp, C.POINTER(DatasetInfo)]),
    "s3r_dataset_field": (C.c_int, [vp, C.c_uint32, C.c_char_p, C.c_size_t, f32p, i32p]),
    "s3r_dataset_field_index": (C.c_int, [vp, C.c_char_p, u32p]),
    "s3r_dataset_tree_blocks": (C.c_int, [vp, C.c_uint32, u32p, C.c_uint64, u64p]),
    "s3r_dataset_subtrees": (C.c_int, [vp, C.c_uint32, C.POINTER(SubtreeInfo), C.c_uint32, u32p]),
    "s3r_dataset_subtree": (C.c_int, [vp, C.c_uint32, u32p, C.POINTER(SubtreeInfo)]),
    "s3r_dataset_subtree_nodes": (C.c_int, [vp, C.c_uint32, u32p, vp, C.c_uint64, u64p]),
    "s3r_dataset_subtree_values": (C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_uint32, u32p, f32p, vp, C.c_uint64,
                                             u64p]),
    "s3r_dataset_frame_topology": (C.c_int, [vp, C.c_uint32, u32p, C.c_uint32, u32p, u64p, vp, C.c_uint64,
                                             C.c_uint32]),
    "s3r_dataset_frame_values": (C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_uint32, u32p, C.c_uint32, u64p, vp,
                                           vp, C.c_uint32]),
    "s3r_dataset_propagate": (C.c_int, [vp, vp, C.c_uint32, vp, vp, vp, u8p, vp]),
    "s3r_field_divide": (C.c_int, [vp, vp, vp, C.c_uint64, vp, vp]),
    "s3r_dataset_frame_upload": (C.c_int, [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, u32p, C.c_uint32, u64p,
                                           vp, vp, C.c_uint32, vp]),
}

EXPORTED = sorted(_SIGS)


class S3RError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"s3r error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libs3r.so (RTLD_GLOBAL not needed); raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m revise_gb300.build` "
                           "(the CUDA extension is required; there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int, ctx=None) -> None:
    if rc != S3R_OK:
        lib = load()
        msg = lib.s3r_last_error(ctx)
        raise S3RError(rc, msg.decode() if msg else "")


def ptr(x) -> C.c_void_p:
    """Device or host address of a torch tensor / numpy array / int as a void*."""
    if x is None:
        return C.c_void_p(0)
    if isinstance(x, int):
        return C.c_void_p(x)
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    if hasattr(x, "ctypes"):
        return C.c_void_p(x.ctypes.data)
    raise TypeError(type(x))


def arr(x, ctype):
    """numpy array -> ctypes pointer of ctype."""
    return x.ctypes.data_as(C.POINTER(ctype))
