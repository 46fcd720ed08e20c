"""GPU-side Python API over the s3r C ABI, with torch providing device memory
and streams (plumbing only: every computation runs in the s3r CUDA kernels).

Mirrors the reference's interfaces for this path:
  Context.interp_dense          DenseFieldInterpolatorTpl_cu_3::interpolate(dst, sparse, nodes)
                                (include/s3dmm_cuda/DenseFieldInterpolatorTpl_cu_3.hpp:103-107)
  DenseFieldRenderer            DenseFieldRenderer_cu (include/s3dmm_cuda/DenseFieldRenderer_cu.hpp:32-54)
  VsWorker                      VsWorker_cu / VsWorkerInterface::renderScenePart
                                (src/s3vs_worker/cuda/VsWorker_cu.cpp:225-313)
  FramePlan                     the batched frame (no reference counterpart)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib, host
from ._lib import FrameDesc, ImagePart, PlanInfo, View, WorkerBlocks, arr, check, ptr


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("revise_gb300 needs a CUDA device (no CPU fallback)")
    return torch


def _stream(stream):
    torch = _torch()
    if stream is None:
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class _CudaArray:
    """Zero-copy view of s3r-owned device memory for torch.as_tensor."""

    def __init__(self, addr: int, shape, typestr: str, owner):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(addr), False),
                                         "version": 2, "strides": None}
        self._owner = owner


def device_array(addr: int, shape, dtype: str, owner=None):
    torch = _torch()
    typestr = {"f4": "<f4", "f2": "<f2", "u2": "<u2", "u4": "<u4"}[dtype]
    return torch.as_tensor(_CudaArray(addr, shape, typestr, owner), device="cuda")


def to_device_n2i(n2i: np.ndarray):
    """(n, 3) uint16 node indices -> device int16 tensor holding the same bits."""
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(n2i, dtype=np.uint16).view(np.int16)).cuda()


class Context:
    """One s3r context (one per host thread, bound to one device)."""

    def __init__(self, device: int = 0):
        _torch()
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.s3r_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            self.lib.s3r_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        check(rc, self.h)

    @property
    def launches(self) -> int:
        return int(self.lib.s3r_ctx_launch_count(self.h))

    # -- dense interpolation ------------------------------------------------
    def interp_dense(self, n2i_dev, sparse_dev, depth: int, out=None, stream=None):
        torch = _torch()
        e = (1 << depth) + 1
        if out is None:
            out = torch.empty(e ** 3, dtype=torch.float32, device="cuda")
        n = int(sparse_dev.numel())
        self._check(self.lib.s3r_interp_dense(self.h, ptr(n2i_dev), ptr(sparse_dev), n, depth, ptr(out),
                                              _stream(stream)))
        return out

    # -- plain render ------------------------------------------------------
    def clear_viewport(self, viewport, W: int, H: int, value: int = 0, stream=None):
        self._check(self.lib.s3r_clear_viewport(self.h, ptr(viewport), W, H, value, _stream(stream)))

    def render_block_argb(self, view: View, brick, depth: int, idx, rect, tf_dev, viewport, stream=None):
        i = (C.c_uint32 * 3)(*[int(x) for x in idx])
        r = (C.c_int32 * 4)(*[int(x) for x in rect])
        self._check(self.lib.s3r_render_block_argb(self.h, C.byref(view), ptr(brick), depth, i, r, ptr(tf_dev),
                                                   ptr(viewport), _stream(stream)))

    def render_block(self, view: View, pres, brick, depth: int, idx, rect, tf_dev, viewport, brick2=None,
                     stream=None):
        """One block in any field mode (pres: revise_gb300.host.presentation)."""
        i = (C.c_uint32 * 3)(*[int(x) for x in idx])
        r = (C.c_int32 * 4)(*[int(x) for x in rect])
        self._check(self.lib.s3r_render_block(self.h, C.byref(view), C.byref(pres), ptr(brick), ptr(brick2), depth,
                                              i, r, ptr(tf_dev), ptr(viewport), _stream(stream)))

    # -- texture-unit render ----------------------------------------------
    def texture(self, depth: int) -> "FieldTexture":
        return FieldTexture(self, depth)

    def tf_texture(self, tf_dev, stream=None) -> "TfTexture":
        t = TfTexture(self, int(tf_dev.numel()) // 4)
        t.set(tf_dev, stream)
        return t

    def interp_dense_texture(self, n2i_dev, sparse_dev, tex: "FieldTexture", stream=None):
        self._check(self.lib.s3r_interp_dense_texture(self.h, ptr(n2i_dev), ptr(sparse_dev), int(sparse_dev.numel()),
                                                      tex.h, _stream(stream)))

    def render_block_texture(self, view: View, pres, tex: "FieldTexture", idx, rect, tf: "TfTexture", viewport,
                             tex2: "FieldTexture" = None, stream=None):
        """One block in any field mode (pres None: Argb) sampled through the texture unit."""
        i = (C.c_uint32 * 3)(*[int(x) for x in idx])
        r = (C.c_int32 * 4)(*[int(x) for x in rect])
        self._check(self.lib.s3r_render_block_texture(self.h, C.byref(view), C.byref(pres) if pres is not None else None,
                                                      tex.h, tex2.h if tex2 is not None else None, i, r, tf.h,
                                                      ptr(viewport), _stream(stream)))

    def bound_rect(self, viewport, W: int, H: int, stream=None):
        r = (C.c_int32 * 4)()
        self._check(self.lib.s3r_bound_rect(self.h, ptr(viewport), W, H, r, _stream(stream)))
        return tuple(r[:])

    def crop(self, image, W: int, rect, dst, stream=None):
        r = (C.c_int32 * 4)(*rect)
        self._check(self.lib.s3r_crop(self.h, ptr(image), W, r, ptr(dst), _stream(stream)))

    def compose_parts(self, parts, dst, dw: int, dh: int, offset=(0, 0), just_copy_first: bool = False,
                      stream=None):
        """parts: list of (device uint32 tensor, (ox, oy), (w, h)) blended in order into dst."""
        arrp = (ImagePart * max(1, len(parts)))()
        for i, (px, origin, size) in enumerate(parts):
            arrp[i].pixels = ptr(px).value
            arrp[i].origin[0], arrp[i].origin[1] = int(origin[0]), int(origin[1])
            arrp[i].size[0], arrp[i].size[1] = int(size[0]), int(size[1])
        self._check(self.lib.s3r_compose_parts(self.h, arrp, len(parts), 1 if just_copy_first else 0, ptr(dst), dw,
                                               dh, int(offset[0]), int(offset[1]), _stream(stream)))


@dataclass
class ImagePartResult:
    """s3vs::RgbaImagePart (include/s3vs/types.hpp:47-57): ARGB32 pixels at an origin."""
    origin: tuple
    size: tuple
    pixels: np.ndarray  # (h, w) uint32


class FramePlan:
    """A batched block set resident on the GPU: binned nodes, brick store, render table."""

    def __init__(self, ctx: Context, w, brick_format: int = _lib.BRICK_F32, tile_cells: int = 16,
                 render_tile: int = 0):
        self.ctx = ctx
        self.lib = ctx.lib
        self.blocks = np.ascontiguousarray(w.blocks, dtype=np.uint32)
        self.node_off = np.ascontiguousarray(w.node_off, dtype=np.uint64)
        self.n2i = np.ascontiguousarray(w.n2i, dtype=np.uint16)
        d = FrameDesc()
        d.level = w.level
        d.nblocks = self.blocks.shape[0]
        d.blocks = arr(self.blocks, C.c_uint32)
        d.node_off = arr(self.node_off, C.c_uint64)
        d.n2i = arr(self.n2i, C.c_uint16)
        d.brick_format = brick_format
        d.tile_cells = tile_cells
        d.render_tile = render_tile
        h = C.c_void_p()
        ctx._check(self.lib.s3r_frame_plan(ctx.h, C.byref(d), C.byref(h)))
        self.h = h
        self.fmt = brick_format
        self.level = w.level
        self._host_inflight = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.s3r_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def info(self) -> PlanInfo:
        i = PlanInfo()
        check(self.lib.s3r_plan_info_get(self.h, C.byref(i)))
        return i

    def bricks(self):
        """Zero-copy device tensor of the brick store and the per-block vertex offsets."""
        p = C.c_void_p()
        off = _lib.u64p()
        check(self.lib.s3r_plan_bricks(self.h, C.byref(p), C.byref(off)))
        nb = self.blocks.shape[0]
        offs = np.ctypeslib.as_array(off, shape=(nb + 1,)).copy()
        dt = "f4" if self.fmt == _lib.BRICK_F32 else ("f2" if self.fmt == _lib.BRICK_F16 else "u2")
        return device_array(p.value, (int(offs[-1]),), dt, self), offs

    def pitches(self) -> np.ndarray:
        """Per block: the brick row pitch in elements (rows padded to whole 32-byte sectors)."""
        p = _lib.u32p()
        check(self.lib.s3r_plan_brick_pitches(self.h, C.byref(p)))
        return np.ctypeslib.as_array(p, shape=(self.blocks.shape[0],)).copy()

    def block_dense(self, b: int, store=None):
        """Block b's (2^d+1)^3 vertices (x fastest) from the brick store, or from a tensor in the store's
        layout such as the adjoint's dL/ddense."""
        if store is None:
            store, offs = self.bricks()
        else:
            offs = self.bricks()[1]
        e = (1 << int(self.blocks[b, 3])) + 1
        pitch = int(self.pitches()[b])
        a = int(offs[b])
        return store[a:a + e * e * pitch].view(e, e, pitch)[:, :, :e].reshape(-1)

    def dense(self, store=None):
        """The brick store (or a tensor in its layout) without the row padding: every block's (2^d+1)^3
        vertices, blocks in order -- the concatenation the single-block interpolator produces."""
        torch = _torch()
        if store is None:
            store, offs = self.bricks()
        else:
            offs = self.bricks()[1]
        pit = self.pitches()
        parts = []
        for b in range(self.blocks.shape[0]):
            e = (1 << int(self.blocks[b, 3])) + 1
            a = int(offs[b])
            parts.append(store[a:a + e * e * int(pit[b])].view(e, e, int(pit[b]))[:, :, :e].reshape(-1))
        return torch.cat(parts)

    def brick_scales(self):
        p = C.c_void_p()
        check(self.lib.s3r_plan_brick_scales(self.h, C.byref(p)))
        if not p.value:
            return None
        return device_array(p.value, (self.blocks.shape[0], 2), "f4", self)

    def interp(self, sparse_dev, stream=None):
        self.ctx._check(self.lib.s3r_frame_interp(self.ctx.h, self.h, ptr(sparse_dev), _stream(stream)))

    def render(self, view: View, tf_dev, rgba=None, argb=None, samples=None, stream=None):
        self.ctx._check(self.lib.s3r_frame_render(self.ctx.h, self.h, C.byref(view), ptr(tf_dev), ptr(rgba),
                                                  ptr(argb), ptr(samples), _stream(stream)))

    def render_mode(self, view: View, pres, tf_dev, bricks2=None, rgba=None, argb=None, stream=None):
        """The batched frame in any field mode; bricks2: the secondary field's brick store (another plan's
        bricks() over the same blocks) for the value-on-isosurface modes."""
        self.ctx._check(self.lib.s3r_frame_render_mode(self.ctx.h, self.h, C.byref(view), C.byref(pres), ptr(tf_dev),
                                                        ptr(bricks2), ptr(rgba), ptr(argb), _stream(stream)))

    def run(self, view: View, sparse_dev, tf_dev, rgba=None, argb=None, samples=None, stream=None):
        self.ctx._check(self.lib.s3r_frame_run(self.ctx.h, self.h, C.byref(view), ptr(sparse_dev), ptr(tf_dev),
                                               ptr(rgba), ptr(argb), ptr(samples), _stream(stream)))

    def run_host(self, view: View, sparse_host, tf_dev, argb_host, stream=None):
        """One frame from host buffers (pinned torch tensors: the sparse values, the W*H int32 ARGB image),
        pipelined with the frames before and after it (s3r_frame_run_host).  On return sparse_host may be
        refilled and the previous call's image is complete; this call's after the next call or host_sync()."""
        torch = _torch()
        for t in (sparse_host, argb_host):
            if t.is_cuda or not t.is_pinned() or not t.is_contiguous():
                raise ValueError("run_host takes contiguous pinned host tensors")
        # the library copies one float per node in and W*H pixels out through plain pointers
        if sparse_host.dtype != torch.float32 or sparse_host.numel() != int(self.info.nodes):
            raise ValueError(f"sparse_host must hold {int(self.info.nodes)} float32 values")
        if argb_host.dtype not in (torch.int32, torch.uint32) or argb_host.numel() != int(view.W) * int(view.H):
            raise ValueError(f"argb_host must hold {int(view.W) * int(view.H)} 32-bit pixels")
        self.ctx._check(self.lib.s3r_frame_run_host(self.ctx.h, self.h, C.byref(view), ptr(sparse_host), ptr(tf_dev),
                                                    ptr(argb_host), _stream(stream)))
        # the image copy into argb_host completes after the next call, and tf_dev is read by a copy queued on
        # the stream: keep both (and the call before's) alive until they are no longer used, so that neither
        # allocator hands their memory out in between
        self._host_inflight = (self._host_inflight + [(argb_host, tf_dev)])[-2:]

    def host_sync(self):
        self.ctx._check(self.lib.s3r_frame_host_sync(self.ctx.h, self.h))
        self._host_inflight = []

    def tile_cells(self, depth: int) -> int:
        """Interpolation tile edge (cells) of this plan's blocks of the given depth."""
        c = C.c_uint32()
        check(self.lib.s3r_plan_tile_cells(self.h, depth, C.byref(c)))
        return int(c.value)

    def autotune(self, view: View, sparse_dev, tf_dev, reps: int = 3, stream=None):
        self.ctx._check(self.lib.s3r_plan_autotune(self.ctx.h, self.h, C.byref(view), ptr(sparse_dev), ptr(tf_dev),
                                                   reps, _stream(stream)))

    def backward(self, view: View, tf_dev, rgba, dl_drgba, dtf, ddense, stream=None):
        self.ctx._check(self.lib.s3r_render_argb_backward(self.ctx.h, self.h, C.byref(view), ptr(tf_dev),
                                                          ptr(rgba), ptr(dl_drgba), ptr(dtf), ptr(ddense),
                                                          _stream(stream)))


class FieldTexture:
    """A block's dense field as a 3-D texture (s3r_texture): fill it from a dense grid or interpolate into it."""

    def __init__(self, ctx: Context, depth: int):
        self.ctx = ctx
        self.depth = depth
        h = C.c_void_p()
        ctx._check(ctx.lib.s3r_texture_create(ctx.h, depth, C.byref(h)))
        self.h = h

    def fill(self, dense_dev, stream=None):
        self.ctx._check(self.ctx.lib.s3r_texture_fill(self.ctx.h, self.h, ptr(dense_dev), _stream(stream)))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.s3r_texture_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TfTexture:
    """A transfer function as a one-row RGBA texture (s3r_tf_texture)."""

    def __init__(self, ctx: Context, tf_n: int):
        self.ctx = ctx
        self.n = tf_n
        h = C.c_void_p()
        ctx._check(ctx.lib.s3r_tf_texture_create(ctx.h, tf_n, C.byref(h)))
        self.h = h

    def set(self, tf_dev, stream=None):
        self.ctx._check(self.ctx.lib.s3r_tf_texture_set(self.ctx.h, self.h, ptr(tf_dev), _stream(stream)))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.s3r_tf_texture_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DenseFieldRenderer:
    """DenseFieldRenderer_cu for the Argb mode: interpolates one block's dense
    field (DeviceField::makeField, DenseFieldRenderer_cu.cu:504-545) and ray-casts
    it into a device ARGB32 viewport (renderDenseField, :279-486).  With the texture
    filter (the reference's sampling) the field goes into a texture per depth and the
    transfer function into a colour texture, as the reference keeps them."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.state = None
        self._dense = None
        self._tf = None
        self._tex = {}
        self._tf_tex = None

    def set_render_shared_state(self, state: "RenderSharedState"):
        self.state = state
        self._tf = None
        self._tf_tex = None

    def clear_viewport(self, viewport):
        s = self.state
        self.ctx.clear_viewport(viewport, s.view.W, s.view.H, 0)

    def render_dense_field(self, viewport, level: int, index, cancelled=lambda: False):
        torch = _torch()
        s = self.state
        b = s.block_index[(int(index[0]), int(index[1]), int(index[2]))]
        depth = int(s.blocks[b, 3])
        n2i_dev, sparse_dev = s.device_nodes(b)
        if self._tf is None:
            self._tf = torch.from_numpy(np.ascontiguousarray(s.tf, dtype=np.float32)).cuda()
        tex = s.view.filter == _lib.FILTER_TEXTURE
        if tex:
            if depth not in self._tex:
                self._tex[depth] = self.ctx.texture(depth)
            self.ctx.interp_dense_texture(n2i_dev, sparse_dev, self._tex[depth])
            if self._tf_tex is None:
                self._tf_tex = self.ctx.tf_texture(self._tf)
        else:
            self._dense = self.ctx.interp_dense(n2i_dev, sparse_dev, depth, out=None)
        if cancelled():
            return
        rect = host.block_view_rect(s.view, index)
        if rect[2] == 0 or rect[3] == 0:
            return
        if tex:
            self.ctx.render_block_texture(s.view, None, self._tex[depth], index, rect, self._tf_tex, viewport)
        else:
            self.ctx.render_block_argb(s.view, self._dense, depth, index, rect, self._tf, viewport)


class RenderSharedState:
    """The parts of s3vs::VsRenderSharedState (include/s3vs/VsRenderSharedState.hpp:29-46)
    the Argb path reads: field service (block nodes and values), camera/view and
    transfer function.  Samples are filtered as the reference's textures are
    (S3R_FILTER_TEXTURE) unless filter says otherwise."""

    def __init__(self, workload, alpha_stop: float = 2.0, filter: int = _lib.FILTER_TEXTURE):
        self.w = workload
        self.view = host.view_for(workload, alpha_stop, filter)
        self.tf = workload.tf
        self.blocks = workload.blocks
        self.block_index = {(int(b[0]), int(b[1]), int(b[2])): i for i, b in enumerate(workload.blocks)}
        self._dev = {}

    def device_all(self):
        """All blocks' nodes and values as single device arrays (n2i as int16 bits, values float32),
        with the host block table and node offsets: the s3r_worker_blocks of s3r_render_scene_part."""
        if "all" not in self._dev:
            torch = _torch()
            w = self.w
            self._dev["all"] = (np.ascontiguousarray(w.blocks, dtype=np.uint32),
                                np.ascontiguousarray(w.node_off, dtype=np.uint64), to_device_n2i(w.n2i),
                                torch.from_numpy(np.ascontiguousarray(w.sparse, dtype=np.float32)).cuda())
        return self._dev["all"]

    def device_nodes(self, b: int):
        if b not in self._dev:
            torch = _torch()
            n2i, vals = self.w.block_nodes(b)
            self._dev[b] = (to_device_n2i(n2i), torch.from_numpy(np.ascontiguousarray(vals)).cuda())
        return self._dev[b]


class VsWorker:
    """VsWorkerInterface with the CUDA worker's renderScenePart: clear, order the
    index box back to front, render every block, read back, crop."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.lib = ctx.lib
        self.renderer = DenseFieldRenderer(ctx)
        self.state = None
        self.viewport = None

    def initialize(self, shader_path: str = "", log_info: bool = False, log_file: str = "", thread_id: int = 0):
        pass  # the context already bound the device (selectGpu)

    def set_render_shared_state(self, state: RenderSharedState):
        self.state = state
        self.renderer.set_render_shared_state(state)

    def update_state(self, flags: int = ~0):
        pass

    def render_scene_part(self, level: int, index_box_min, index_box_max, cancelled=lambda: False):
        part = self.render_scene_part_device(level, index_box_min, index_box_max, cancelled)
        if part is None:
            return None
        origin, size, pixels = part
        if size[0] == 0:
            return ImagePartResult((0, 0), (0, 0), np.zeros((0, 0), dtype=np.uint32))
        pix = pixels.cpu().numpy().view(np.uint32).reshape(size[1], size[0])
        return ImagePartResult(origin, size, pix)

    def render_scene_part_native(self, level: int, index_box_min, index_box_max, pres=None, sparse2_dev=None):
        """renderScenePart as one native call (s3r_render_scene_part): clear, back-to-front block loop
        (interpolate + render per block), bounding rectangle; the cropped part stays in device memory:
        (origin, size, int32 tensor), size (0, 0) when nothing was drawn."""
        torch = _torch()
        s = self.state
        W, H = s.view.W, s.view.H
        if self.viewport is None or self.viewport.numel() != W * H:
            self.viewport = torch.empty(W * H, dtype=torch.int32, device="cuda")
        blocks, node_off, n2i_dev, sparse_dev = s.device_all()
        wb = WorkerBlocks()
        wb.nblocks = blocks.shape[0]
        wb.blocks = arr(blocks, C.c_uint32)
        wb.node_off = arr(node_off, C.c_uint64)
        wb.n2i = ptr(n2i_dev)
        wb.sparse = ptr(sparse_dev)
        wb.sparse2 = ptr(sparse2_dev)
        bmin = (C.c_uint32 * 3)(*[int(x) for x in index_box_min])
        bmax = (C.c_uint32 * 3)(*[int(x) for x in index_box_max])
        rect = (C.c_int32 * 4)()
        if self.renderer._tf is None:
            self.renderer._tf = torch.from_numpy(np.ascontiguousarray(s.tf, dtype=np.float32)).cuda()
        self.ctx._check(self.lib.s3r_render_scene_part(self.ctx.h, C.byref(s.view),
                                                       C.byref(pres) if pres is not None else None, C.byref(wb),
                                                       bmin, bmax, ptr(self.renderer._tf), ptr(self.viewport), rect,
                                                       None))
        if rect[2] == 0:
            return (0, 0), (0, 0), torch.zeros(1, dtype=torch.int32, device="cuda")
        crop = torch.empty(rect[2] * rect[3], dtype=torch.int32, device="cuda")
        self.ctx.crop(self.viewport, W, list(rect), crop)
        return (int(rect[0]), int(rect[1])), (int(rect[2]), int(rect[3])), crop

    def render_scene_part_plan(self, plan, level: int, index_box_min, index_box_max, pres=None, bricks2=None):
        """renderScenePart from a FramePlan's brick store (interpolated with plan.interp for all blocks):
        one render launch per block of the box, back to front; the cropped part in device memory."""
        torch = _torch()
        s = self.state
        W, H = s.view.W, s.view.H
        if self.viewport is None or self.viewport.numel() != W * H:
            self.viewport = torch.empty(W * H, dtype=torch.int32, device="cuda")
        if self.renderer._tf is None:
            self.renderer._tf = torch.from_numpy(np.ascontiguousarray(s.tf, dtype=np.float32)).cuda()
        bmin = (C.c_uint32 * 3)(*[int(x) for x in index_box_min])
        bmax = (C.c_uint32 * 3)(*[int(x) for x in index_box_max])
        rect = (C.c_int32 * 4)()
        self.ctx._check(self.lib.s3r_render_scene_part_bricks(self.ctx.h, plan.h, C.byref(s.view),
                                                              C.byref(pres) if pres is not None else None,
                                                              ptr(bricks2), bmin, bmax, ptr(self.renderer._tf),
                                                              ptr(self.viewport), rect, None))
        if rect[2] == 0:
            return (0, 0), (0, 0), torch.zeros(1, dtype=torch.int32, device="cuda")
        crop = torch.empty(rect[2] * rect[3], dtype=torch.int32, device="cuda")
        self.ctx.crop(self.viewport, W, list(rect), crop)
        return (int(rect[0]), int(rect[1])), (int(rect[2]), int(rect[3])), crop

    def render_scene_part_device(self, level: int, index_box_min, index_box_max, cancelled=lambda: False):
        """renderScenePart with the cropped part left in device memory: (origin, size, int32 tensor),
        size (0, 0) when nothing was drawn; None when cancelled."""
        torch = _torch()
        s = self.state
        W, H = s.view.W, s.view.H
        if self.viewport is None or self.viewport.numel() != W * H:
            self.viewport = torch.empty(W * H, dtype=torch.int32, device="cuda")
        self.renderer.clear_viewport(self.viewport)
        cmin, cmax = host.index_box_world(level, index_box_min, index_box_max)
        order = host.b2f_order(index_box_min, index_box_max, cmin, cmax, s.w.eye)
        for idx in order:
            if cancelled():
                return None
            if tuple(int(x) for x in idx) not in s.block_index:
                continue
            self.renderer.render_dense_field(self.viewport, level, idx, cancelled)
        rect = self.ctx.bound_rect(self.viewport, W, H)
        if rect[2] == 0:
            return (0, 0), (0, 0), torch.zeros(1, dtype=torch.int32, device="cuda")
        crop = torch.empty(rect[2] * rect[3], dtype=torch.int32, device="cuda")
        self.ctx.crop(self.viewport, W, rect, crop)
        return (int(rect[0]), int(rect[1])), (int(rect[2]), int(rect[3])), crop
