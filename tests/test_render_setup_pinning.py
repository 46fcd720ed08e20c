"""The host-side parameter set-up of the reference's renderer, pinned by running its own code.

oracle/_ref/libs3r_refsetup.so is the reference's DenseFieldRenderer_cu (src/s3dmm_cuda/DenseFieldRenderer_cu.cu)
compiled from its sources and linked against a stand-in CUDA runtime (oracle/cuda_stub.cpp) that runs no
kernel but records each launch: renderDenseField then runs on the CPU over the reference-format fixture
dataset, and the RenderKernelParam it would launch renderKernel<mode> with is compared field by field, bit
for bit, with this library's set-up of the same block: the cube (s3r_block_cube), the eye, screen axes,
screen size and pixel size (s3r_camera_from_view, from the same camera transform), the view rectangle
(s3r_block_view_rect; a rectangle the reference leaves empty launches nothing), the absolute threshold
and isosurface levels (relative values through the reference's relToAbsFieldValue, sorted and made
unique), the field range and subtree depth, the quality, the isosurface opacity and the light position
(s3r_default_light).  The camera transform's inverse and normalisation are VisualizationLibrary's, which
is not vendored: both sides restate them for a rigid camera (oracle/shims_cuda/vlCore/Matrix4.hpp).
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from revise_gb300 import _lib, host
from revise_gb300.dataset import BlockTreeFieldService

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "oracle" / "_ref" / "libs3r_refsetup.so"
DATA = ROOT / "tests" / "golden" / "dataset" / "shell.dat"

pytestmark = pytest.mark.skipif(not LIB.exists(), reason="reference set-up harness not built (make -C oracle refsetup)")

CAMERAS = [  # eye, center, up, fovy, W, H
    ((0.0, 10.0, 35.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 1920, 1080),
    ((7.0, -4.0, 11.0), (0.5, 0.2, -0.3), (0.1, 1.0, 0.2), 45.0, 97, 61),
    ((-13.0, 6.0, -9.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 30.0, 640, 480),
    ((1.5, 2.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 320, 200),  # the eye inside the block tree
]
MODES = [  # mode, relative threshold, relative isosurface level, relative levels
    (_lib.MODE_ARGB, 0.5, 0.5, []),
    (_lib.MODE_ISOSURFACE, 0.3, 0.45, []),
    (_lib.MODE_ISOSURFACES, 0.5, 0.5, [0.8, 0.2, 0.5, 0.2, 0.35]),
]


def _reference(view_m, fovy, W, H, mode, thr, iso, levels, level, blocks):
    lib = C.CDLL(str(LIB))
    lib.ref_setup_error.restype = C.c_char_p
    n = blocks.shape[0]
    out = np.zeros((n, 88), np.uint32)
    lv = np.ascontiguousarray(levels, np.float32)
    rc = lib.ref_setup_params(str(DATA).encode(), view_m.ctypes.data_as(C.POINTER(C.c_float)), C.c_float(fovy),
                              C.c_uint32(W), C.c_uint32(H), C.c_uint32(mode), C.c_float(thr), C.c_float(iso),
                              C.c_float(0.6), lv.ctypes.data_as(C.POINTER(C.c_float)), C.c_uint32(lv.size),
                              C.c_float(1.5), C.c_uint32(level), C.c_uint32(n),
                              np.ascontiguousarray(blocks, np.uint32).ctypes.data_as(C.POINTER(C.c_uint32)),
                              out.ctypes.data_as(C.POINTER(C.c_uint32)))
    assert rc == 0, lib.ref_setup_error()
    return out


def _f(x):
    return np.asarray(x, np.float32).view(np.uint32)


@pytest.mark.parametrize("cam", range(len(CAMERAS)))
@pytest.mark.parametrize("mode", range(len(MODES)))
def test_render_setup_equals_reference(cam, mode):
    eye, center, up, fovy, W, H = CAMERAS[cam]
    m, thr_rel, iso_rel, levels_rel = MODES[mode]
    view_m = host.view_matrix_look_at(eye, center, up)
    camera = host.camera_from_view(view_m, fovy, W, H)
    with BlockTreeFieldService(str(DATA)) as svc:
        lo, hi = svc.field_range(0)
        md = svc.metadata()
        checked = launched = 0
        for level in range(md.level_count()):
            subs = md.level_blocks(level)
            if not subs:
                continue
            blocks = np.array([s.index for s in subs], np.uint32).reshape(-1, 3)
            ref = _reference(view_m, fovy, W, H, m, thr_rel, iso_rel, levels_rel, level, blocks)
            thr = host.relative_to_absolute(lo, hi, iso_rel if m == _lib.MODE_ISOSURFACE else thr_rel)
            if m == _lib.MODE_ISOSURFACES:
                thr = 0.0
            view = host.make_view(camera, W, H, level, lo, hi, thr, 1.5, 256)
            light = host.default_light(view)
            levels = sorted(set(host.relative_to_absolute(lo, hi, r) for r in levels_rel))
            for s, rec in zip(subs, ref):
                checked += 1
                rect = host.block_view_rect(view, s.index)
                if rect[2] == 0 or rect[3] == 0:
                    assert rec[85] == 0, (level, s.index, rect)  # the reference launches nothing either
                    continue
                assert rec[85] == 1, (level, s.index, rect)
                launched += 1
                c, h = host.block_cube(level, s.index)
                f = rec.view(np.float32)
                assert np.array_equal(rec[0:3], _f(c)) and rec[3] == _f(h) and rec[4] == level
                assert np.array_equal(rec[5:8], _f(camera.eye[:])), (rec[5:8].view(np.float32), camera.eye[:])
                assert np.array_equal(rec[8:11], _f(camera.e1[:]))
                assert np.array_equal(rec[11:14], _f(camera.e2[:]))
                assert np.array_equal(rec[14:17], _f(camera.n[:]))
                assert rec[17] == _f(camera.w) and rec[18] == _f(camera.h)
                assert rec[19] == _f(np.float32(camera.h) / np.float32(H))
                assert np.array_equal(rec[20:24], rect.astype(np.uint32)), (level, s.index, rec[20:24], rect)
                assert rec[24] == _f(thr), (f[24], thr)
                assert f[25] == np.float32(0.6) and f[26] == np.float32(1.5)
                assert rec[27] == s.depth
                assert rec[28] == _f(lo) and rec[29] == _f(hi)
                assert rec[30] == 1 and np.array_equal(rec[31:34], _f(light.pos[:]))
                if m == _lib.MODE_ISOSURFACES:
                    assert rec[34] == len(levels) and np.array_equal(rec[35:35 + len(levels)], _f(levels))
        assert checked > 0 and launched > 0
