"""Host-side logic of the s3r C ABI (no GPU): symbols, ordering, transfer
function, blend, camera and view-rectangle set-up."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from revise_gb300 import _lib, host, workloads

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "s3r.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(s3r_\w+)\s*\(", text, re.M)))


def test_library_loads_and_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.s3r_abi_version() == _lib.ABI_VERSION
    # every binding the Python layer declares exists in the header too
    assert set(_lib.EXPORTED) <= set(syms)


def test_header_constants_match_the_bindings():
    text = (ROOT / "include" / "s3r.h").read_text()

    def define(name):
        return int(re.search(rf"#define {name} (\d+)u?", text).group(1))

    assert define("S3R_RENDER_TILES_WALK") == _lib.RENDER_TILES_WALK
    assert define("S3R_RENDER_TILES") == _lib.RENDER_TILES
    assert define("S3R_ABI_VERSION") == _lib.ABI_VERSION
    assert define("S3R_MAX_DEPTH") == _lib.MAX_DEPTH


def test_b2f_order_matches_reference(golden):
    for i in range(int(golden["b2f_count"])):
        a = golden[f"b2f_{i}_args"]
        bmin, bmax = a[0:3].astype(int).tolist(), a[3:6].astype(int).tolist()
        got = host.b2f_order(bmin, bmax, a[6:9], a[9:12], a[12:15])
        assert np.array_equal(got, golden[f"b2f_{i}_order"]), (i, a)


def test_b2f_order_is_a_permutation_of_the_box():
    got = host.b2f_order([1, 2, 0], [5, 4, 3], [-1, -1, -1], [1, 1, 1], [0.1, 5.0, -0.3])
    assert got.shape == (4 * 2 * 3, 3)
    assert len({tuple(x) for x in got.tolist()}) == 24


def test_color_transfer_matches_reference(golden):
    for i in range(int(golden["ctf_count"])):
        got = host.make_color_transfer(golden[f"ctf_{i}_xs"], golden[f"ctf_{i}_rgba"], int(golden[f"ctf_{i}_count"]))
        assert np.array_equal(got, golden[f"ctf_{i}_out"]), i


def test_host_blend_matches_reference(golden):
    for i in range(int(golden["blend_count"])):
        dst = golden[f"blend_{i}_dst"].copy()
        ox, oy, just, offx, offy = golden[f"blend_{i}_args"].tolist()
        host.blend_image_part(dst, golden[f"blend_{i}_src"], (ox, oy), bool(just), (offx, offy))
        assert np.array_equal(dst, golden[f"blend_{i}_out"]), i


def test_blend_rejects_parts_outside_destination():
    dst = np.zeros((4, 4), np.uint32)
    src = np.zeros((2, 2), np.uint32)
    with pytest.raises(_lib.S3RError):
        host.blend_image_part(dst, src, (3, 3))


def test_camera_look_at_matches_numpy():
    eye, center, up = np.array([0.0, 10.0, 35.0]), np.zeros(3), np.array([0.0, 1.0, 0.0])
    cam = host.camera_look_at(eye, center, up, 60.0, 1920, 1080)
    z = (eye - center) / np.linalg.norm(eye - center)
    x = np.cross(up, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    np.testing.assert_allclose(cam.e1[:], x, atol=1e-7)
    np.testing.assert_allclose(cam.e2[:], y, atol=1e-7)
    np.testing.assert_allclose(cam.n[:], -0.1 * z, atol=1e-7)
    np.testing.assert_allclose(cam.h, 0.2 * np.tan(np.pi / 6), rtol=1e-6)
    np.testing.assert_allclose(cam.w, cam.h / 1080 * 1920, rtol=1e-6)
    R = np.array(cam.view_r[:]).reshape(3, 3)
    np.testing.assert_allclose(R @ eye + np.array(cam.view_t[:]), 0, atol=1e-5)


@pytest.mark.parametrize("cfg", ["small", "cfg1", "cfg2"])
def test_view_rect_matches_oracle(cfg):
    w = workloads.small() if cfg == "small" else (workloads.cfg1() if cfg == "cfg1" else None)
    if w is None:
        w = workloads.small(level=2, depths=(1,), W=1920, H=1080, eye=(0.0, 10.0, 35.0))
    v = host.view_for(w)
    ov = oracle.view_from(v)
    m = 1 << w.level
    for ix in range(m):
        for iy in range(m):
            for iz in range(m):
                a = host.block_view_rect(v, (ix, iy, iz))
                b = oracle.block_view_rect(ov, v.cam.view_r[:], v.cam.view_t[:], (ix, iy, iz))
                assert np.array_equal(a, b), (ix, iy, iz, a, b)
                assert a[2] >= 0 and a[3] >= 0


def test_view_rect_eye_inside_covers_viewport():
    cam = host.camera_look_at((0.1, 0.2, 0.3), (0.0, 0.0, -10.0), (0, 1, 0), 50.0, 64, 48)
    v = host.make_view(cam, 64, 48, 0, 0.0, 1.0, 0.5, 1.0, 256)
    assert host.block_view_rect(v, (0, 0, 0)).tolist() == [0, 0, 64, 48]


def test_block_cube_and_index_box_world():
    c, h = host.block_cube(2, (0, 3, 1))
    assert h == np.float32(1.25)
    np.testing.assert_array_equal(c, np.array([-3.75, 3.75, -1.25], np.float32))
    cmin, cmax = host.index_box_world(4, (0, 0, 0), (16, 16, 16))
    np.testing.assert_allclose(cmin, -5.0)
    np.testing.assert_allclose(cmax, 5.0)


def test_invalid_arguments_return_status_and_message(lib):
    cnt = C.c_uint32()
    rc = lib.s3r_b2f_order(None, None, None, None, None, None, 0, C.byref(cnt))
    assert rc == _lib.S3R_ERR_INVALID
    assert lib.s3r_last_error(None)
    out = (C.c_float * 4)()
    assert lib.s3r_make_color_transfer(None, None, 3, 4, out) == _lib.S3R_ERR_INVALID
    v = host.make_view(host.camera_look_at((0, 0, 5), (0, 0, 0), (0, 1, 0), 40, 8, 8), 8, 8, 0, 1.0, 1.0, 0.5, 1.0,
                       16)
    r = (C.c_int32 * 4)()
    assert lib.s3r_block_view_rect(C.byref(v), (C.c_uint32 * 3)(0, 0, 0), r) == _lib.S3R_ERR_INVALID
    with pytest.raises(_lib.S3RError, match="field range"):
        host.block_view_rect(v, (0, 0, 0))
