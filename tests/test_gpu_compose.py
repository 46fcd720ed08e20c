"""Device image-part kernels vs the reference's integer blend (golden) and getBoundRect."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def test_compose_parts_matches_reference_blend(ctx, golden):
    for i in range(int(golden["blend_count"])):
        dst = golden[f"blend_{i}_dst"]
        src = golden[f"blend_{i}_src"]
        ox, oy, just, offx, offy = golden[f"blend_{i}_args"].tolist()
        d = _dev(dst)
        s = _dev(src)
        ctx.compose_parts([(s, (ox, oy), (src.shape[1], src.shape[0]))], d, dst.shape[1], dst.shape[0], (offx, offy),
                          just_copy_first=bool(just))
        got = d.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, golden[f"blend_{i}_out"]), i


def test_compose_many_parts_in_order(ctx):
    from revise_gb300 import host
    rng = np.random.default_rng(3)
    dst = rng.integers(0, 2 ** 32, size=(30, 40), dtype=np.uint64).astype(np.uint32)
    parts = []
    for _ in range(6):
        w, h = rng.integers(3, 15, size=2)
        src = rng.integers(0, 2 ** 32, size=(h, w), dtype=np.uint64).astype(np.uint32)
        parts.append((src, (int(rng.integers(0, 40 - w)), int(rng.integers(0, 30 - h)))))
    want = dst.copy()
    for src, o in parts:
        host.blend_image_part(want, src, o)
    d = _dev(dst)
    ctx.compose_parts([(_dev(s), o, (s.shape[1], s.shape[0])) for s, o in parts], d, 40, 30)
    assert np.array_equal(d.cpu().numpy().view(np.uint32), want)


def test_bound_rect_and_crop(ctx):
    img = np.zeros((50, 70), np.uint32)
    img[7, 12] = 0x01000000
    img[33, 60] = 0xff123456
    img[20, 5] = 0x80ffffff
    d = _dev(img)
    rect = ctx.bound_rect(d, 70, 50)
    assert rect == (5, 7, 56, 27)
    import torch
    out = torch.empty(rect[2] * rect[3], dtype=torch.int32, device="cuda")
    ctx.crop(d, 70, rect, out)
    assert np.array_equal(out.cpu().numpy().view(np.uint32).reshape(27, 56), img[7:34, 5:61])
    assert ctx.bound_rect(_dev(np.zeros((4, 4), np.uint32)), 4, 4) == (0, 0, 0, 0)
