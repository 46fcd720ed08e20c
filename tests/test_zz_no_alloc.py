"""s3r_interp_dense_noalloc, the allocation-free variant of s3r_interp_dense for
callers that cannot call cudaMalloc (their device memory belongs to their own
pool, or a device-wide synchronizing allocation would stall their frame loop).
Called through the C ABI, it must give the same grids as s3r_interp_dense
(bit-identical: the tolerance of every interpolation test here), on two calls in
a row that share its fixed scratch array, and must reject depths beyond its
8.6 MB scratch.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from revise_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def _same(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_no_alloc_matches_allocating_entry_point_on_two_calls(ctx):
    import torch
    from revise_gb300.api import to_device_n2i
    lib = _lib.load()
    w = workloads.small(seed=21, level=1, depths=(7, 4), mask_fraction=0.2)
    deep = int(np.flatnonzero(w.blocks[:, 3] == 7)[0])
    shallow = int(np.flatnonzero(w.blocks[:, 3] == 4)[0])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for b in (deep, shallow):  # the second call reuses the scratch the first one filled
        n2i, sp = w.block_nodes(b)
        d = int(w.blocks[b, 3])
        n2i_dev = to_device_n2i(n2i)
        sp_dev = torch.from_numpy(sp).cuda()
        want = ctx.interp_dense(n2i_dev, sp_dev, d).cpu().numpy()
        out = torch.empty(((1 << d) + 1) ** 3, dtype=torch.float32, device="cuda")
        rc = lib.s3r_interp_dense_noalloc(_lib.ptr(n2i_dev), _lib.ptr(sp_dev), sp.shape[0], d, _lib.ptr(out), stream)
        _lib.check(rc)
        torch.cuda.synchronize()
        assert _same(out.cpu().numpy(), want), (b, d)


def test_no_alloc_rejects_depth_beyond_its_scratch():
    lib = _lib.load()
    rc = lib.s3r_interp_dense_noalloc(C.c_void_p(0), C.c_void_p(0), 0, 8, C.c_void_p(1), C.c_void_p(0))
    assert rc == _lib.S3R_ERR_INVALID
    assert b"S3R_NOALLOC_MAX_DEPTH" in lib.s3r_last_error(None)
