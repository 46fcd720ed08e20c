"""The C++ drop-ins (revise_gb300/adapters) run through the reference's own interfaces on the GPU.

tests/adapters/adapter_check.cpp is compiled here against the reference's headers (the staged tree
oracle/_ref/tree, with the build shims of oracle/shims*) and this library:

* seam 1: every subtree of the reference-format fixture dataset through the reference's
  BlockTreeFieldService<3>::interpolateWith with DenseFieldInterpolatorGb300 and with the reference's own
  DenseFieldInterpolator<3>: the grids are bit-identical;
* seams 2 and 3: VsWorkerGb300 (rendering every block with DenseFieldRendererGb300) renders a level of the
  dataset from a VsRenderSharedState -- camera transform, viewport, field of view, quality, relative threshold,
  colour control points -- and its RgbaImagePart is compared with the reference's own CUDA kernels
  (oracle/refcu_harness.cpp: its interpolation and renderKernel<mode> from its sources) run block by block in
  the same order with the set-up the reference's renderer derives from the same state: at most 1 LSB.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import refcu
from revise_gb300 import _lib, host, workloads
from revise_gb300.build import cuda_home
from revise_gb300.dataset import BlockTreeFieldService

ROOT = Path(__file__).resolve().parents[1]
TREE = ROOT / "oracle" / "_ref" / "tree"
DATA = ROOT / "tests" / "golden" / "dataset" / "shell.dat"

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not (TREE / "include" / "s3dmm" / "BlockTreeFieldService.hpp").exists(),
                                 reason="reference headers not staged (make -C oracle stage REFERENCE=<root>)")]

FLAGS = ["-std=c++20", "-O2", "-DS3DMM_REAL_TYPE=float", "-DS3DMM_ENABLE_CUDA", "-DS3DMM_PROGRESS_REPORT"]


@pytest.fixture(scope="module")
def adapter_check(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    cuda = cuda_home()
    out = tmp_path_factory.mktemp("adapters")
    inc = [f"-I{ROOT / 'oracle' / 'shims_cuda'}", f"-I{ROOT / 'oracle' / 'shims'}", f"-I{TREE / 'include'}",
           f"-I{TREE / 'src' / 's3dmm_cuda'}"]
    cmds = [
        [str(cuda / "bin" / "nvcc"), *FLAGS, "-Xcompiler", "-fPIC", *inc, "-c",
         str(TREE / "src" / "s3dmm_cuda" / "DeviceMemHandle.cu"), "-o", str(out / "DeviceMemHandle.o")],
        ["g++", *FLAGS, "-ffp-contract=off", *inc, f"-I{ROOT / 'revise_gb300' / 'adapters'}", f"-I{ROOT / 'include'}",
         f"-I{cuda / 'include'}", "-c", str(ROOT / "tests" / "adapters" / "adapter_check.cpp"), "-o",
         str(out / "adapter_check.o")],
        ["g++", *FLAGS, f"-I{ROOT / 'oracle' / 'shims_cpu'}", f"-I{ROOT / 'oracle' / 'shims'}", f"-I{TREE / 'include'}",
         "-c", str(TREE / "src" / "s3dmm" / "ProgressReport.cpp"), "-o", str(out / "ProgressReport.o")],
    ]
    procs = [subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for c in cmds]
    for c, p in zip(cmds, procs):
        log = p.communicate()[0]
        assert p.returncode == 0, " ".join(c) + "\n" + log[-3000:]
    exe = out / "adapter_check"
    link = ["g++", "-o", str(exe), str(out / "DeviceMemHandle.o"), str(out / "adapter_check.o"),
            str(out / "ProgressReport.o"), f"-L{ROOT / 'revise_gb300'}", "-ls3r", f"-Wl,-rpath,{ROOT / 'revise_gb300'}",
            f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}", "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_interpolator_adapter_through_interpolate_with(adapter_check):
    r = subprocess.run([str(adapter_check), "interp", str(DATA)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    _, subtrees, vertices, bad = r.stdout.split()
    print(f"seam 1: {subtrees} subtrees, {vertices} dense vertices, {bad} differ")
    assert int(subtrees) > 100 and int(vertices) > 0 and int(bad) == 0


CASES = [  # mode, eye, relative threshold, relative isosurface level, W, H, fovy
    (_lib.MODE_ARGB, (4.0, 7.0, 16.0), 0.5, 0.5, 160, 120, 45.0),
    (_lib.MODE_ARGB, (-9.0, 5.0, 6.0), 0.3, 0.5, 97, 61, 60.0),
    (_lib.MODE_ISOSURFACE, (4.0, 7.0, 16.0), 0.5, 0.62, 160, 120, 45.0),
    (_lib.MODE_DOMAIN_VOXELS, (6.0, -8.0, 10.0), 0.2, 0.5, 128, 96, 50.0),
]


@pytest.mark.skipif(not refcu.available(), reason="reference CUDA cubins not built here")
@pytest.mark.parametrize("case", range(len(CASES)))
def test_worker_and_renderer_adapters_vs_reference_kernels(adapter_check, tmp_path, case):
    mode, eye, thr_rel, iso_rel, W, H, fovy = CASES[case]
    level, quality, opacity = 1, 1.5, 0.6
    xs, rgba = workloads.colormap_points()
    m = host.view_matrix_look_at(eye, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    inp = tmp_path / "in.txt"
    lines = [f"{level} {mode} {W} {H} {fovy!r} {quality!r} {thr_rel!r} {iso_rel!r} {opacity!r}",
             " ".join(repr(float(x)) for x in m), str(len(xs))]
    lines += [" ".join(repr(float(v)) for v in (x, *c)) for x, c in zip(xs, rgba)]
    inp.write_text("\n".join(lines) + "\n")
    outp = tmp_path / "part.bin"
    r = subprocess.run([str(adapter_check), "worker", str(DATA), str(inp), str(outp)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = outp.read_bytes()
    ox, oy, pw, ph = np.frombuffer(raw[:16], np.int32)
    part = np.frombuffer(raw[16:], np.uint32).reshape(ph, pw) if pw else np.zeros((0, 0), np.uint32)

    # the reference's kernels over the same blocks, with the set-up its renderer derives from the same state
    with BlockTreeFieldService(str(DATA)) as svc:
        lo, hi = svc.field_range(0)
        frame = svc.read_level(svc.level_topology(level), 0, 0)
    cam = host.camera_from_view(m, fovy, W, H)
    thr = host.relative_to_absolute(lo, hi, iso_rel if mode == _lib.MODE_ISOSURFACE else thr_rel)
    view = host.make_view(cam, W, H, level, lo, hi, thr, quality, 512, filter=_lib.FILTER_TEXTURE)
    pres = host.presentation(mode, view, isosurface_opacity=opacity)
    refcu.set_tf(workloads.color_table(xs, rgba, 512))
    mm = 1 << level
    order = host.b2f_order([0, 0, 0], [mm, mm, mm], *host.index_box_world(level, [0, 0, 0], [mm, mm, mm]),
                           [float(x) for x in cam.eye])
    where = {tuple(int(x) for x in b[:3]): i for i, b in enumerate(frame.blocks)}
    ref = np.zeros(W * H, np.uint32)
    for idx in order.tolist():
        b = where[tuple(idx)]
        n2i, sp = frame.block_nodes(b)
        rect = host.block_view_rect(view, idx)
        if mode == _lib.MODE_ARGB:
            refcu.render_block(view, n2i, sp, int(frame.blocks[b, 3]), idx, rect, ref)
        else:
            refcu.render_block_mode(view, pres, n2i, sp, int(frame.blocks[b, 3]), idx, rect, ref)
    ref = ref.reshape(H, W)
    ys, xs_ = np.nonzero(ref >> 24)
    assert ys.size > 0
    assert (ox, oy, pw, ph) == (xs_.min(), ys.min(), xs_.max() - xs_.min() + 1, ys.max() - ys.min() + 1)
    crop = ref[oy:oy + ph, ox:ox + pw]
    d = np.abs(part.view(np.uint8).reshape(-1, 4).astype(int) - crop.view(np.uint8).reshape(-1, 4).astype(int)).max(1)
    print(f"seams 2+3, mode {mode}: part {pw}x{ph} at ({ox}, {oy}), {(d > 0).sum()} pixels differ, max {d.max()} LSB")
    assert d.max() <= 1
