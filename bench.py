#!/usr/bin/env python3
"""Benchmark of the batched, graph-captured frame on one GPU per rank.

A step is one frame of the 4096-block configuration (16^3 blocks of octree
depth 3..7, ~626 M dense vertices, 1920x1080): interpolation of every block
from its sparse nodes into the HBM-resident brick store, then the front-to-back
ray cast of the whole block cube, replayed as one CUDA graph.  Inputs are
seeded synthetic data with the configuration's shapes and distributions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU implementation of the path -- its
dense-field generator, DenseFieldInterpolator<3>, compiled from its own header
(oracle/_ref, staged reference sources; the C restatement in oracle/ where that
was not built) -- on all host cores over a bounded sample of the same blocks.
The reference has no CPU ray caster, so that number covers interpolation only
(which favours it).

For N > 1 (torchrun), every rank runs the same frame on its own GPU (replicas:
the path has no exchange step on one node), value = all ranks' vertices / the
slowest rank's time.  One JSON line is printed by rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "dense Gvertices/s; Gsamples/s & ms/frame @1080p; adjoint/forward time ratio"
UNIT = "Gvertices/s"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--config", choices=["cfg3", "cfg2", "cfg3-l3"], default="cfg3",
                    help="cfg3-l3: the same block recipe at level 3 (512 blocks, ~97 M vertices), "
                         "the small case for kernel captures")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--render-tile", type=int, default=None,
                    help="render form and CTA shape id (s3r.h S3R_RENDER_TILES); implies --no-autotune")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the adjoint, 16-bit and reference-CUDA measurements")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="only the adjoint measurement (cfg5), one JSON line; for profiling the backward kernel")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def make_workload(name):
    from revise_gb300 import workloads
    if name == "cfg3-l3":
        return workloads.cfg3(level=3)
    return workloads.cfg3() if name == "cfg3" else workloads.cfg2()


# ------------------------------------------------------------------ CPU legs
#
# The reference's CPU dense-field generator is DenseFieldInterpolator<3>::interpolate
# (include/s3dmm/DenseFieldInterpolator.hpp:198-419).  Where its header has been compiled here
# (oracle/_ref/libs3r_ref.so, built from the staged reference sources) that code itself is timed
# (kind "reference"); else the C restatement in oracle/ (kind "port").

_W = {}


def _cpu_worker_init(depths, n2i_list, sp_list, use_ref):
    """Pool initializer: the sample's blocks, sent once per worker."""
    import oracle
    _W.update(depths=depths, n2i=n2i_list, sp=sp_list, fn=oracle.ref_interp if use_ref else oracle.interp_f32)
    _W["fn"](n2i_list[0], sp_list[0], depths[0])  # load the library before the timed region


def _cpu_interp_chunk(ids):
    """Worker: interpolate the listed sample blocks, return the dense vertices produced."""
    v = 0
    for i in ids:
        d = _W["depths"][i]
        _W["fn"](_W["n2i"][i], _W["sp"][i], d)
        v += ((1 << d) + 1) ** 3
    return v


def _cpu_rate_guess():
    """Dense vertices/s one host core interpolates (measured on this machine's hosts, for sizing samples):
    ~15 M for the reference's header, ~60 M for the restatement."""
    import oracle
    return 15e6 if oracle.ref_available() else 60e6


def _sample_blocks(w, seconds_budget, seed=0):
    """A random block sample whose CPU interpolation takes roughly the budget (single core)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    order = rng.permutation(w.nblocks)
    target = seconds_budget * _cpu_rate_guess()
    picked, tot = [], 0
    for b in order:
        d = int(w.blocks[b, 3])
        picked.append(int(b))
        tot += ((1 << d) + 1) ** 3
        if tot >= target:
            break
    return picked


class CpuInterp:
    """The reference's CPU dense-field generator over a block sample on `processes` host processes: the
    pool is started (spawn) and the sample sent to every worker once, before any timing; a timed step is
    one map of the sample's blocks over the warm workers."""

    def __init__(self, w, blocks, processes: int):
        import oracle
        self.kind = "reference" if oracle.ref_available() else "port"
        self.depths = [int(w.blocks[b, 3]) for b in blocks]
        self.vertices = sum(((1 << d) + 1) ** 3 for d in self.depths)
        self.processes = processes
        n2i = [w.block_nodes(b)[0] for b in blocks]
        sp = [w.block_nodes(b)[1] for b in blocks]
        order = sorted(range(len(blocks)), key=lambda i: -self.vertices_of(i))
        self.chunks = [order[k::processes] for k in range(processes)]  # largest blocks dealt round-robin
        self.pool = None
        if processes == 1:
            _cpu_worker_init(self.depths, n2i, sp, self.kind == "reference")
        else:
            import multiprocessing as mp
            self.pool = mp.get_context("spawn").Pool(processes, initializer=_cpu_worker_init,
                                                     initargs=(self.depths, n2i, sp, self.kind == "reference"))
            self.pool.map(_cpu_interp_chunk, [[] for _ in range(processes)], chunksize=1)  # workers up

    def vertices_of(self, i):
        return ((1 << self.depths[i]) + 1) ** 3

    def step(self):
        """Vertices/s of one pass over the sample (wall time of the pass only)."""
        t = time.perf_counter()
        if self.pool is None:
            v = _cpu_interp_chunk(self.chunks[0])
        else:
            v = sum(self.pool.map(_cpu_interp_chunk, self.chunks, chunksize=1))
        return v / (time.perf_counter() - t)

    def close(self):
        if self.pool is not None:
            self.pool.close()
            self.pool.join()


def _repo_native_libraries():
    """The shared objects of this repository mapped into the process (what ran natively)."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                p = line.split()[-1] if line.strip() else ""
                if p.endswith(".so") and str(ROOT) in p:
                    out.add(str(Path(p).relative_to(ROOT)))
    except OSError:
        pass
    return sorted(out)


def run_reference(a):
    rank, world, _ = dist_env()
    if world > 1 and rank != 0:
        return 0
    import oracle
    oracle.port()
    w = make_workload(a.config)
    cores = os.cpu_count() or 1
    budget = max(1.0, a.cpu_seconds / max(1, a.steps + a.warmup)) * cores
    blocks = _sample_blocks(w, budget, seed=1)
    cpu = CpuInterp(w, blocks, cores)
    rates = []
    for i in range(a.warmup + a.steps):
        r = cpu.step()
        if i >= a.warmup:
            rates.append(r)
    cpu.close()
    value = statistics.median(rates) / 1e9
    what = ("the reference's DenseFieldInterpolator<3> compiled from its header (oracle/_ref/libs3r_ref.so)"
            if cpu.kind == "reference" else "DenseFieldInterpolator<3> restated (oracle/s3r_oracle.c)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": w.vertices / (value * 1e9) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"{a.config}: {w.nblocks} blocks, depths {int(w.blocks[:, 3].min())}-"
                               f"{int(w.blocks[:, 3].max())}, {w.vertices} dense vertices",
                   "what": "dense-field generation only (the reference has no CPU ray caster)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": cpu.kind,
                         "sample": f"{len(blocks)} blocks ({cpu.vertices} vertices) per step, {cores} processes "
                                   f"started once before the warm-up, {what}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not a.no_extras:
        line["reference_cuda"] = reference_cuda_frames(w, a)
    line["native_libraries"] = _repo_native_libraries()
    print(json.dumps(line))
    return 0


def reference_cuda_frames(w, a):
    """The reference's own GPU renderer on the same frame: its CUDA kernels (compiled from its sources into
    oracle/_ref/*.cubin) driven block by block in back-to-front order by the restated worker loop -- per
    block: upload of the sparse values, the d-pass dense interpolation, renderKernel<Argb> into the shared
    viewport; then the image read back and cropped.  The camera, the block order (the reference's own
    BackToFrontOrder, oracle/_ref/libs3r_ref.so) and the view rectangles come from the oracle side, not
    from this library.  Wall-clock ms per frame."""
    try:
        import numpy as np
        import torch
        import oracle
        from oracle import refcu
        if not (torch.cuda.is_available() and refcu.available()):
            return {"unavailable": "reference cubins not built (they compile from the staged reference tree)"}
        if not oracle.ref_available():
            return {"unavailable": "the reference's BackToFrontOrder (oracle/_ref/libs3r_ref.so) is not built"}
        cam = oracle.look_at_camera(w.eye, w.center, w.up, w.fovy, w.W, w.H)
        view = refcu.harness_view(cam, w.W, w.H, w.level, w.field_min, w.field_max, w.threshold, w.quality,
                                  w.tf.shape[0])
        ov = oracle.orc_view(cam, w.W, w.H, w.level, w.field_min, w.field_max, w.threshold, w.quality,
                             w.tf.shape[0], 1)
        refcu.set_tf(np.ascontiguousarray(w.tf, np.float32))
        m = 1 << w.level
        order = oracle.ref_b2f_order([0, 0, 0], [m, m, m], [-5.0] * 3, [5.0] * 3, w.eye)
        idx = {tuple(b[:3]): i for i, b in enumerate(w.blocks.tolist())}
        oi = np.array([idx[tuple(b)] for b in order.tolist()])
        rects = np.array([oracle.block_view_rect(ov, cam["view_r"], cam["view_t"], w.blocks[b, :3])
                          for b in range(w.nblocks)], np.int32)
        times = []
        for i in range(2 + max(1, min(a.steps, 5))):
            _, _, ms = refcu.worker(view, w, oi, rects)
            if i >= 2:
                times.append(ms)
        ms = statistics.median(times)
        out = {"ms_per_frame": ms, "frames_per_s": 1e3 / ms, "frames": len(times),
               "what": "reference CUDA kernels, reference worker loop (per-block H2D, interpolate, render)"}
        try:
            im, rm = refcu.worker_kernel_ms(view, w, oi, rects)
            out["kernel_ms"] = {"interpolation": im, "render": rm, "total": im + rm,
                                "how": "the same loop with every kernel launch bracketed by CUDA events and waited "
                                       "for: kernel time only, host copies and launch gaps excluded"}
        except Exception as e:  # the wall-clock figure stands without it
            out["kernel_ms"] = {"unavailable": f"{type(e).__name__}: {e}"}
        return out
    except Exception as e:  # the CPU line stands without it
        return {"unavailable": f"{type(e).__name__}: {e}"}


# ------------------------------------------------------------------ clocks

class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = None
        self.start_line = 0

    def mark(self):
        """The timed region starts now: samples written so far are not reported (but the last of them, taken
        under the warm-up's load, stands in when the region is shorter than one sampling interval)."""
        if self.f is not None:
            with open(self.f.name) as fh:
                self.start_line = len(fh.read().splitlines())

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "10"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the timed region starts once the sampler runs (its first line is written)
        t_end = time.time() + 5.0
        while time.time() < t_end and self.proc.poll() is None:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.f.read().splitlines()
        for line in lines[self.start_line:] or lines[-1:]:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ GPU arm

def run_gb300(a):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    from revise_gb300 import _lib, host, workloads
    from revise_gb300.api import Context, FramePlan

    w = make_workload(a.config)
    ctx = Context(dev)
    view = host.view_for(w)
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=16, render_tile=a.render_tile or 0)
    stream = torch.cuda.current_stream()
    sparse = torch.from_numpy(w.sparse).cuda()
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    W, H = w.W, w.H
    rgba = torch.zeros(W * H * 4, dtype=torch.float32, device="cuda")
    argb = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    samples = torch.zeros(1, dtype=torch.int64, device="cuda")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    if not a.no_autotune and a.render_tile is None:
        plan.autotune(view, sparse, tf, reps=3)
    info = plan.info
    depths = sorted({int(d) for d in w.blocks[:, 3]})
    tiles_by_depth = {str(d): plan.tile_cells(d) for d in depths}
    V = int(info.vertices)
    alg_bytes = 10 * int(info.nodes) + 4 * V  # n2i + values per node, one dense write per vertex

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed(fn, k):
        """k runs of fn, each bracketed by CUDA events on the stream, L2 flushed between runs."""
        ts = []
        for _ in range(k):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            ts.append((e0, e1))
        torch.cuda.synchronize()
        return [x.elapsed_time(y) for x, y in ts]

    frame = lambda: plan.run(view, sparse, tf, rgba, argb)  # noqa: E731
    clocks = Clocks(dev)
    clocks.start()  # sampling runs through the warm-up; only samples after mark() are reported
    for _ in range(max(3, a.warmup)):
        frame()
    torch.cuda.synchronize()
    clocks.mark()
    barrier()
    l0 = ctx.launches
    step_ms = timed(frame, a.steps)
    launches = ctx.launches - l0
    barrier()
    clk = clocks.stop()
    ms = sum(step_ms) / len(step_ms)
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    # kernel-level figures (same stream, CUDA events): interpolation and render alone
    interp_ms = timed(lambda: plan.interp(sparse), max(5, a.steps // 2))
    samples.zero_()
    render_ms = timed(lambda: plan.render(view, tf, rgba, None, samples), max(5, a.steps // 2))
    nsamp = int(samples.item()) / max(5, a.steps // 2)
    t_interp = statistics.median(interp_ms)
    t_render = statistics.median(render_ms)

    # end to end through the C ABI with host buffers: H2D of the sparse values, frame, D2H of the image
    sparse_host = torch.from_numpy(w.sparse).pin_memory()
    img_host = torch.empty(W * H, dtype=torch.int32).pin_memory()
    sparse_e2e = torch.empty_like(sparse)

    def e2e_step():
        sparse_e2e.copy_(sparse_host, non_blocking=True)
        plan.run(view, sparse_e2e, tf, rgba, argb)
        img_host.copy_(argb, non_blocking=True)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = timed(e2e_step, max(5, a.steps // 2))
    t_e2e_serial = sum(e2e_ms) / len(e2e_ms)

    # the same through s3r_frame_run_host: K frames back to back from pinned host buffers, each frame's
    # H2D overlapping the previous frame and its D2H the next one; timed from the first submit until
    # the last image has landed in host memory (pipeline fill and drain included)
    K = max(10, a.steps)
    for _ in range(3):
        plan.run_host(view, sparse_host, tf, img_host)
    plan.host_sync()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(K):
        plan.run_host(view, sparse_host, tf, img_host)
    plan.host_sync()
    e1.record(stream)
    torch.cuda.synchronize()
    t_e2e = e0.elapsed_time(e1) / K
    if dist is not None:
        t = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())

    extras = {}
    if not a.no_extras and rank == 0:
        extras = measure_extras(ctx, torch, np)
        extras["ingest"] = measure_ingest(ctx, torch, np, w, with_reference=not a.no_cpu)
        extras["modes"] = measure_modes(ctx, torch, np, with_reference=not a.no_cpu)
        extras["worker_loop"] = measure_worker_loop(ctx, torch, np, w)

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = peaks.get("hbm_gbs")
    peak_note = "of measured"
    if not hbm:
        hbm, peak_note = 6800.0, "of fallback"
    achieved = alg_bytes / (t_interp * 1e-3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "interp_tiles_cfg3_traffic.json"
    if tp.exists() and a.config == "cfg3":
        traffic = json.loads(tp.read_text()).get("dram_bytes_per_launch")
    # the render: DRAM bytes per frame and L2 hit rate from the committed ncu capture of the same
    # render form on this workload, over this run's CUDA-event time
    render_roof = None
    rp = ROOT / "profiles" / "frame_render_cfg3_traffic.json"
    if rp.exists() and a.config == "cfg3":
        rj = json.loads(rp.read_text())
        form = rj.get("render_tiles", {}).get(str(int(info.render_tile)))
        if form:
            gbs = form["dram_bytes_per_frame"] / (t_render * 1e-3) / 1e9
            render_roof = {"bound": "hbm", "kernels": form["kernels"], "traffic": form["dram_bytes_per_frame"],
                           "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm, "peak_source": peak_note,
                           "l2_hit_rate": form.get("l2_hit_rate"), "how": rj.get("how")}

    cpu = None
    if rank == 0 and not a.no_cpu:
        blocks = _sample_blocks(w, a.cpu_seconds, seed=2)
        ci = CpuInterp(w, blocks, 1)
        t0 = time.perf_counter()
        rate = ci.step()
        secs = time.perf_counter() - t0
        cpu = {"value": rate / 1e9, "unit": UNIT, "cores": 1, "kind": ci.kind,
               "sample": f"{len(blocks)} of {w.nblocks} blocks ({ci.vertices} vertices, {secs:.1f} s), one core, "
                         "dense-field generation only (DenseFieldInterpolator<3>"
                         + (", the reference's header compiled here)" if ci.kind == "reference" else ", restated)")}

    if rank == 0:
        value = world * V / (ms * 1e-3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, revise_gb300/workloads.py)",
            "config": {"workload": f"{a.config}: {w.nblocks} blocks ({1 << w.level}^3 at level {w.level}), octree depths "
                                   f"{int(w.blocks[:, 3].min())}-{int(w.blocks[:, 3].max())}, "
                                   f"{V} dense vertices, {int(info.nodes)} sparse nodes, {W}x{H}, "
                                   "interpolate + ray-cast per frame, CUDA graph",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                       "l2": "L2 flushed (2x129 MB write) between timed steps; 2.5 GB brick store per step",
                       "tile_cells": int(info.tile_cells), "tile_cells_by_depth": tiles_by_depth,
                       "render_tile": int(info.render_tile),
                       "render_form": "block-major" if int(info.render_tile) >= _lib.RENDER_TILES_WALK else "per-ray walk"},
            "ms_per_frame": ms, "frames_per_s": 1e3 / ms,
            "interp": {"ms": t_interp, "gvertices_per_s": V / (t_interp * 1e-3) / 1e9,
                       "algorithmic_bytes": alg_bytes},
            "render": {"ms": t_render, "gsamples_per_s": nsamp / (t_render * 1e-3) / 1e9, "samples": nsamp,
                       "roofline": render_roof},
            "roofline": {"bound": "hbm", "kernel": "interp_tiles_kernel (batched tile interpolation)",
                         "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "peak_source": peak_note, "traffic": traffic},
            "e2e": {"value": V / (t_e2e * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": t_e2e,
                    "h2d_bytes_per_step": int(sparse.numel() * 4), "d2h_bytes_per_step": int(W * H * 4),
                    "how": f"s3r_frame_run_host, {K} frames back to back from pinned host buffers, copies "
                           "overlapped with the neighbouring frames and consecutive frames overlapped on the GPU "
                           "(two slots, two brick stores, two streams), first submit to last image in host memory; "
                           f"no L2 flush between frames: every frame writes the {info.brick_bytes / 1e9:.2f} GB "
                           "brick store (the L2 holds 129 MB)"},
            "e2e_serial": {"value": V / (t_e2e_serial * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": t_e2e_serial,
                           "how": "per step: H2D, frame (s3r_frame_run), D2H in series on one stream, L2 flushed "
                                  "between steps"},
            "gpu_launches": int(launches),
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        line.update(extras)
        # the key figures once more, last, so that a reader of only the end of the line sees them
        summ = {"ms_per_frame": ms, "interp_ms": t_interp, "interp_roofline_frac": achieved / hbm, "render_ms": t_render,
                "render_roofline_frac": render_roof["frac"] if render_roof else None,
                "e2e_ms_per_frame": t_e2e}
        if "adjoint" in extras:
            summ["adjoint_forward_ratio"] = extras["adjoint"]["adjoint_forward_ratio"]
        sp = [v["speedup"] for v in extras.get("modes", {}).values() if isinstance(v, dict) and "speedup" in v]
        if sp:
            summ["per_block_modes_speedup_min_max"] = [min(sp), max(sp)]
        pc = extras.get("precision_cfg2")
        if pc:
            summ["cfg2_ms_f32_f16_bf16"] = [pc[k]["ms_per_frame"] for k in ("f32", "f16", "bf16")]
        line["summary"] = summ
        print(json.dumps(line))
    plan.close()
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def measure_ingest(ctx, torch, np, w, with_reference: bool):
    """Sparse-field ingestion from the reference's on-disk format: the workload written as a dataset
    (outside the timing), then per frame its level read and uploaded (s3r_dataset_frame_upload:
    parallel positioned reads into pinned staging, one host-to-device copy) against the reference
    worker's pattern (per block: open, seek, read of the field file, then separate copies of the
    block's node list and values to the device)."""
    import shutil
    import tempfile
    import time
    from revise_gb300 import workloads
    from revise_gb300.dataset import BlockTreeFieldService, write_dataset
    tmp = tempfile.mkdtemp(prefix="s3r_ingest_")
    try:
        t0 = time.perf_counter()
        base = tmp + "/" + w.name + ".dat"
        write_dataset(base, workloads.tree_blocks(w), 7, w.level, [("f", workloads.dataset_values(w))])
        t_write = time.perf_counter() - t0
        svc = BlockTreeFieldService(base)
        fr = svc.level_topology(w.level, w.blocks[:, :3])
        assert np.array_equal(fr.blocks, w.blocks) and np.array_equal(fr.node_off, w.node_off)
        dev = torch.empty(fr.nodes, dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream()
        nbytes = fr.nodes * 4

        def batched():
            svc.upload(ctx, fr, 0, 0, dev, stream=stream)
            stream.synchronize()

        for _ in range(3):
            batched()
        ts = []
        for _ in range(10):
            t = time.perf_counter()
            batched()
            ts.append(time.perf_counter() - t)
        ms = statistics.median(ts) * 1e3
        host = dev.cpu().numpy()
        svc.read_level(fr, 0, 0)
        ok = bool(np.array_equal(host.view(np.uint32), fr.sparse.view(np.uint32)))
        out = {"workload": f"{w.name}: level {w.level}, {fr.nblocks} subtrees, {fr.nodes} nodes "
                           f"({nbytes / 1e6:.1f} MB of values) from a reference-format dataset in the page cache",
               "dataset_write_s": t_write, "ms_per_level": ms, "gb_per_s": nbytes / (ms * 1e-3) / 1e9,
               "threads": os.cpu_count(), "h2d_copies": 1, "identical_to_host_read": ok}
        # upstream generation: level w.level-1 from the uploaded level (s3r_dataset_propagate + divide)
        from revise_gb300.dataset import field_divide
        md = svc.metadata()
        subs4 = md.level_blocks(w.level)
        vals4 = np.concatenate([svc.field_values(0, 0, w.level, x.index)[1] for x in subs4])
        child = torch.from_numpy(vals4).cuda()
        np3 = sum(x.node_count for x in md.level_blocks(w.level - 1))
        sums = torch.empty(np3, device="cuda")
        wts = torch.empty(np3, device="cuda")
        vals3 = torch.empty(np3, device="cuda")
        t0 = time.perf_counter()
        counts = svc.propagate(ctx, w.level - 1, child, sums, wts)
        t_index = time.perf_counter() - t0

        def prop():
            svc.propagate(ctx, w.level - 1, child, sums, wts, stream=stream)
            field_divide(ctx, sums, wts, vals3, stream=stream)

        for _ in range(3):
            prop()
        pms = []
        for _ in range(10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prop()
            e1.record(stream)
            torch.cuda.synchronize()
            pms.append(e0.elapsed_time(e1))
        out["propagate"] = {"level": w.level - 1, "parents": int(counts.size), "complete_parents": int((counts == 8).sum()),
                            "parent_nodes": int(np3), "child_nodes": int(vals4.size), "index_build_s": t_index,
                            "ms_per_level": statistics.median(pms)}
        if with_reference:
            import oracle
            from oracle import fieldgen
            t0 = time.perf_counter()
            cv, o = {}, 0
            for x in subs4:
                cv[tuple(x.index)] = (x.depth, vals4[o:o + x.node_count])
                o += x.node_count
            res = []
            for x in md.level_blocks(w.level - 1):
                n2i = md.block_tree_nodes(w.level - 1, x.index)
                f = np.zeros(x.node_count, np.float32)
                wt = np.zeros(x.node_count, np.float32)
                kids = []
                for c in range(8):
                    ci = (2 * x.index[0] + (c & 1), 2 * x.index[1] + ((c >> 1) & 1), 2 * x.index[2] + (c >> 2))
                    if ci in cv:
                        kids.append((c, cv[ci][0], md.block_tree_nodes(w.level, ci), cv[ci][1]))
                fieldgen.propagate_into(n2i, x.depth, kids, f, wt)
                res.append(fieldgen.divide(f, wt))
            t_port = time.perf_counter() - t0
            same = bool(np.array_equal(np.concatenate(res).view(np.uint32), vals3.cpu().numpy().view(np.uint32)))
            out["propagate"].update({"port_s": t_port, "port_kind": "numpy restatement (oracle/fieldgen.py), 1 core",
                                     "identical_to_port": same})
            subs = [svc.metadata().subtree_data(w.level, ix) for ix in w.blocks[:, :3]]
            offs = np.array([x.values_offset for x in subs], dtype=np.uint64)
            cnts = np.array([x.node_count for x in subs], dtype=np.uint64)
            n2i = [torch.from_numpy(w.block_nodes(b)[0].view(np.int16)) for b in range(w.nblocks)]
            no = [int(v) for v in w.node_off]

            def per_block():
                vals, _ = oracle.read_blocks_per_call(base + ".s3dmm-field#f", offs, cnts)
                v = torch.from_numpy(vals)
                for b in range(w.nblocks):
                    n2i[b].to("cuda")
                    v[no[b]:no[b + 1]].to("cuda")
                torch.cuda.synchronize()

            per_block()
            tr = []
            for _ in range(3):
                t = time.perf_counter()
                per_block()
                tr.append(time.perf_counter() - t)
            rms = statistics.median(tr) * 1e3
            out["reference_pattern"] = {"ms_per_level": rms, "gb_per_s": nbytes / (rms * 1e-3) / 1e9,
                                        "threads": 1, "h2d_copies": 2 * w.nblocks, "kind": "port",
                                        "speedup_batched": rms / ms}
        svc.close()
        return out
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


MODE_NAMES = {0: "isosurface", 1: "isosurfaces", 2: "max_intensity", 3: "argb", 4: "argb_light",
              5: "domain_voxels", 6: "value_on_isosurface", 7: "value_on_isosurfaces"}


def measure_modes(ctx, torch, np, with_reference: bool):
    """Every field mode of the per-block renderer (s3r_render_block; texture filter, and the exact
    filter beside it) over cfg2's 64
    blocks of depth 6 at 1920x1080, back to front into one viewport: the summed CUDA-event times of the
    64 render launches (each block's dense field interpolated first, not timed); beside it the same
    measurement of the reference's own renderKernel<mode> (its kernels from cubins) when built."""
    from revise_gb300 import _lib, host, workloads
    from revise_gb300.api import to_device_n2i
    w = workloads.cfg2()
    m = 1 << w.level
    order = host.b2f_order([0, 0, 0], [m, m, m], [-5.0] * 3, [5.0] * 3, w.eye)
    where = {tuple(b[:3]): i for i, b in enumerate(w.blocks.tolist())}
    oi = np.array([where[tuple(b)] for b in order.tolist()])
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    dense, dense2 = {}, {}
    u = np.empty_like(w.sparse)
    for b in range(w.nblocks):
        a, c = int(w.node_off[b]), int(w.node_off[b + 1])
        x = w.n2i[a:c].astype(np.float64) / (1 << int(w.blocks[b, 3])) + w.blocks[b, :3]
        u[a:c] = (0.25 * x[:, 0] + 0.2 * x[:, 1] + 0.1 * x[:, 2]).astype(np.float32)
    texs, texs2 = {}, {}
    for b in range(w.nblocks):
        n2i, sp = w.block_nodes(b)
        d = int(w.blocks[b, 3])
        dn = to_device_n2i(n2i)
        dense[b] = ctx.interp_dense(dn, torch.from_numpy(np.ascontiguousarray(sp)).cuda(), d)
        a, c = int(w.node_off[b]), int(w.node_off[b + 1])
        dense2[b] = ctx.interp_dense(dn, torch.from_numpy(np.ascontiguousarray(u[a:c])).cuda(), d)
        # the same fields as textures (the reference keeps a block's field in a texture)
        texs[b], texs2[b] = ctx.texture(d), ctx.texture(d)
        texs[b].fill(dense[b])
        texs2[b].fill(dense2[b])
    tf_tex = ctx.tf_texture(tf)
    refcu = None
    if with_reference:
        try:
            from oracle import refcu as _r
            if _r.available():
                refcu = _r
                refcu.set_tf(np.ascontiguousarray(w.tf, np.float32))
        except Exception:
            refcu = None
    out = {"workload": "cfg2: 4x4x4 blocks of depth 6 (17.6 M dense vertices), 1920x1080, 64 render launches "
                       "back to front, interpolation excluded; ms: s3r_render_block_texture (fields and transfer "
                       "function in textures, sampled by the texture unit as the reference samples), the 64 launches "
                       "replayed from one CUDA graph, as reference_kernels_ms times the reference's renderKernel<mode> "
                       "(per_launch_events: an event pair around each launch, host overhead included); "
                       "ms_software_texture_filter / ms_exact_filter: s3r_render_block on linear bricks; batched_ms: "
                       "the whole frame in one s3r_frame_render_mode launch (exact filter, FP32 compositing) on "
                       "resident bricks"}
    from revise_gb300.api import FramePlan
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=16)
    plan.interp(torch.from_numpy(w.sparse).cuda())
    plan2 = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=16)
    plan2.interp(torch.from_numpy(np.ascontiguousarray(u)).cuda())
    bricks2, _ = plan2.bricks()
    frame_img = torch.zeros(w.W * w.H * 4, device="cuda")
    span = w.field_max - w.field_min
    for mode, name in MODE_NAMES.items():
        view = host.view_for(w, filter=_lib.FILTER_TEXTURE)
        rel = lambda r: float(np.float32(w.field_min + r * span))  # noqa: E731
        if mode in (_lib.MODE_ISOSURFACE, _lib.MODE_VALUE_ON_ISOSURFACE):
            view.threshold = rel(0.45)
        elif mode in (_lib.MODE_ISOSURFACES, _lib.MODE_VALUE_ON_ISOSURFACES):
            view.threshold = 0.0
        levels = [rel(x) for x in (0.2, 0.35, 0.5, 0.65, 0.8)] if mode in (
            _lib.MODE_ISOSURFACES, _lib.MODE_VALUE_ON_ISOSURFACES) else []
        two = mode in (_lib.MODE_VALUE_ON_ISOSURFACE, _lib.MODE_VALUE_ON_ISOSURFACES)
        pres = host.presentation(mode, view, isosurface_opacity=0.6, levels=levels,
                                 secondary_range=(0.0, 1.1) if two else (0.0, 1.0))
        clear = 0x7FC00000 if mode == _lib.MODE_MAX_INTENSITY else 0
        rects = np.array([host.block_view_rect(view, w.blocks[b, :3]) for b in range(w.nblocks)], np.int32)
        vp = torch.full((w.W * w.H,), clear, dtype=torch.int64, device="cuda").to(torch.int32)

        def frame():
            evs = []
            for b in oi:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                ctx.render_block(view, pres, dense[b], int(w.blocks[b, 3]), [int(x) for x in w.blocks[b, :3]],
                                 rects[b], tf, vp, brick2=dense2[b] if two else None)
                e1.record()
                evs.append((e0, e1))
            torch.cuda.synchronize()
            return sum(x.elapsed_time(y) for x, y in evs)

        frame()
        ours_sw = statistics.median([frame() for _ in range(3)])

        def frame_tex():
            evs = []
            for b in oi:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                ctx.render_block_texture(view, pres, texs[b], [int(x) for x in w.blocks[b, :3]], rects[b], tf_tex, vp,
                                         tex2=texs2[b] if two else None)
                e1.record()
                evs.append((e0, e1))
            torch.cuda.synchronize()
            return sum(x.elapsed_time(y) for x, y in evs)

        frame_tex()
        ours_events = statistics.median([frame_tex() for _ in range(3)])
        # the same 64 launches back to back from one captured CUDA graph (no host overhead between launches),
        # as the reference's kernels are timed below
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            for b in oi:
                ctx.render_block_texture(view, pres, texs[b], [int(x) for x in w.blocks[b, :3]], rects[b], tf_tex, vp,
                                         tex2=texs2[b] if two else None, stream=side)
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        ours = e0.elapsed_time(e1) / 5
        del g
        view.filter = _lib.FILTER_EXACT
        frame()
        ours_exact = statistics.median([frame() for _ in range(3)])
        bview = host.view_for(w, filter=_lib.FILTER_EXACT)
        bview.threshold = view.threshold

        def batched():
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            plan.render_mode(bview, pres, tf, bricks2 if two else None, frame_img)
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)

        batched()
        bms = statistics.median([batched() for _ in range(5)])
        view.filter = _lib.FILTER_TEXTURE
        rec = {"ms": ours, "ms_per_launch_events": ours_events, "ms_software_texture_filter": ours_sw,
               "ms_exact_filter": ours_exact, "batched_ms": bms}
        if refcu is not None:
            try:
                rms = refcu.time_render_graph(view, pres, w, oi, rects, u if two else None)
                rms_ev = statistics.median([refcu.time_render(view, pres, w, oi, rects, u if two else None, clear)[0]
                                            for _ in range(3)])
                rec.update({"reference_kernels_ms": rms, "reference_kernels_ms_per_launch_events": rms_ev,
                            "speedup": rms / ours, "speedup_batched": rms / bms})
            except Exception as e:
                rec["reference_kernels"] = f"unavailable: {type(e).__name__}: {e}"
        out[name] = rec
    plan.close()
    plan2.close()
    return out


def event_ms(torch, fn, k=10):
    """Mean ms of fn over k runs after 3 warm-up runs, CUDA events on the current stream."""
    for _ in range(3):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(k):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / k


def measure_adjoint(ctx, torch, np):
    """Forward render and adjoint (backward) times on the 8-block differentiation config (cfg5)."""
    from revise_gb300 import host, workloads
    from revise_gb300.api import FramePlan
    w = workloads.cfg5()
    view = host.view_for(w)
    plan = FramePlan(ctx, w)
    sp = torch.from_numpy(w.sparse).cuda()
    tf = torch.from_numpy(np.ascontiguousarray(w.tf)).cuda()
    rgba = torch.zeros(w.W * w.H * 4, device="cuda")
    plan.autotune(view, sp, tf, reps=3)  # the forward is the fastest render form for this view
    plan.interp(sp)
    dl = torch.rand_like(rgba) * 0.01
    dtf = torch.zeros(w.tf.size, device="cuda")
    bricks, _ = plan.bricks()
    dd = torch.zeros(bricks.numel(), device="cuda")

    fwd = event_ms(torch, lambda: plan.render(view, tf, rgba))
    bwd = event_ms(torch, lambda: plan.backward(view, tf, rgba, dl, dtf, dd))
    rt = int(plan.info.render_tile)
    plan.close()
    return {"workload": "cfg5: 2x2x2 blocks depth 6, 512x512", "forward_render_ms": fwd, "backward_ms": bwd,
            "adjoint_forward_ratio": bwd / fwd, "forward_render_tile": rt}


def measure_worker_loop(ctx, torch, np, w):
    """The per-block drop-in path over the whole frame: s3r_render_scene_part (the native
    VsWorker_cu::renderScenePart) on the full block cube as one index box, texture filter as the
    reference samples -- per block interpolation from resident nodes and render, back to front --
    wall time per frame including the bounding-rectangle read back."""
    import time
    from revise_gb300 import _lib
    from revise_gb300.api import RenderSharedState, VsWorker
    st = RenderSharedState(w, filter=_lib.FILTER_TEXTURE)
    wk = VsWorker(ctx)
    wk.set_render_shared_state(st)
    m = 1 << w.level
    wk.render_scene_part_native(w.level, (0, 0, 0), (m, m, m))
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        t = time.perf_counter()
        wk.render_scene_part_native(w.level, (0, 0, 0), (m, m, m))
        torch.cuda.synchronize()
        ts.append((time.perf_counter() - t) * 1e3)
    launches0 = ctx.launches
    wk.render_scene_part_native(w.level, (0, 0, 0), (m, m, m))
    launches = int(ctx.launches - launches0)
    # the same loop rendering from the batched plan's bricks: one interpolation launch per frame
    from revise_gb300.api import FramePlan
    plan = FramePlan(ctx, w, _lib.BRICK_F32, tile_cells=16)
    sparse = torch.from_numpy(w.sparse).cuda()

    def planned():
        plan.interp(sparse)
        wk.render_scene_part_plan(plan, w.level, (0, 0, 0), (m, m, m))

    planned()
    torch.cuda.synchronize()
    tp = []
    for _ in range(3):
        t = time.perf_counter()
        planned()
        torch.cuda.synchronize()
        tp.append((time.perf_counter() - t) * 1e3)
    plan.close()
    return {"workload": f"{w.name}: {w.nblocks} blocks as one box, {w.W}x{w.H}, Argb, texture filter, nodes resident",
            "ms_per_frame": statistics.median(ts), "launches_per_frame": launches,
            "from_plan_bricks_ms_per_frame": statistics.median(tp)}


def measure_extras(ctx, torch, np):
    """Adjoint/forward ratio on the 8-block differentiation config and 16-bit-brick frame rates (cfg2)."""
    from revise_gb300 import _lib, host, workloads
    from revise_gb300.api import FramePlan
    out = {"adjoint": measure_adjoint(ctx, torch, np)}
    w2 = workloads.cfg2()
    v2 = host.view_for(w2)
    sp2 = torch.from_numpy(w2.sparse).cuda()
    tf2 = torch.from_numpy(np.ascontiguousarray(w2.tf)).cuda()
    prec = {}
    imgs = {}
    for name, fmt in (("f32", _lib.BRICK_F32), ("f16", _lib.BRICK_F16), ("bf16", _lib.BRICK_BF16)):
        img = torch.zeros(w2.W * w2.H * 4, device="cuda")
        p = FramePlan(ctx, w2, fmt)
        p.autotune(v2, sp2, tf2, reps=3)
        ms = event_ms(torch, lambda: p.run(v2, sp2, tf2, img))
        imgs[name] = img
        prec[name] = {"ms_per_frame": ms, "frames_per_s": 1e3 / ms, "render_tile": int(p.info.render_tile)}
        p.close()
    for name in ("f16", "bf16"):
        # image error of the 16-bit bricks against the FP32-brick image of the same frame (RGBA, per channel);
        # against the FP64 oracle the test suite states it (tests/test_gpu_render.py)
        d = (imgs[name] - imgs["f32"]).abs()
        prec[name].update({"max_abs_err_vs_f32": float(d.max()), "mean_abs_err_vs_f32": float(d.mean()),
                           "frames_per_s_vs_f32": prec["f32"]["ms_per_frame"] / prec[name]["ms_per_frame"]})
    out["precision_cfg2"] = prec
    return out


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    if a.adjoint_only:
        import numpy as np
        import torch
        from revise_gb300.api import Context
        ctx = Context(0)
        print(json.dumps({"adjoint": measure_adjoint(ctx, torch, np)}))
        ctx.close()
        return 0
    return run_gb300(a)


if __name__ == "__main__":
    sys.exit(main())
