"""Builds the s3r shared library (sm_103a CUDA kernels + C ABI host code) in-tree.

    python -m revise_gb300.build            # library -> revise_gb300/libs3r.so
    python -m revise_gb300.build --oracle   # also the test oracle (oracle/_build, oracle/_ref)

Each CUDA translation unit is compiled separately and in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the host side is compiled with
g++ -ffp-contract=off; everything links into one shared library with the CUDA
runtime linked statically.  No cmake.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libs3r.so"
INCLUDE = ROOT / "include"

CUDA_SOURCES = ["interp.cu", "render.cu", "compose.cu", "noalloc.cu", "propagate.cu"]
HOST_SOURCES = ["host.cpp", "dataset.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    if os.environ.get("S3R_BUILD_VERBOSE") and proc.stdout.strip():
        print(proc.stdout)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, ptxas_verbose: bool = False) -> Path:
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    headers = [INCLUDE / "s3r.h", CSRC / "s3r_internal.h", CSRC / "interp_tile.cuh"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE),
                   "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(obj)]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for src in HOST_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(cuda / "include"),
                         "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
              "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    return LIB


def build_oracle(reference: str | None = None) -> None:
    """The checkers under oracle/: the C restatement always; the reference's own code from the staged
    tree oracle/_ref/tree (staged first when the reference project root is given, as `reference` or in the
    REFERENCE environment variable)."""
    oracle = ROOT / "oracle"
    _run(["make", "-s", "-C", str(oracle), "port"])
    ref = reference or os.environ.get("REFERENCE")
    if ref:
        _run(["make", "-s", "-C", str(oracle), "stage", f"REFERENCE={ref}"])
    if (oracle / "_ref" / "tree" / "include" / "s3dmm" / "DenseFieldInterpolator.hpp").exists():
        _run(["make", "-s", "-C", str(oracle), "ref", "refcu", "refsetup", f"NVCC={cuda_home() / 'bin' / 'nvcc'}"])
    # the harness around the reference's CUDA kernels builds anywhere the cubins exist
    if (oracle / "_ref" / "ref_render.cubin").exists() and (oracle / "_ref" / "ref_interp.cubin").exists():
        _run(["make", "-s", "-C", str(oracle), "refcu-harness", f"NVCC={cuda_home() / 'bin' / 'nvcc'}"])


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--oracle", action="store_true")
    ap.add_argument("--ptxas-verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build_library(force=a.force, ptxas_verbose=a.ptxas_verbose))
    if a.oracle:
        build_oracle()
    return 0


if __name__ == "__main__":
    sys.exit(main())
