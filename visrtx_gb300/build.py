"""In-tree build of libvrtx (CUDA kernels + C ABI) for sm_103a.

The library is a plain shared object with a C ABI (include/vrtx.h); it has
no Python or torch dependency. Translation units compile in parallel:
nvcc for the .cu files, g++ for the host object layer, then one nvcc link.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libvrtx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["bvh.cu", "radix_sort.cu", "scene.cu", "render.cu", "render_counting.cu", "render_volume.cu", "render_ao.cu",
              "dm.cu"]
CPP_SOURCES = ["device.cpp", "anari_shim.cpp"]
# Translation units whose arithmetic decides ids, depth and colour: compiled
# without implicit multiply-add contraction, so every operation rounds as
# written (the CPU oracle is built the same way, -ffp-contract=off); fused
# multiply-adds there are explicit fmaf calls. The differentiable marcher
# (dm.cu) is built the same way so that its forward kernel, its adjoint's
# recomputation and the fused training step round every sample alike.
NO_FMAD = {"render.cu", "render_counting.cu", "render_volume.cu", "render_ao.cu", "scene.cu",
           "dm.cu"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libvrtx needs the CUDA toolkit to build")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, defines: tuple = (),
          lib_path: str | None = None, obj_dir: str | None = None) -> str:
    """Builds visrtx_gb300/lib/libvrtx.so if any source changed; returns its
    path. `defines` (e.g. ("VRTX_RENDER_MIN_BLOCKS=4",)) and a separate
    lib_path/obj_dir build a tuning variant beside the default library."""
    global OBJ, LIB
    saved = (OBJ, LIB)
    if lib_path:
        LIB = lib_path
        OBJ = obj_dir or os.path.join(os.path.dirname(lib_path), "_obj")
    try:
        return _build(verbose, ptxas_info, [f"-D{d}" for d in defines])
    finally:
        OBJ, LIB = saved


def _build(verbose: bool, ptxas_info: bool, dflags: list) -> str:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "vrtx.h"))
    headers.append(os.path.join(ROOT, "include", "anari_visrtx.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
                   "--extended-lambda", "-Xcompiler", "-fPIC", *dflags, "-c", s, "-o", o]
            if src in NO_FMAD:
                cmd.insert(1, "-fmad=false")
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         "-fvisibility=hidden", "-I", os.path.join(cuda, "include"),
                         "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="build libvrtx.so (sm_103a)")
    ap.add_argument("--ptxas", action="store_true", help="print ptxas register / spill info")
    ap.add_argument("--define", action="append", default=[],
                    help="NAME=VALUE for a tuning macro (e.g. VRTX_AO_LEAF_TURN=0); needs --lib")
    ap.add_argument("--lib", default=None, help="output path of a tuning variant")
    a = ap.parse_args()
    if a.define and not a.lib:
        ap.error("--define builds a variant: give its --lib path")
    obj = os.path.join(os.path.dirname(os.path.abspath(a.lib)), "_obj") if a.lib else None
    build(verbose=True, ptxas_info=a.ptxas, defines=tuple(a.define),
          lib_path=os.path.abspath(a.lib) if a.lib else None, obj_dir=obj)
