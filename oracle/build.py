"""Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so,
and, where the reference tree is present, oracle/_ref/libnvdbref.so.

The reference's renderer cannot be compiled here (its device path needs
OptiX headers fetched at configure time and the ANARI-SDK, neither present);
see oracle.h for the parity status. Two parts of it do compile with g++
alone, from the headers where they lie under the reference tree, with the
output only in oracle/_ref/:
  * the NanoVDB library it vendors (external/nanovdb, header-only):
    ref_nvdb.cpp drives its grid builder, sampler and validator
    (libnvdbref.so);
  * its transfer-function helpers (devices/rtx/utility/colorMapHelpers.h
    with gpu/gpu_math.h and the vendored glm): ref_tf.cpp repeats
    TransferFunction1D::discritizeTFData's calls, runs gpu_math.h's and
    uniformGrid.h's sampling and grid helpers, and repeats
    intersectVolume's glm calls (libtfref.so);
  * the vendored glm's colour packing (glm::convertLinearToSRGB,
    glm::packUnorm4x8): ref_glm.cpp repeats writeOutputColor's calls
    (libglmref.so);
  * its macrocell walk (devices/rtx/gpu/dda.h, dda3): ref_dda.cpp runs it
    (libddaref.so), with floating-point contraction on, as nvcc builds the
    reference's device code (-fmad=true): -ffp-contract=fast, with -mfma
    on x86-64, where the fused multiply-add is not in the base instruction
    set;
  * its primary-ray generation (devices/rtx/gpu/cameraCreateRay.h):
    ref_camera.cpp runs it without contraction (libcamref.so, each
    operation rounded once, as the oracle and the library's kernels round
    it) and with it (libcamref_fused.so, to size the gap).
  * its structured-field sampler (devices/rtx/gpu/sampleSpatialField.h):
    ref_field.cpp records the texture coordinate it fetches at
    (libfieldref.so);
  * its image staging (devices/rtx/utility/CudaImageTexture.cpp,
    convertComponentUint8 / Float and transformToStagingBuffer*):
    ref_image.cpp includes that .cpp (its staging functions are
    file-local) and runs them (libimgref.so, linked to the CUDA runtime
    for the .cpp's array and texture calls, which it never makes).
  Those headers include the OptiX-bound gpu_objects.h, and the .cpp its
  helium-bound CudaImageTexture.h, so these are compiled through
  oracle/_ref/gpu_inc/{gpu,utility}/, links to the reference's files beside
  links to the stand-ins oracle/ref_shim/gpu_objects.h and
  CudaImageTexture.h, made for the compile and removed after it;
  oracle/ref_shim/anari/anari.h names the ANARI data types.
The GPU machine has no reference tree and never builds them.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")


def build() -> str:
    src = [os.path.join(HERE, "oracle.cpp")]
    hdr = [os.path.join(HERE, "oracle.h")]
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(f) for f in src + hdr):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-o", tmp, *src, "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


# The VisRTX source tree: VISRTX_REFERENCE_TREE, or build_ref(tree=...);
# the default is where this recipe's build machine mounts it.
REF_TREE = os.environ.get("VISRTX_REFERENCE_TREE", "/root/reference")
REF_OUT = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_OUT, "libnvdbref.so")
REF_TF_LIB = os.path.join(REF_OUT, "libtfref.so")
REF_GLM_LIB = os.path.join(REF_OUT, "libglmref.so")
REF_DDA_LIB = os.path.join(REF_OUT, "libddaref.so")
REF_CAM_LIB = os.path.join(REF_OUT, "libcamref.so")
REF_CAM_FUSED_LIB = os.path.join(REF_OUT, "libcamref_fused.so")
REF_IMG_LIB = os.path.join(REF_OUT, "libimgref.so")
REF_FIELD_LIB = os.path.join(REF_OUT, "libfieldref.so")
GPU_HEADERS = ("dda.h", "gpu_debug.h", "gpu_math.h", "gpu_decl.h", "uniformGrid.h",
               "cameraCreateRay.h", "sampleSpatialField.h")
UTILITY_FILES = ("CudaImageTexture.cpp", "AnariTypeHelpers.h")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _compile_ref(src: str, out: str, incs: list[str], contract: str = "off",
                 deps: tuple[str, ...] = (), libs: tuple[str, ...] = ()) -> str:
    os.makedirs(REF_OUT, exist_ok=True)
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(f)
                                   for f in (src, *deps)):
        return out
    tmp = out + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-ffp-contract={contract}"]
    if contract == "fast" and platform.machine().lower() in ("x86_64", "amd64"):
        cmd.append("-mfma")
    for i in incs:
        cmd += ["-I", i]
    cmd += ["-o", tmp, src, *libs, "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle/_ref build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, out)
    return out


def build_ref(tree: str | None = None) -> str | None:
    """oracle/_ref/libnvdbref.so (ref_nvdb.cpp over the reference's vendored
    NanoVDB headers), oracle/_ref/libtfref.so (ref_tf.cpp over its
    transfer-function helpers), oracle/_ref/libglmref.so (ref_glm.cpp
    over its vendored glm), oracle/_ref/libddaref.so (ref_dda.cpp over
    its dda.h), oracle/_ref/libcamref{,_fused}.so (ref_camera.cpp over
    its cameraCreateRay.h), oracle/_ref/libfieldref.so (ref_field.cpp over
    its sampleSpatialField.h) and oracle/_ref/libimgref.so (ref_image.cpp
    over its CudaImageTexture.cpp) from the reference tree `tree` (default
    REF_TREE); returns the NanoVDB harness's path, or None when the
    reference tree is absent."""
    root = tree or REF_TREE
    inc = os.path.join(root, "external", "nanovdb", "include")
    if not os.path.isdir(inc):
        return None
    lib = _compile_ref(os.path.join(HERE, "ref_nvdb.cpp"), REF_LIB, [inc])
    rtx = os.path.join(root, "devices", "rtx")
    glm = os.path.join(root, "external", "glm", "include")
    if os.path.isfile(os.path.join(rtx, "utility", "colorMapHelpers.h")) and os.path.isdir(glm):
        _compile_ref(os.path.join(HERE, "ref_tf.cpp"), REF_TF_LIB, [rtx, glm])
        _compile_ref(os.path.join(HERE, "ref_glm.cpp"), REF_GLM_LIB, [glm])
        if all(os.path.isfile(os.path.join(rtx, "gpu", h)) for h in GPU_HEADERS) and all(
                os.path.isfile(os.path.join(rtx, "utility", f)) for f in UTILITY_FILES):
            # the links point into the reference tree: made for the compile
            # only, so that no dangling link is left in oracle/_ref
            inc = _gpu_include_dir(rtx)
            shims = os.path.join(HERE, "ref_shim")
            shim = (os.path.join(shims, "gpu_objects.h"),)
            cam = os.path.join(HERE, "ref_camera.cpp")
            cuda_lib = os.path.join(CUDA_HOME, "lib64")
            try:
                _compile_ref(os.path.join(HERE, "ref_dda.cpp"), REF_DDA_LIB, [inc, glm],
                             contract="fast", deps=shim)
                _compile_ref(cam, REF_CAM_LIB, [inc, glm], contract="off", deps=shim)
                _compile_ref(cam, REF_CAM_FUSED_LIB, [inc, glm], contract="fast", deps=shim)
                if os.path.isdir(os.path.join(CUDA_HOME, "include")):
                    nvdb = os.path.join(root, "external", "nanovdb", "include")
                    _compile_ref(os.path.join(HERE, "ref_field.cpp"), REF_FIELD_LIB,
                                 [inc, nvdb, glm, os.path.join(CUDA_HOME, "include")],
                                 deps=shim)
                    _compile_ref(os.path.join(HERE, "ref_image.cpp"), REF_IMG_LIB,
                                 [inc, shims, glm, os.path.join(CUDA_HOME, "include")],
                                 deps=(os.path.join(shims, "CudaImageTexture.h"),
                                       os.path.join(shims, "anari", "anari.h")),
                                 libs=(f"-L{cuda_lib}", f"-Wl,-rpath,{cuda_lib}", "-lcudart"))
            finally:
                shutil.rmtree(inc, ignore_errors=True)
    return lib


def _gpu_include_dir(rtx: str) -> str:
    """oracle/_ref/gpu_inc: gpu/ holds links to the reference's dda.h and
    cameraCreateRay.h, the headers they include, and
    oracle/ref_shim/gpu_objects.h; utility/ links to its
    CudaImageTexture.cpp and AnariTypeHelpers.h and to
    oracle/ref_shim/CudaImageTexture.h: their own-directory includes find
    the stand-ins."""
    inc = os.path.join(REF_OUT, "gpu_inc")
    shims = os.path.join(HERE, "ref_shim")
    links = {os.path.join("gpu", h): os.path.join(rtx, "gpu", h) for h in GPU_HEADERS}
    links[os.path.join("gpu", "gpu_objects.h")] = os.path.join(shims, "gpu_objects.h")
    for f in UTILITY_FILES:
        links[os.path.join("utility", f)] = os.path.join(rtx, "utility", f)
    links[os.path.join("utility", "CudaImageTexture.h")] = os.path.join(
        shims, "CudaImageTexture.h")
    for name, target in links.items():
        p = os.path.join(inc, name)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        if os.path.lexists(p):
            os.remove(p)
        os.symlink(target, p)
    return inc


if __name__ == "__main__":
    import sys

    print(build())
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None))
