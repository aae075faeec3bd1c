"""ctypes binding of libvrtx's C ABI (include/vrtx.h).

Loading fails loudly when the shared library is missing: there is no CPU or
Python fallback for anything this package computes.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libvrtx.so")

# VRTXDataType codes (include/vrtx.h)
UNKNOWN = 0
STRING = 1
VOID_POINTER = 2
BOOL = 3
FUNCTION_POINTER = 4
STRING_LIST = 6
OBJECT = 100
ARRAY1D, ARRAY2D, ARRAY3D = 101, 102, 103
CAMERA, FRAME, GEOMETRY, GROUP, INSTANCE, LIGHT, MATERIAL, RENDERER = range(104, 112)
SURFACE, SAMPLER, SPATIAL_FIELD, VOLUME, WORLD = range(112, 117)
DEVICE = 117
INT32, INT32_VEC2, INT8, UINT8 = 200, 201, 202, 203
UINT32, UINT32_VEC2, UINT32_VEC3, UINT32_VEC4 = 210, 211, 212, 213
UINT64 = 214
FIXED8, UFIXED8, FIXED16, UFIXED16 = 220, 221, 222, 223
FLOAT16, BFLOAT16 = 230, 231
FLOAT32, FLOAT32_VEC2, FLOAT32_VEC3, FLOAT32_VEC4 = 240, 241, 242, 243
FLOAT32_BOX1, FLOAT32_BOX2, FLOAT32_BOX3 = 244, 245, 246
FLOAT32_MAT3x4, FLOAT32_MAT4 = 247, 248
FLOAT64, FLOAT64_BOX1 = 250, 251
UFIXED8_VEC4, UFIXED8_RGBA_SRGB = 260, 261
DATA_TYPE = 270

SEVERITY_FATAL_ERROR, SEVERITY_ERROR, SEVERITY_WARNING = 0, 1, 2
SEVERITY_PERFORMANCE_WARNING, SEVERITY_INFO, SEVERITY_DEBUG = 3, 4, 5
NO_WAIT, WAIT = 0, 1

STATUS_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                        C.c_int, C.c_int, C.c_char_p)
DELETER = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)

# every exported entry point with (restype, argtypes)
SIGNATURES = {
    "vrtxNewDevice": (C.c_void_p, [STATUS_CB, C.c_void_p]),
    "vrtxDeviceSetParameter": (None, [C.c_void_p, C.c_char_p, C.c_int, C.c_void_p]),
    "vrtxDeviceCommitParameters": (None, [C.c_void_p]),
    "vrtxDeviceRelease": (None, [C.c_void_p]),
    "vrtxDeviceGetProperty": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_void_p,
                                        C.c_uint64, C.c_uint32]),
    "vrtxDeviceIsValid": (C.c_int, [C.c_void_p]),
    "vrtxGetObjectSubtypes": (C.POINTER(C.c_char_p), [C.c_void_p, C.c_int]),
    "vrtxGetObjectExtensions": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_char_p]),
    "vrtxGetInstanceExtensions": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "vrtxNewArray1D": (C.c_void_p, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_uint64]),
    "vrtxNewArray2D": (C.c_void_p, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_uint64, C.c_uint64]),
    "vrtxNewArray3D": (C.c_void_p, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_uint64, C.c_uint64, C.c_uint64]),
    "vrtxMapArray": (C.c_void_p, [C.c_void_p, C.c_void_p]),
    "vrtxUnmapArray": (None, [C.c_void_p, C.c_void_p]),
    "vrtxNewCamera": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewGeometry": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewLight": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewMaterial": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewRenderer": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewSampler": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewSpatialField": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewVolume": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewSurface": (C.c_void_p, [C.c_void_p]),
    "vrtxNewGroup": (C.c_void_p, [C.c_void_p]),
    "vrtxNewInstance": (C.c_void_p, [C.c_void_p, C.c_char_p]),
    "vrtxNewWorld": (C.c_void_p, [C.c_void_p]),
    "vrtxNewFrame": (C.c_void_p, [C.c_void_p]),
    "vrtxSetParameter": (None, [C.c_void_p, C.c_void_p, C.c_char_p, C.c_int, C.c_void_p]),
    "vrtxUnsetParameter": (None, [C.c_void_p, C.c_void_p, C.c_char_p]),
    "vrtxUnsetAllParameters": (None, [C.c_void_p, C.c_void_p]),
    "vrtxCommitParameters": (None, [C.c_void_p, C.c_void_p]),
    "vrtxRelease": (None, [C.c_void_p, C.c_void_p]),
    "vrtxRetain": (None, [C.c_void_p, C.c_void_p]),
    "vrtxGetProperty": (C.c_int, [C.c_void_p, C.c_void_p, C.c_char_p, C.c_int,
                                  C.c_void_p, C.c_uint64, C.c_uint32]),
    "vrtxRenderFrame": (None, [C.c_void_p, C.c_void_p]),
    "vrtxFrameReady": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vrtxDiscardFrame": (None, [C.c_void_p, C.c_void_p]),
    "vrtxMapFrame": (C.c_void_p, [C.c_void_p, C.c_void_p, C.c_char_p,
                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_int)]),
    "vrtxUnmapFrame": (None, [C.c_void_p, C.c_void_p, C.c_char_p]),
    "vrtxDebugCopyAccel": (C.c_uint64, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                        C.c_uint64]),
    "vrtxWorldBuildMilliseconds": (C.c_float, [C.c_void_p, C.c_void_p]),
    "vrtxDebugDiscretizeTF": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                        C.c_float, C.c_float, C.c_void_p, C.c_float,
                                        C.c_void_p]),
    "vrtxDebugWriteColors": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_int,
                                       C.c_void_p]),
    "vrtxDebugStageImage": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_uint64, C.c_void_p,
                                      C.c_void_p]),
    "vrtxDebugRadixSort": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int]),
    "vrtxFrameKernelMilliseconds": (C.c_float, [C.c_void_p, C.c_void_p]),
    "vrtxFrameKernelLaunches": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vrtxDeviceStream": (C.c_void_p, [C.c_void_p]),
    "vrtxDMForward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "vrtxDMBackward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                 C.c_void_p]),
    "vrtxDMPlanCreate": (C.c_void_p, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                      C.c_int, C.c_int, C.c_void_p]),
    "vrtxDMPlanForward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vrtxDMPlanBackward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vrtxDMPlanStepL2": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "vrtxDMPlanSetLaunch": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "vrtxDMPlanRelease": (None, [C.c_void_p]),
    "vrtxDMForwardNoAlloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
}


DM_PLAIN = 1  # VRTX_DM_PLAIN


class VRTXExtensions(C.Structure):
    """The extension flags of include/vrtx.h (one int per feature)."""
    _fields_ = [(n, C.c_int) for n in (
        "VISRTX_ARRAY_CUDA", "VISRTX_CUDA_OUTPUT_BUFFERS", "VISRTX_INSTANCE_ATTRIBUTES",
        "VISRTX_MATERIAL_MDL", "VISRTX_SPATIAL_FIELD_NANOVDB",
        "VISRTX_TRIANGLE_BACK_FACE_CULLING", "VISRTX_TRIANGLE_FACE_VARYING_ATTRIBUTES")]

    def as_dict(self) -> dict[str, bool]:
        return {n: bool(getattr(self, n)) for n, _ in self._fields_}


class VRTXDMVolume(C.Structure):
    _fields_ = [
        ("density", C.c_void_p), ("densityType", C.c_int), ("dims", C.c_int * 3),
        ("tf", C.c_void_p), ("tfSize", C.c_int), ("opacityScale", C.c_float),
        ("step", C.c_float), ("unitDistance", C.c_float), ("valueLo", C.c_float),
        ("valueHi", C.c_float), ("gradDensity", C.c_void_p), ("gradTf", C.c_void_p),
        ("gradOpacityScale", C.c_void_p), ("opacityScaleDevice", C.c_void_p),
        ("flags", C.c_int), ("tfType", C.c_int),
    ]


class VRTXDMView(C.Structure):
    _fields_ = [
        ("volume", C.c_int), ("width", C.c_int), ("height", C.c_int),
        ("eye", C.c_float * 3), ("d00", C.c_float * 3), ("du", C.c_float * 3),
        ("dv", C.c_float * 3), ("background", C.c_float * 3), ("pixelOffset", C.c_int64),
    ]


_lib = None
_lib_path = None
_lock = threading.Lock()


def load(path: str | None = None) -> C.CDLL:
    """Loads libvrtx.so (built by visrtx_gb300.build) and declares its ABI."""
    global _lib, _lib_path
    with _lock:
        p = os.path.realpath(path or LIB_PATH)
        if _lib is not None:
            if path is not None and p != _lib_path:
                raise RuntimeError(f"libvrtx is already loaded from {_lib_path}; "
                                   f"one process loads one library (asked for {p})")
            return _lib
        if not os.path.exists(p):
            raise RuntimeError(
                f"libvrtx.so not found at {p}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` "
                "(there is no CPU fallback)")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        _lib_path = p
        return lib
