"""CPU checks of the C ABI: the library loads, exports every entry point
include/vrtx.h declares, and reports errors (no crash, null handles) when
there is no CUDA device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        names += re.findall(r"VRTX_API\s+[\w\s\*]+?\b(vrtx\w+)\s*\(", src)
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "vrtxNewDevice" in names and "vrtxRenderFrame" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol(built):
    from visrtx_gb300 import _lib

    lib = _lib.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the same set
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_no_gpu_reports_and_returns_null(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from visrtx_gb300 import anari

    dev = anari.Device(0)
    assert not dev.is_valid()
    assert any("no CUDA device" in m for m in dev.errors())
    h = dev.lib.vrtxNewGeometry(dev.h, b"triangle")
    assert not h
    # frame calls on null handles are no-ops
    dev.lib.vrtxRenderFrame(dev.h, None)
    w, hh, t = C.c_uint32(7), C.c_uint32(7), C.c_int(7)
    p = dev.lib.vrtxMapFrame(dev.h, None, b"channel.color", C.byref(w), C.byref(hh), C.byref(t))
    assert not p and w.value == 0 and hh.value == 0 and t.value == 0
    dev.release()


def test_dm_rejects_invalid_arguments(built):
    """Argument validation of the differentiable marcher happens on the host
    before any launch."""
    from visrtx_gb300 import _lib, anari

    dev = anari.Device(0)
    vol = _lib.VRTXDMVolume()
    view = _lib.VRTXDMView()
    rc = dev.lib.vrtxDMForward(dev.h, C.byref(vol), 1, C.byref(view), 1, None, None, 16, 8, None)
    assert rc < 0
    rc = dev.lib.vrtxDMForward(dev.h, C.byref(vol), 0, C.byref(view), 1, C.c_void_p(8),
                               C.c_void_p(8), 16, 8, None)
    assert rc < 0
    assert dev.errors()
    # plan entry points without a plan refuse before touching a device
    assert dev.lib.vrtxDMPlanStepL2(None, C.c_void_p(8), 1.0, None, None, None) == -1
    assert dev.lib.vrtxDMPlanForward(None, C.c_void_p(8), C.c_void_p(8), None) == -1
    assert dev.lib.vrtxDMPlanSetLaunch(None, 0, 1) == -1
    dev.release()


def test_feature_queries(built):
    """Subtype lists, the device's extension list and the extension flags of
    VisRTXFeatureUtility.cpp: host-only queries, answered without a GPU."""
    from visrtx_gb300 import _lib as L
    from visrtx_gb300 import anari

    dev = anari.Device(0)
    ext = dev.extensions()
    assert "ANARI_KHR_SPATIAL_FIELD_NANOVDB" in ext and "ANARI_NV_ARRAY_CUDA" in ext
    assert "ANARI_KHR_GEOMETRY_CURVE" in ext and len(ext) == len(set(ext))
    assert dev.object_subtypes(L.GEOMETRY) == ["triangle", "quad", "sphere", "cylinder",
                                               "cone", "curve"]
    assert "nanovdb" in dev.object_subtypes(L.SPATIAL_FIELD)
    assert "physicallyBased" in dev.object_subtypes(L.MATERIAL)
    assert dev.object_subtypes(L.SURFACE) == [] and dev.object_subtypes(12345) == []
    flags = dev.instance_extensions()
    assert flags["VISRTX_ARRAY_CUDA"] and flags["VISRTX_CUDA_OUTPUT_BUFFERS"]
    assert flags["VISRTX_SPATIAL_FIELD_NANOVDB"] and flags["VISRTX_TRIANGLE_BACK_FACE_CULLING"]
    assert not flags["VISRTX_MATERIAL_MDL"] and not flags["VISRTX_INSTANCE_ATTRIBUTES"]
    assert not flags["VISRTX_TRIANGLE_FACE_VARYING_ATTRIBUTES"]
    tri = dev.object_extensions(L.GEOMETRY, "triangle")
    assert tri["VISRTX_TRIANGLE_BACK_FACE_CULLING"] and not tri["VISRTX_ARRAY_CUDA"]
    assert dev.object_extensions(L.SPATIAL_FIELD, "nanovdb")["VISRTX_SPATIAL_FIELD_NANOVDB"]
    assert not any(dev.object_extensions(L.GEOMETRY, "sphere").values())
    assert dev.object_extensions(L.GEOMETRY, "neural") is None
    assert dev.object_extensions(L.DEVICE, "") == flags
    # the reference reads the property of the object it is given: only the
    # device carries one
    e = L.VRTXExtensions()
    assert dev.lib.vrtxGetInstanceExtensions(C.byref(e), dev.h, C.c_void_p(1)) == 0
    dev.release()


def test_binding_arity_matches_header():
    """Every ctypes signature takes as many arguments as the header's
    declaration, so a binding cannot drift from the ABI unnoticed."""
    from visrtx_gb300 import _lib

    decls = {}
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            for name, params in re.findall(r"VRTX_API\s+[\w\s\*]+?\b(vrtx\w+)\s*\(([^)]*)\)\s*;",
                                           src):
                p = params.strip()
                decls[name] = 0 if p in ("", "void") else p.count(",") + 1
    assert decls and set(decls) <= set(_lib.SIGNATURES)
    wrong = {n: (k, len(_lib.SIGNATURES[n][1])) for n, k in decls.items()
             if len(_lib.SIGNATURES[n][1]) != k}
    assert not wrong, wrong


def test_cuda_device_change_after_init_is_ignored(built):
    """The GPU is chosen once, when the device initialises; a later
    'cudaDevice' is reported as a warning and ignored
    (VisRTXDevice.cpp:464-470), so objects never move off the GPU that owns
    their memory."""
    from visrtx_gb300 import _lib as L
    from visrtx_gb300 import anari

    dev = anari.Device(0)
    dev.lib.vrtxNewWorld(dev.h)  # initialises (or fails to, without a GPU)
    before = len(dev.messages)
    v = C.c_int32(1)
    dev.lib.vrtxDeviceSetParameter(dev.h, b"cudaDevice", L.INT32, C.byref(v))
    dev.lib.vrtxDeviceCommitParameters(dev.h)
    new = dev.messages[before:]
    assert any(s == L.SEVERITY_WARNING and "is ignored" in m for s, m in new), new
    dev.release()


def test_force_init_initialises_at_commit(built):
    """'forceInit' makes the device initialise at commit rather than at the
    first object creation (VisRTXDevice.cpp:473-476)."""
    import torch

    from visrtx_gb300 import _lib as L
    from visrtx_gb300 import anari

    dev = anari.Device(0)
    assert not dev.messages
    v = C.c_int32(1)
    dev.lib.vrtxDeviceSetParameter(dev.h, b"forceInit", L.BOOL, C.byref(v))
    dev.lib.vrtxDeviceCommitParameters(dev.h)
    if torch.cuda.is_available():
        assert dev.is_valid()
    else:
        assert any("no CUDA device" in m for m in dev.errors())
    dev.release()


def test_library_image_staging_matches_reference(built):
    """The library's image staging (the host code an image sampler and the
    renderer's background image commit with, through vrtxDebugStageImage,
    no GPU involved) equals bit for bit the reference's own
    utility/CudaImageTexture.cpp staging (tests/golden/image_golden.npz),
    including its choice of float or 8-bit texels; unsupported types and
    missing buffers return -1."""
    import numpy as np

    from tests.test_oracle import image_golden_cases
    from visrtx_gb300 import _lib as L

    lib = L.load()
    for name, et, bg, texels, want in image_golden_cases():
        t = np.ascontiguousarray(texels)
        f4 = np.zeros((len(t), 4), np.float32)
        u8 = np.zeros((len(t), 4), np.uint8)
        rc = lib.vrtxDebugStageImage(et, bg, t.ctypes.data, len(t), f4.ctypes.data,
                                     u8.ctypes.data)
        assert rc == (1 if want.dtype == np.float32 else 0), name
        got = f4 if rc == 1 else u8
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), name
    one = np.zeros(4, np.float32)
    assert lib.vrtxDebugStageImage(L.FLOAT64, 0, one.ctypes.data, 1, one.ctypes.data,
                                   None) == -1
    assert lib.vrtxDebugStageImage(L.UFIXED8, 0, one.ctypes.data, 1, one.ctypes.data,
                                   None) == -1
    assert lib.vrtxDebugStageImage(L.UFIXED16, 1, one.ctypes.data, 1, None, None) == -1


def test_library_tf_discretization_matches_reference(built):
    """The library's TF discretisation (the host code a transferFunction1D
    volume commits with, through vrtxDebugDiscretizeTF, no GPU involved)
    equals bit for bit the tables the reference's own helpers computed
    (tests/golden/tf_golden.npz); invalid arguments return -1."""
    import numpy as np

    from tests.test_oracle import tf_golden_cases
    from visrtx_gb300 import _lib as L

    lib = L.load()
    for i, (c, o, vr, uc, uo, ref) in enumerate(tf_golden_cases()):
        out = np.zeros((256, 4), np.float32)
        uc = np.ascontiguousarray(uc, np.float32)
        rc = lib.vrtxDebugDiscretizeTF(
            c.ctypes.data if c is not None else None, 0 if c is None else len(c),
            0 if c is None else c.shape[1], o.ctypes.data if o is not None else None,
            0 if o is None else len(o), vr[0], vr[1], uc.ctypes.data, uo, out.ctypes.data)
        assert rc == 0
        assert np.array_equal(out, ref), (i, float(np.abs(out - ref).max()))
    one = np.ones((1, 3), np.float32)
    out = np.zeros((256, 4), np.float32)
    uc = np.ones(4, np.float32)
    assert lib.vrtxDebugDiscretizeTF(one.ctypes.data, 1, 3, None, 0, 0.0, 1.0, uc.ctypes.data,
                                     1.0, out.ctypes.data) == -1
    assert lib.vrtxDebugDiscretizeTF(None, 0, 0, None, 0, 0.0, 1.0, uc.ctypes.data, 1.0,
                                     None) == -1
