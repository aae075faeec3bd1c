"""The ANARI-facing entry points (include/anari_visrtx.h): the ANARI 1.0 C
API calls and VisRTX's makeVisRTXDevice / visrtxGetObjectExtensions /
visrtxGetInstanceExtensions, driven through ctypes with ANARI type codes
only. On CPU: every declared function is exported, devices without a GPU
report in ANARI codes and hand out null objects, and the feature queries
answer. On a GPU: the plain-traversal workload (a seeded triangle soup, one
directional light, matte, the "default" renderer) built and rendered
through the anari* names alone equals the same scene built through the
library's own calls, bit for bit, and matches the CPU oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "anari_visrtx.h")

STATUS_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                        C.c_char_p)


def _consts():
    src = open(HEADER).read()
    return {k: int(v) for k, v in re.findall(r"#define (ANARI_\w+) (\d+)", src)}


A = _consts()


def _declared():
    src = open(HEADER).read()
    return re.findall(r"ANARI_SHIM_API\s+[\w\s\*]+?\b(\w+)\s*\(", src)


class Anari:
    """ctypes bindings of the shim with the argument types of the header."""

    def __init__(self):
        from visrtx_gb300 import _lib

        self.lib = C.CDLL(_lib.load()._name)
        P, I, U64, S = C.c_void_p, C.c_int, C.c_uint64, C.c_char_p
        sig = {
            "anariLoadLibrary": (P, [S, STATUS_CB, P]), "anariNewDevice": (P, [P, S]),
            "anariGetDeviceSubtypes": (P, [P]), "anariUnloadLibrary": (None, [P]),
            "makeVisRTXDevice": (P, [STATUS_CB, P]),
            "anariNewArray1D": (P, [P, P, P, P, I, U64]),
            "anariNewGeometry": (P, [P, S]), "anariNewMaterial": (P, [P, S]),
            "anariNewSurface": (P, [P]), "anariNewWorld": (P, [P]),
            "anariNewLight": (P, [P, S]), "anariNewCamera": (P, [P, S]),
            "anariNewRenderer": (P, [P, S]), "anariNewFrame": (P, [P]),
            "anariNewObject": (P, [P, S, S]),
            "anariSetParameter": (None, [P, P, S, I, P]),
            "anariCommitParameters": (None, [P, P]), "anariRelease": (None, [P, P]),
            "anariRenderFrame": (None, [P, P]), "anariFrameReady": (I, [P, P, C.c_uint32]),
            "anariMapFrame": (P, [P, P, S, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_int)]),
            "anariUnmapFrame": (None, [P, P, S]),
            "anariGetObjectSubtypes": (P, [P, I]),
            "anariGetProperty": (I, [P, P, S, I, P, U64, C.c_uint32]),
            "anariMapParameterArray1D": (P, [P, P, S, I, U64, C.POINTER(U64)]),
            "anariUnmapParameterArray": (None, [P, P, S]),
            "visrtxGetObjectExtensions": (I, [P, P, I, S]),
        }
        for name, (res, args) in sig.items():
            f = getattr(self.lib, name)
            f.restype = res
            f.argtypes = args
        self.messages = []
        self.cb = STATUS_CB(self._status)

    def _status(self, user, dev, src, src_type, severity, code, msg):
        self.messages.append((src_type, severity, msg.decode(errors="replace") if msg else ""))

    def __getattr__(self, name):
        return getattr(self.lib, name)

    # parameter helpers (ANARI codes)
    def vec(self, dev, obj, name, vals, t):
        arr = (C.c_float * len(vals))(*map(float, vals))
        self.lib.anariSetParameter(dev, obj, name.encode(), t, arr)

    def f32(self, dev, obj, name, v):
        self.lib.anariSetParameter(dev, obj, name.encode(), A["ANARI_FLOAT32"],
                                   C.byref(C.c_float(v)))

    def i32(self, dev, obj, name, v, t="ANARI_INT32"):
        self.lib.anariSetParameter(dev, obj, name.encode(), A[t], C.byref(C.c_int32(v)))

    def obj(self, dev, obj, name, handle, t):
        self.lib.anariSetParameter(dev, obj, name.encode(), A[t], C.byref(C.c_void_p(handle)))

    def string(self, dev, obj, name, v):
        self.lib.anariSetParameter(dev, obj, name.encode(), A["ANARI_STRING"], v.encode())


@pytest.fixture(scope="module")
def shim(built):
    return Anari()


def test_header_functions_are_exported(shim):
    names = _declared()
    assert {"makeVisRTXDevice", "visrtxGetObjectExtensions", "visrtxGetInstanceExtensions",
            "anariNewDevice", "anariRenderFrame", "anariMapFrame"} <= set(names)
    missing = [n for n in names if not hasattr(shim.lib, n)]
    assert not missing, missing


def test_library_device_subtypes_and_feature_queries(shim):
    lib = shim.anariLoadLibrary(b"visrtx", shim.cb, None)
    assert lib
    subs = C.cast(shim.anariGetDeviceSubtypes(lib), C.POINTER(C.c_char_p))
    assert subs[0] == b"visrtx"
    assert not shim.anariLoadLibrary(b"helide", shim.cb, None)
    dev = shim.anariNewDevice(lib, b"default")
    assert dev
    geo = C.cast(shim.anariGetObjectSubtypes(dev, A["ANARI_GEOMETRY"]), C.POINTER(C.c_char_p))
    kinds = []
    i = 0
    while geo[i]:
        kinds.append(geo[i])
        i += 1
    assert b"triangle" in kinds and b"sphere" in kinds
    ext = (C.c_int * 7)()
    assert shim.visrtxGetObjectExtensions(ext, dev, A["ANARI_SPATIAL_FIELD"], b"nanovdb") == 1
    assert ext[4] == 1  # VISRTX_SPATIAL_FIELD_NANOVDB
    shim.anariRelease(dev, dev)
    shim.anariUnloadLibrary(lib)


def test_no_gpu_reports_in_anari_codes(shim):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    shim.messages.clear()
    dev = shim.makeVisRTXDevice(shim.cb, None)
    assert dev
    assert not shim.anariNewGeometry(dev, b"triangle")
    assert any(sev == A["ANARI_SEVERITY_FATAL_ERROR"] and "no CUDA device" in m
               for _, sev, m in shim.messages), shim.messages
    shim.anariRelease(dev, dev)


def _soup_through_anari(shim, spec):
    """Builds and renders the soup spec with anari* calls only; returns the
    mapped channels."""
    dev = shim.makeVisRTXDevice(shim.cb, None)
    keep = []
    s = spec.surfaces[0]
    verts = np.ascontiguousarray(s.vertices, np.float32)
    keep.append(verts)
    va = shim.anariNewArray1D(dev, verts.ctypes.data, None, None, A["ANARI_FLOAT32_VEC3"],
                              len(verts))
    geom = shim.anariNewGeometry(dev, b"triangle")
    shim.obj(dev, geom, "vertex.position", va, "ANARI_ARRAY1D")
    shim.anariCommitParameters(dev, geom)
    mat = shim.anariNewObject(dev, b"material", b"matte")
    shim.vec(dev, mat, "color", s.color, A["ANARI_FLOAT32_VEC3"])
    shim.f32(dev, mat, "opacity", float(s.opacity))
    shim.string(dev, mat, "alphaMode", s.alpha_mode)
    shim.f32(dev, mat, "alphaCutoff", float(s.cutoff))
    shim.anariCommitParameters(dev, mat)
    surf = shim.anariNewSurface(dev)
    shim.obj(dev, surf, "geometry", geom, "ANARI_GEOMETRY")
    shim.obj(dev, surf, "material", mat, "ANARI_MATERIAL")
    shim.i32(dev, surf, "id", s.id, "ANARI_UINT32")
    shim.anariCommitParameters(dev, surf)
    l = spec.lights[0]
    light = shim.anariNewLight(dev, b"directional")
    shim.vec(dev, light, "color", l.color, A["ANARI_FLOAT32_VEC3"])
    shim.vec(dev, light, "direction", l.direction, A["ANARI_FLOAT32_VEC3"])
    shim.f32(dev, light, "irradiance", float(l.irradiance))
    shim.anariCommitParameters(dev, light)
    world = shim.anariNewWorld(dev)
    # the surface list as a parameter array mapped in place
    stride = C.c_uint64(0)
    p = shim.anariMapParameterArray1D(dev, world, b"surface", A["ANARI_SURFACE"], 1,
                                      C.byref(stride))
    assert p and stride.value == C.sizeof(C.c_void_p)
    C.cast(p, C.POINTER(C.c_void_p))[0] = surf
    shim.anariUnmapParameterArray(dev, world, b"surface")
    lights = (C.c_void_p * 1)(light)
    la = shim.anariNewArray1D(dev, C.cast(lights, C.c_void_p), None, None, A["ANARI_LIGHT"], 1)
    shim.obj(dev, world, "light", la, "ANARI_ARRAY1D")
    shim.i32(dev, world, "id", spec.world_id, "ANARI_UINT32")
    shim.anariCommitParameters(dev, world)
    c = spec.camera
    cam = shim.anariNewCamera(dev, b"perspective")
    shim.vec(dev, cam, "position", c.position, A["ANARI_FLOAT32_VEC3"])
    shim.vec(dev, cam, "direction", c.direction, A["ANARI_FLOAT32_VEC3"])
    shim.vec(dev, cam, "up", c.up, A["ANARI_FLOAT32_VEC3"])
    shim.f32(dev, cam, "aspect", float(c.aspect))
    shim.vec(dev, cam, "imageRegion", c.region, A["ANARI_FLOAT32_BOX2"])
    shim.f32(dev, cam, "fovy", float(c.fovy))
    shim.anariCommitParameters(dev, cam)
    r = spec.renderer
    ren = shim.anariNewRenderer(dev, b"default")
    shim.vec(dev, ren, "background", r.background, A["ANARI_FLOAT32_VEC4"])
    shim.vec(dev, ren, "ambientColor", r.ambient_color, A["ANARI_FLOAT32_VEC3"])
    if r.ambient_radiance is not None:
        shim.f32(dev, ren, "ambientRadiance", float(r.ambient_radiance))
    shim.f32(dev, ren, "ambientOcclusionDistance", float(r.ao_distance))
    shim.i32(dev, ren, "cullTriangleBackfaces", int(r.cull), "ANARI_BOOL")
    shim.f32(dev, ren, "volumeSamplingRate", float(r.volume_sampling_rate))
    shim.i32(dev, ren, "pixelSamples", r.pixel_samples)
    shim.i32(dev, ren, "ambientSamples", r.ambient_samples)
    shim.i32(dev, ren, "maxDepth", r.max_depth)
    shim.i32(dev, ren, "maxRayDepth", r.max_ray_depth)
    shim.i32(dev, ren, "checkerboarding", int(r.checkerboard), "ANARI_BOOL")
    shim.anariCommitParameters(dev, ren)
    frame = shim.anariNewFrame(dev)
    size = (C.c_uint32 * 2)(spec.width, spec.height)
    shim.anariSetParameter(dev, frame, b"size", A["ANARI_UINT32_VEC2"], size)
    for ch, t in (("color", "ANARI_UFIXED8_RGBA_SRGB"), ("depth", "ANARI_FLOAT32"),
                  ("primitiveId", "ANARI_UINT32"), ("objectId", "ANARI_UINT32"),
                  ("instanceId", "ANARI_UINT32")):
        shim.i32(dev, frame, "channel." + ch, A[t], "ANARI_DATA_TYPE")
    shim.obj(dev, frame, "renderer", ren, "ANARI_RENDERER")
    shim.obj(dev, frame, "camera", cam, "ANARI_CAMERA")
    shim.obj(dev, frame, "world", world, "ANARI_WORLD")
    shim.anariCommitParameters(dev, frame)
    shim.anariRenderFrame(dev, frame)
    assert shim.anariFrameReady(dev, frame, A["ANARI_WAIT"]) == 1
    out = {}
    for ch, dt in (("color", np.uint32), ("depth", np.float32), ("primitiveId", np.uint32),
                   ("objectId", np.uint32), ("instanceId", np.uint32)):
        w, h, t = C.c_uint32(), C.c_uint32(), C.c_int()
        p = shim.anariMapFrame(dev, frame, ("channel." + ch).encode(), C.byref(w), C.byref(h),
                               C.byref(t))
        assert p and (w.value, h.value) == (spec.width, spec.height)
        want = {"color": "ANARI_UFIXED8_RGBA_SRGB", "depth": "ANARI_FLOAT32"}.get(ch,
                                                                                  "ANARI_UINT32")
        assert t.value == A[want]
        buf = (C.c_uint8 * (w.value * h.value * 4)).from_address(p)
        out[ch] = np.frombuffer(bytes(buf), dt).reshape(h.value, w.value)
        shim.anariUnmapFrame(dev, frame, ("channel." + ch).encode())
    for o in (va, geom, mat, surf, light, la, world, cam, ren, frame):
        shim.anariRelease(dev, o)
    shim.anariRelease(dev, dev)
    return out


@pytest.mark.gpu
def test_soup_renders_through_anari_names(shim, device):
    """The plain-traversal workload (here 20k triangles at 128x96) through
    anari* calls: equal to the library-call build bit for bit, and within
    the parity bar of the oracle."""
    from tests.parity import compare, render_gpu, render_oracle
    from visrtx_gb300 import scenes as S

    spec = S.soup_spec(n=20_000, width=128, height=96, renderer="default")
    shim.messages.clear()
    out = _soup_through_anari(shim, spec)
    assert not [m for m in shim.messages if m[1] <= A["ANARI_SEVERITY_ERROR"]], shim.messages
    ref = render_gpu(device, spec)
    for ch in ("color", "depth", "primitiveId", "objectId", "instanceId"):
        assert np.array_equal(out[ch], ref[ch]), ch
    rep = compare(out, render_oracle(spec))
    assert (out["depth"] < 1e29).mean() > 0.2
    print(rep)


@pytest.mark.gpu
def test_multithreaded_object_creation(shim):
    """The reference's API test (tests/api/TestMultiThreadedObjectCreation.
    cpp:57-95) through the ANARI names: 4 threads released together each
    create 100 x (directional light, perspective camera, triangle geometry,
    world, frame) on one device made by makeVisRTXDevice, then release them;
    every handle is valid and no fatal or error status is reported. ctypes
    drops the GIL around each call, so the threads run inside the library at
    once."""
    import threading

    msgs = []

    def status(user, device, source, source_type, severity, code, message):
        msgs.append((severity, message))

    cb = STATUS_CB(status)
    dev = shim.makeVisRTXDevice(cb, None)
    assert dev
    gate = threading.Event()
    results = [None] * 4

    def work(k):
        gate.wait()
        objs = []
        for _ in range(100):
            objs.append(shim.anariNewLight(dev, b"directional"))
            objs.append(shim.anariNewCamera(dev, b"perspective"))
            objs.append(shim.anariNewGeometry(dev, b"triangle"))
            objs.append(shim.anariNewWorld(dev))
            objs.append(shim.anariNewFrame(dev))
        results[k] = sum(1 for o in objs if o)
        for o in objs:
            shim.anariRelease(dev, o)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    gate.set()
    for t in threads:
        t.join()
    assert results == [500] * 4
    bad = [m for s, m in msgs if s <= A["ANARI_SEVERITY_ERROR"]]
    assert not bad, bad[:5]
    shim.anariRelease(dev, dev)


@pytest.mark.gpu
def test_device_force_init(shim):
    """The reference's other API test (tests/api/TestDeviceInit.cpp:37-44)
    through the ANARI names: makeVisRTXDevice, "forceInit" set on the
    device and committed initialises CUDA at once with no fatal or error
    status, and the device reports its "visrtx" property; then it is
    released."""
    msgs = []

    def status(user, device, source, source_type, severity, code, message):
        msgs.append((severity, message))

    cb = STATUS_CB(status)
    dev = shim.makeVisRTXDevice(cb, None)
    assert dev
    on = C.c_int32(1)
    shim.lib.anariSetParameter(C.c_void_p(dev), C.c_void_p(dev), b"forceInit",
                               A["ANARI_BOOL"], C.byref(on))
    shim.lib.anariCommitParameters(C.c_void_p(dev), C.c_void_p(dev))
    bad = [m for s, m in msgs if s <= A["ANARI_SEVERITY_ERROR"]]
    assert not bad, bad
    flag = C.c_int32(0)
    assert shim.lib.anariGetProperty(C.c_void_p(dev), C.c_void_p(dev), b"visrtx",
                                     A["ANARI_BOOL"], C.byref(flag), 4, 1) == 1
    assert flag.value == 1
    shim.anariRelease(dev, dev)
