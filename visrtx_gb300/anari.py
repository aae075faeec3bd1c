"""Python host API over libvrtx, shaped like ANARI's (anariNewDevice,
anariNewArray*, anariNew<Object>, anariSetParameter, anariCommitParameters,
anariRenderFrame, anariFrameReady, anariMapFrame, anariRelease).

Object subtypes, parameter names, frame channels and defaults are VisRTX's
(devices/rtx/*.json, renderer/Renderer.cpp:152-170, frame/Frame.cu:75-94).
Every call goes through the C ABI of libvrtx; nothing here renders.
"""
from __future__ import annotations

import ctypes as C
from typing import Any, Iterable

import numpy as np

from . import _lib as L

_NP_TYPES = {
    (np.dtype(np.float32), 1): L.FLOAT32,
    (np.dtype(np.float32), 2): L.FLOAT32_VEC2,
    (np.dtype(np.float32), 3): L.FLOAT32_VEC3,
    (np.dtype(np.float32), 4): L.FLOAT32_VEC4,
    (np.dtype(np.uint32), 1): L.UINT32,
    (np.dtype(np.uint32), 2): L.UINT32_VEC2,
    (np.dtype(np.uint32), 3): L.UINT32_VEC3,
    (np.dtype(np.uint32), 4): L.UINT32_VEC4,
    (np.dtype(np.uint8), 1): L.UFIXED8,
    (np.dtype(np.int8), 1): L.FIXED8,
    (np.dtype(np.uint16), 1): L.UFIXED16,
    (np.dtype(np.int16), 1): L.FIXED16,
}


class DataType(int):
    """A parameter whose value is a data type (e.g. "channel.color")."""


class Object:
    type_code = L.OBJECT

    def __init__(self, device: "Device", handle: int, subtype: str = ""):
        if not handle:
            raise RuntimeError(f"libvrtx returned a null {type(self).__name__} handle "
                               f"(subtype '{subtype}'); see device.messages")
        self.device = device
        self.handle = C.c_void_p(handle)
        self.subtype = subtype
        self._keep: dict[str, Any] = {}

    # parameters -----------------------------------------------------------
    def set(self, name: str, value: Any, dtype: int | None = None) -> "Object":
        lib = self.device.lib
        key = name.encode()
        if isinstance(value, Object):
            h = C.c_void_p(value.handle.value)
            lib.vrtxSetParameter(self.device.h, self.handle, key, value.type_code, C.byref(h))
            self._keep[name] = value
            return self
        if isinstance(value, DataType):
            v = C.c_int32(int(value))
            lib.vrtxSetParameter(self.device.h, self.handle, key, L.DATA_TYPE, C.byref(v))
            return self
        if isinstance(value, str):
            lib.vrtxSetParameter(self.device.h, self.handle, key, L.STRING,
                                 C.c_char_p(value.encode()))
            return self
        if dtype is None:
            if isinstance(value, bool):
                dtype = L.BOOL
            elif isinstance(value, (int, np.integer)):
                dtype = L.INT32
            elif isinstance(value, (float, np.floating)):
                dtype = L.FLOAT32
            else:
                arr = np.asarray(value)
                if arr.shape == (4, 4):
                    dtype = L.FLOAT32_MAT4
                else:
                    n = arr.size
                    if arr.dtype.kind in "ui":
                        dtype = {2: L.UINT32_VEC2, 3: L.UINT32_VEC3, 4: L.UINT32_VEC4}[n]
                    else:
                        dtype = {2: L.FLOAT32_VEC2, 3: L.FLOAT32_VEC3, 4: L.FLOAT32_VEC4}[n]
        buf = _pack(value, dtype)
        lib.vrtxSetParameter(self.device.h, self.handle, key, dtype, buf)
        return self

    def unset(self, name: str) -> "Object":
        self.device.lib.vrtxUnsetParameter(self.device.h, self.handle, name.encode())
        self._keep.pop(name, None)
        return self

    def commit(self) -> "Object":
        self.device.lib.vrtxCommitParameters(self.device.h, self.handle)
        return self

    def get_property(self, name: str, dtype: int, wait: bool = True):
        size = {L.FLOAT32: 4, L.INT32: 4, L.BOOL: 4, L.FLOAT32_BOX3: 24}[dtype]
        buf = (C.c_uint8 * size)()
        ok = self.device.lib.vrtxGetProperty(self.device.h, self.handle, name.encode(),
                                             dtype, buf, size, L.WAIT if wait else L.NO_WAIT)
        if not ok:
            return None
        raw = bytes(buf)
        if dtype == L.FLOAT32:
            return np.frombuffer(raw, np.float32)[0].item()
        if dtype in (L.INT32, L.BOOL):
            v = np.frombuffer(raw, np.int32)[0].item()
            return bool(v) if dtype == L.BOOL else v
        return np.frombuffer(raw, np.float32).reshape(2, 3).copy()

    def release(self) -> None:
        if self.handle is not None and self.device.h is not None:
            self.device.lib.vrtxRelease(self.device.h, self.handle)
        self.handle = None
        self._keep.clear()


def _pack(value: Any, dtype: int):
    if dtype == L.BOOL:
        return C.byref(C.c_int32(1 if value else 0))
    if dtype == L.INT32:
        return C.byref(C.c_int32(int(value)))
    if dtype == L.UINT32:
        return C.byref(C.c_uint32(int(value) & 0xFFFFFFFF))
    if dtype == L.FLOAT32:
        return C.byref(C.c_float(float(value)))
    if dtype == L.FLOAT32_MAT4:
        # row-major 4x4 in, column-major (glm/ANARI) out
        return _Buf(np.ascontiguousarray(np.asarray(value, np.float32).reshape(4, 4).T))
    if dtype in (L.UINT32_VEC2, L.UINT32_VEC3, L.UINT32_VEC4, L.INT32_VEC2):
        a = np.ascontiguousarray(np.asarray(value, np.uint32 if dtype != L.INT32_VEC2 else np.int32))
    elif dtype == L.FLOAT64_BOX1:
        a = np.ascontiguousarray(np.asarray(value, np.float64))
    else:
        a = np.ascontiguousarray(np.asarray(value, np.float32))
    return _Buf(a)


class _Buf:
    """Keeps a numpy buffer alive for the duration of a ctypes call."""

    def __init__(self, a: np.ndarray):
        self.a = a
        self._as_parameter_ = a.ctypes.data_as(C.c_void_p)


class Array(Object):
    def __init__(self, device, handle, elem_type, data):
        super().__init__(device, handle)
        self.elem_type = elem_type
        self._data = data  # keeps application memory alive (shared array)

    def release(self) -> None:
        super().release()
        self._data = None  # the library privatised what it still needs


class Device:
    """An ANARI-style device on one GPU (replaces makeVisRTXDevice)."""

    def __init__(self, cuda_device: int = 0, lib_path: str | None = None):
        self.lib = L.load(lib_path)
        self.messages: list[tuple[int, str]] = []
        self._cb = L.STATUS_CB(self._status)
        self.h = C.c_void_p(self.lib.vrtxNewDevice(self._cb, None))
        if cuda_device:
            v = C.c_int32(cuda_device)
            self.lib.vrtxDeviceSetParameter(self.h, b"cudaDevice", L.INT32, C.byref(v))

    def _status(self, user, dev, src, src_type, severity, code, msg):
        self.messages.append((int(severity), msg.decode(errors="replace") if msg else ""))

    def errors(self) -> list[str]:
        return [m for s, m in self.messages if s <= L.SEVERITY_ERROR]

    def is_valid(self) -> bool:
        return bool(self.lib.vrtxDeviceIsValid(self.h))

    @property
    def stream(self) -> int:
        return self.lib.vrtxDeviceStream(self.h) or 0

    # feature queries (VisRTXDevice::getObjectSubtypes, VisRTXFeatureUtility.cpp)
    @staticmethod
    def _strings(p) -> list[str]:
        out = []
        i = 0
        while p and p[i] is not None:
            out.append(p[i].decode())
            i += 1
        return out

    def extensions(self) -> list[str]:
        """The device's "extension" property."""
        p = C.POINTER(C.c_char_p)()
        if not self.lib.vrtxDeviceGetProperty(self.h, b"extension", L.STRING_LIST,
                                              C.byref(p), C.sizeof(p), L.WAIT):
            return []
        return self._strings(p)

    def object_subtypes(self, object_type: int) -> list[str]:
        return self._strings(self.lib.vrtxGetObjectSubtypes(self.h, object_type))

    def object_extensions(self, object_type: int, subtype: str) -> dict[str, bool] | None:
        """visrtxGetObjectExtensions: the flags of one subtype, None if unknown."""
        e = L.VRTXExtensions()
        if not self.lib.vrtxGetObjectExtensions(C.byref(e), self.h, object_type,
                                                subtype.encode()):
            return None
        return e.as_dict()

    def instance_extensions(self) -> dict[str, bool] | None:
        """visrtxGetInstanceExtensions on the device."""
        e = L.VRTXExtensions()
        if not self.lib.vrtxGetInstanceExtensions(C.byref(e), self.h, None):
            return None
        return e.as_dict()

    # arrays -----------------------------------------------------------------
    def new_array(self, data, elem_type: int | None = None) -> Array:
        """1D/2D/3D array. `data` is a numpy array (shared with the library
        until released, then privatised), a list of Objects (object array), or
        a torch CUDA tensor (used in place, NV_ARRAY_CUDA)."""
        if isinstance(data, (list, tuple)) and data and isinstance(data[0], Object):
            handles = (C.c_void_p * len(data))(*[o.handle.value for o in data])
            et = elem_type or data[0].type_code
            h = self.lib.vrtxNewArray1D(self.h, handles, None, None, et, len(data))
            a = Array(self, h, et, (handles, list(data)))
            a.type_code = L.ARRAY1D
            return a
        if hasattr(data, "data_ptr") and getattr(data, "is_cuda", False):
            t = data
            if elem_type is None:
                raise ValueError("elem_type is required for device arrays")
            comps = _components(elem_type)
            n = t.numel() // comps
            h = self.lib.vrtxNewArray1D(self.h, C.c_void_p(t.data_ptr()), None, None, elem_type, n)
            a = Array(self, h, elem_type, t)
            a.type_code = L.ARRAY1D
            return a
        arr = np.ascontiguousarray(data)
        if elem_type is None:
            comps = arr.shape[-1] if arr.ndim >= 2 and arr.shape[-1] in (2, 3, 4) else 1
            elem_type = _NP_TYPES[(arr.dtype, comps)]
        comps = _components(elem_type)
        if elem_type in (L.FLOAT32_MAT4,):
            arr = np.ascontiguousarray(np.swapaxes(arr.reshape(-1, 4, 4), 1, 2))  # column-major
        n = arr.size // comps
        h = self.lib.vrtxNewArray1D(self.h, arr.ctypes.data_as(C.c_void_p), None, None,
                                    elem_type, n)
        a = Array(self, h, elem_type, arr)
        a.type_code = L.ARRAY1D
        return a

    def new_array2d(self, data, elem_type: int | None = None) -> Array:
        """2D array from a (ny, nx) or (ny, nx, c) numpy array (x fastest);
        `elem_type` gives the element type of c-channel data."""
        arr = np.ascontiguousarray(data)
        if elem_type is None:
            elem_type = _NP_TYPES[(arr.dtype, arr.shape[2] if arr.ndim == 3 else 1)]
        ny, nx = arr.shape[:2]
        h = self.lib.vrtxNewArray2D(self.h, arr.ctypes.data_as(C.c_void_p), None, None,
                                    elem_type, nx, ny)
        a = Array(self, h, elem_type, arr)
        a.type_code = L.ARRAY2D
        return a

    def new_array3d(self, data, elem_type: int | None = None) -> Array:
        """3D array from a (nz, ny, nx) or (nz, ny, nx, c) numpy array (x
        fastest), or a CUDA tensor of shape (nz, ny, nx) (used in place,
        NV_ARRAY_CUDA)."""
        if hasattr(data, "data_ptr") and getattr(data, "is_cuda", False):
            nz, ny, nx = data.shape
            et = elem_type or L.FLOAT32
            h = self.lib.vrtxNewArray3D(self.h, C.c_void_p(data.data_ptr()), None, None, et,
                                        nx, ny, nz)
            a = Array(self, h, et, data)
            a.type_code = L.ARRAY3D
            return a
        arr = np.ascontiguousarray(data)
        if elem_type is None:
            elem_type = _NP_TYPES[(arr.dtype, arr.shape[3] if arr.ndim == 4 else 1)]
        nz, ny, nx = arr.shape[:3]
        h = self.lib.vrtxNewArray3D(self.h, arr.ctypes.data_as(C.c_void_p), None, None,
                                    elem_type, nx, ny, nz)
        a = Array(self, h, elem_type, arr)
        a.type_code = L.ARRAY3D
        return a

    # objects ----------------------------------------------------------------
    def _obj(self, cls, fn, type_code, subtype=None):
        h = fn(self.h, subtype.encode()) if subtype is not None else fn(self.h)
        o = cls(self, h, subtype or "")
        o.type_code = type_code
        return o

    def new_camera(self, subtype="perspective"):
        return self._obj(Object, self.lib.vrtxNewCamera, L.CAMERA, subtype)

    def new_geometry(self, subtype):
        return self._obj(Object, self.lib.vrtxNewGeometry, L.GEOMETRY, subtype)

    def new_material(self, subtype="matte"):
        return self._obj(Object, self.lib.vrtxNewMaterial, L.MATERIAL, subtype)

    def new_light(self, subtype="directional"):
        return self._obj(Object, self.lib.vrtxNewLight, L.LIGHT, subtype)

    def new_renderer(self, subtype="default"):
        return self._obj(Object, self.lib.vrtxNewRenderer, L.RENDERER, subtype)

    def new_spatial_field(self, subtype="structuredRegular"):
        return self._obj(Object, self.lib.vrtxNewSpatialField, L.SPATIAL_FIELD, subtype)

    def new_volume(self, subtype="transferFunction1D"):
        return self._obj(Object, self.lib.vrtxNewVolume, L.VOLUME, subtype)

    def new_sampler(self, subtype="image2D"):
        return self._obj(Object, self.lib.vrtxNewSampler, L.SAMPLER, subtype)

    def new_surface(self):
        return self._obj(Object, self.lib.vrtxNewSurface, L.SURFACE)

    def new_group(self):
        return self._obj(Object, self.lib.vrtxNewGroup, L.GROUP)

    def new_instance(self, subtype="transform"):
        return self._obj(Object, self.lib.vrtxNewInstance, L.INSTANCE, subtype)

    def new_world(self):
        return self._obj(Object, self.lib.vrtxNewWorld, L.WORLD)

    def new_frame(self):
        return self._obj(Frame, self.lib.vrtxNewFrame, L.FRAME)

    def release(self) -> None:
        if self.h is not None and self.h.value:
            self.lib.vrtxDeviceRelease(self.h)
        self.h = None


def _components(et: int) -> int:
    return {L.FLOAT32_VEC2: 2, L.FLOAT32_VEC3: 3, L.FLOAT32_VEC4: 4, L.UINT32_VEC2: 2,
            L.UINT32_VEC3: 3, L.UINT32_VEC4: 4, L.FLOAT32_MAT4: 16}.get(et, 1)


_CHANNEL_DTYPES = {
    L.UFIXED8_RGBA_SRGB: (np.uint32, 1), L.UFIXED8_VEC4: (np.uint32, 1),
    L.FLOAT32_VEC4: (np.float32, 4), L.FLOAT32: (np.float32, 1), L.UINT32: (np.uint32, 1),
    L.FLOAT32_VEC3: (np.float32, 3),
}


class Frame(Object):
    type_code = L.FRAME

    def render(self) -> "Frame":
        self.device.lib.vrtxRenderFrame(self.device.h, self.handle)
        return self

    def wait(self) -> None:
        self.device.lib.vrtxFrameReady(self.device.h, self.handle, L.WAIT)

    def ready(self) -> bool:
        return bool(self.device.lib.vrtxFrameReady(self.device.h, self.handle, L.NO_WAIT))

    def map_raw(self, channel: str):
        w, h, t = C.c_uint32(), C.c_uint32(), C.c_int()
        p = self.device.lib.vrtxMapFrame(self.device.h, self.handle, channel.encode(),
                                         C.byref(w), C.byref(h), C.byref(t))
        return p, w.value, h.value, t.value

    def map(self, channel: str) -> np.ndarray | None:
        """Host copy of a channel as (height, width[, comps]) numpy array."""
        p, w, h, t = self.map_raw(channel)
        if not p:
            return None
        dt, comps = _CHANNEL_DTYPES[t]
        n = w * h * comps
        buf = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)),
                                    shape=(n * np.dtype(dt).itemsize,))
        out = buf.view(dt).copy()
        self.device.lib.vrtxUnmapFrame(self.device.h, self.handle, channel.encode())
        return out.reshape((h, w, comps) if comps > 1 else (h, w))

    def kernel_ms(self) -> float:
        return float(self.device.lib.vrtxFrameKernelMilliseconds(self.device.h, self.handle))

    def stats(self) -> dict:
        """libvrtx traversal counters of the last render (see
        "vrtx.stats" in device.cpp)."""
        buf = (C.c_uint64 * 8)()
        ok = self.device.lib.vrtxGetProperty(self.device.h, self.handle, b"vrtx.stats",
                                             L.UINT64, buf, 64, L.WAIT)
        if not ok:
            return {}
        keys = ("rays", "nodes", "tri_tests", "sphere_tests", "blas_entries", "volume_samples",
                "volume_fetches", "error_flags")
        return dict(zip(keys, (int(v) for v in buf)))

    def kernel_launches(self) -> int:
        return int(self.device.lib.vrtxFrameKernelLaunches(self.device.h, self.handle))

    def ao_trace(self) -> dict:
        """The wavefront AO any-hit kernel alone in the last render: its
        counters and the summed device time of its launches (ms)."""
        buf = (C.c_uint64 * 5)()
        ok = self.device.lib.vrtxGetProperty(self.device.h, self.handle, b"vrtx.aoTraceStats",
                                             L.UINT64, buf, 40, L.WAIT)
        ms = self.get_property("vrtx.aoTraceMilliseconds", L.FLOAT32)
        keys = ("rays", "nodes", "tri_tests", "sphere_tests", "blas_entries")
        out = dict(zip(keys, (int(v) for v in buf))) if ok else {}
        out["ms"] = float(ms or 0.0)
        return out


def rgba8(color: np.ndarray) -> np.ndarray:
    """Unpacks UFIXED8 RGBA pixels (uint32, R in the low byte) to (..., 4) uint8."""
    return color.view(np.uint8).reshape(color.shape + (4,))
