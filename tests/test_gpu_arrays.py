"""Array ownership through the C ABI (array/Array.cpp:69-119,164-182, the
ownership rules vrtxNewArray1D documents):
- shared arrays (application memory, no deleter) are read in place, their
  changes reach the frame through map/unmap, and they are privatised (copied)
  when their public handle is released while an object still uses them;
- captured arrays (application memory and a deleter) call the deleter once,
  when the last reference drops;
- managed arrays (no application memory) are filled through vrtxMapArray;
- CUDA device pointers (NV_ARRAY_CUDA) are used in place.

Every case renders one sphere of radius 0.5 seen along +z from z = -3 and
reads the depth of the centre pixel, whose corner ray (raycast) points along
+z exactly: depth = 2.5 + z of the sphere's centre."""
import ctypes as C

import numpy as np
import pytest

from visrtx_gb300 import _lib as L
from visrtx_gb300 import anari as A

pytestmark = pytest.mark.gpu

N = 32


def sphere(dev, positions: A.Array):
    g = dev.new_geometry("sphere")
    g.set("vertex.position", positions)
    g.set("radius", 0.5)
    g.commit()
    return g


def frame_around(dev, g, keep: list):
    """The rest of the scene around a committed sphere geometry: a frame
    ready to render (every handle appended to keep)."""
    m = dev.new_material("matte")
    m.commit()
    s = dev.new_surface()
    s.set("geometry", g).set("material", m)
    s.set("id", 7, L.UINT32)
    s.commit()
    surfaces = dev.new_array([s])
    w = dev.new_world()
    w.set("surface", surfaces)
    w.commit()
    cam = dev.new_camera("perspective")
    cam.set("position", (0.0, 0.0, -3.0), L.FLOAT32_VEC3)
    cam.set("direction", (0.0, 0.0, 1.0), L.FLOAT32_VEC3)
    cam.set("aspect", 1.0)
    cam.commit()
    r = dev.new_renderer("raycast")
    r.commit()
    f = dev.new_frame()
    f.set("size", (N, N), L.UINT32_VEC2)
    f.set("channel.depth", A.DataType(L.FLOAT32))
    f.set("channel.objectId", A.DataType(L.UINT32))
    f.set("renderer", r).set("camera", cam).set("world", w)
    f.commit()
    keep += [g, m, s, surfaces, w, cam, r, f]
    return f


def centre_depth(f) -> float:
    f.render()
    f.wait()
    depth = f.map("channel.depth")
    oid = f.map("channel.objectId")
    assert oid[N // 2, N // 2] == 7
    return float(depth[N // 2, N // 2])


def test_shared_array_map_unmap(device):
    dev = device
    pos = np.zeros((1, 3), np.float32)
    a = dev.new_array(pos, L.FLOAT32_VEC3)
    keep = []
    f = frame_around(dev, sphere(dev, a), keep)
    assert centre_depth(f) == pytest.approx(2.5, abs=1e-4)
    # the application changes its memory between map and unmap
    p = dev.lib.vrtxMapArray(dev.h, a.handle)
    assert p == pos.ctypes.data  # shared: the map is the application's memory
    pos[0, 2] = 1.0
    dev.lib.vrtxUnmapArray(dev.h, a.handle)
    assert centre_depth(f) == pytest.approx(3.5, abs=1e-4)
    assert not dev.errors()


def test_shared_array_privatised_on_release(device):
    """Released before the first frame while the geometry still uses it: the
    library keeps a private copy, so later writes to the application's
    memory do not reach the frame."""
    dev = device
    pos = np.array([[0.0, 0.0, 1.0]], np.float32)
    a = dev.new_array(pos, L.FLOAT32_VEC3)
    g = dev.new_geometry("sphere")
    g.set("vertex.position", a)
    a.release()  # the public reference drops; the geometry still holds one
    pos[0, 2] = 5.0
    g.set("radius", 0.5)
    g.commit()
    keep = []
    f = frame_around(dev, g, keep)
    assert centre_depth(f) == pytest.approx(3.5, abs=1e-4)
    assert not dev.errors()


def test_captured_array_deleter_called_once(device):
    dev = device
    pos = np.array([[0.0, 0.0, 1.0]], np.float32)
    calls = []
    cb = L.DELETER(lambda user, mem: calls.append((user, mem)))
    h = dev.lib.vrtxNewArray1D(dev.h, pos.ctypes.data_as(C.c_void_p), C.cast(cb, C.c_void_p),
                               C.c_void_p(1234), L.FLOAT32_VEC3, 1)
    a = A.Array(dev, h, L.FLOAT32_VEC3, pos)
    keep = []
    f = frame_around(dev, sphere(dev, a), keep)
    assert centre_depth(f) == pytest.approx(3.5, abs=1e-4)
    a.release()
    assert calls == []  # the geometry still holds the array
    assert centre_depth(f) == pytest.approx(3.5, abs=1e-4)
    dev.release()  # every remaining object goes, the array last
    assert calls == [(1234, pos.ctypes.data)]


def test_managed_array_filled_through_map(device):
    dev = device
    h = dev.lib.vrtxNewArray1D(dev.h, None, None, None, L.FLOAT32_VEC3, 1)
    a = A.Array(dev, h, L.FLOAT32_VEC3, None)
    p = dev.lib.vrtxMapArray(dev.h, a.handle)
    assert p
    src = np.array([0.0, 0.0, 2.0], np.float32)
    C.memmove(p, src.ctypes.data, src.nbytes)
    dev.lib.vrtxUnmapArray(dev.h, a.handle)
    keep = []
    f = frame_around(dev, sphere(dev, a), keep)
    assert centre_depth(f) == pytest.approx(4.5, abs=1e-4)
    assert not dev.errors()


def test_cuda_array_used_in_place(device):
    """NV_ARRAY_CUDA: a device pointer is read in place; changes made on the
    device reach the frame through map/unmap."""
    torch = pytest.importorskip("torch")
    dev = device
    t = torch.tensor([[0.0, 0.0, 1.0]], dtype=torch.float32, device="cuda")
    a = dev.new_array(t, L.FLOAT32_VEC3)
    keep = []
    f = frame_around(dev, sphere(dev, a), keep)
    assert centre_depth(f) == pytest.approx(3.5, abs=1e-4)
    assert dev.lib.vrtxMapArray(dev.h, a.handle) == t.data_ptr()
    t[0, 2] = -1.0
    torch.cuda.synchronize()
    dev.lib.vrtxUnmapArray(dev.h, a.handle)
    assert centre_depth(f) == pytest.approx(1.5, abs=1e-4)
    assert not dev.errors()


def test_object_array_from_gpu_memory_is_rejected(device):
    """Arrays of object handles must live in host memory (Array.cpp:78-81):
    one made from a CUDA pointer is refused with an error and a null
    handle, and its memory is left alone."""
    import torch

    buf = torch.zeros(4, dtype=torch.int64, device="cuda")
    dev = device
    h = dev.lib.vrtxNewArray1D(dev.h, C.c_void_p(buf.data_ptr()), None, None, L.SURFACE, 4)
    assert not h
    assert any("object arrays from GPU memory" in m for m in dev.errors())
    dev.messages.clear()
    torch.cuda.synchronize()
    assert int(buf.sum()) == 0
