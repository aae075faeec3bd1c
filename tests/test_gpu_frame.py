"""Frame-level behaviour through the C ABI (frame/Frame.cu:163-310,559-588):
the completion callback, the duration / numSamples / nextFrameReset
properties, frameReady polling, the sample limit and invalid frames."""
import ctypes as C

import pytest

from visrtx_gb300 import _lib as L
from visrtx_gb300 import scenes as S
from tests.parity import render_gpu

pytestmark = pytest.mark.gpu

COMPLETION_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_void_p)


def test_completion_callback_and_frame_properties(device):
    dev = device
    spec = S.soup_spec(n=2000, width=64, height=48, renderer="raycast")
    g = render_gpu(dev, spec)
    f = g["frame"]
    calls = []
    cb = COMPLETION_CB(lambda user, d, fr: calls.append((user, d, fr)))
    fp = C.c_void_p(C.cast(cb, C.c_void_p).value)
    ud = C.c_void_p(4321)
    dev.lib.vrtxSetParameter(dev.h, f.handle, b"frameCompletionCallback", L.FUNCTION_POINTER,
                             C.byref(fp))
    dev.lib.vrtxSetParameter(dev.h, f.handle, b"frameCompletionCallbackUserData",
                             L.VOID_POINTER, C.byref(ud))
    f.commit()
    assert f.get_property("nextFrameReset", L.BOOL)  # the commit is a change
    f.render()
    f.wait()
    assert f.ready()
    # fired once, after the frame's work, from the stream (cudaLaunchHostFunc)
    assert calls == [(4321, dev.h.value, f.handle.value)]
    dur = f.get_property("duration", L.FLOAT32)
    assert 0.0 < dur < 10.0
    # numSamples is the frame id of the last frame (Frame.cu:176-180): 0 for
    # the first frame after a reset
    assert f.get_property("numSamples", L.INT32) == 0
    assert not f.get_property("nextFrameReset", L.BOOL)
    # raycast's sample limit is 1 and the limit is checked before the frame
    # id advances (Frame.cu:251-253): the second frame (id 1) still renders,
    # the third does no work and fires no callback
    f.render()
    f.wait()
    assert len(calls) == 2
    assert f.get_property("numSamples", L.INT32) == 1
    f.render()
    f.wait()
    assert len(calls) == 2
    assert f.get_property("numSamples", L.INT32) == 1
    # a camera change resets accumulation: the next render runs again
    cam = g["frame"]._keep["camera"]
    cam.set("fovy", 0.9)
    cam.commit()
    assert f.get_property("nextFrameReset", L.BOOL)
    f.render()
    f.wait()
    assert len(calls) == 3
    assert f.get_property("numSamples", L.INT32) == 0
    assert not dev.errors()


def test_invalid_frame_is_skipped_with_an_error(device):
    """A frame without a world renders nothing and reports an ERROR
    (Frame.cu:216-234); frameReady answers at once."""
    dev = device
    spec = S.soup_spec(n=200, width=16, height=16, renderer="raycast")
    g = render_gpu(dev, spec)
    f = g["frame"]
    f.unset("world")
    f.commit()
    n0 = len(dev.errors())
    f.render()
    assert f.ready()
    errs = dev.errors()[n0:]
    assert errs and any("ANARIWorld" in e for e in errs)


def test_calls_keep_the_threads_current_device(built):
    """Each call runs on the device's own GPU and restores the calling
    thread's current device (CUDADeviceScope, VisRTXDevice.cpp:790-814).
    Needs two GPUs: the library renders on GPU 1 while the thread stays on
    GPU 0."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    from visrtx_gb300 import anari

    torch.cuda.set_device(0)
    dev = anari.Device(1)
    try:
        spec = S.soup_spec(n=500, width=32, height=24, renderer="raycast")
        g = render_gpu(dev, spec)
        assert torch.cuda.current_device() == 0
        ptr, w, h, _ = g["frame"].map_raw("channel.depthCUDA")
        assert ptr and (w, h) == (32, 24)
        assert not dev.errors()
    finally:
        dev.release()
    assert torch.cuda.current_device() == 0


@pytest.mark.parametrize("renderer", ["default", "ao"])
def test_traversal_step_limit_sets_error_flag(device, renderer):
    """The device-side traversal bound ends a ray's traversal and sets bit 1
    of the frame's error flags instead of spinning; "vrtx.maxTraversalSteps"
    lowers it so that the guard runs out on a real scene. The context stays
    usable: with the default bound the next frame is clean and equal to a
    frame that never hit the guard. "ao" over opaque surfaces runs the
    wavefront kernels (closest-hit primary rays and the resumable any-hit
    loop), "default" the per-pixel kernel."""
    import numpy as np

    if renderer == "ao":
        spec = S.instanced_spec(subdiv=3, n_inst=8, n_spheres=3000, width=64, height=48, spp=1,
                                ao_samples=4, renderer="ao")
    else:
        spec = S.soup_spec(n=4000, width=64, height=48, renderer="default")
    g = render_gpu(device, spec)
    f = g["frame"]
    assert f.stats()["error_flags"] == 0
    clean = f.map("channel.color")
    f.set("vrtx.maxTraversalSteps", 3)
    f.commit()
    f.render()
    f.wait()
    assert f.stats()["error_flags"] & 2
    f.unset("vrtx.maxTraversalSteps")
    f.commit()
    f.render()
    f.wait()
    assert f.stats()["error_flags"] == 0
    assert np.array_equal(f.map("channel.color"), clean)
    assert not device.errors()


def test_frame_allocation_failure_is_reported_and_recovers(device):
    """Host-side fault injection: the device is told to fail the next frame
    allocation ("vrtx.failFrameAllocations"; no CUDA call is made for it).
    The commit reports the failure and frees what it had allocated, render
    skips the frame with an error (no kernel touches a missing buffer), map
    returns nothing; the next commit allocates again and the frame equals
    one that never failed. Nothing faults the GPU."""
    import numpy as np

    dev = device
    spec = S.soup_spec(n=2000, width=64, height=48, renderer="raycast")
    ref = render_gpu(dev, spec)
    assert not dev.errors()
    # the first 1, 3 or 9 allocations of the frame's commit fail: the
    # accumulation buffer alone, the first channels too, or every buffer and
    # counter (6 buffers, then 3 counters)
    for fail_at in (1, 3, 9):
        k = C.c_int32(fail_at)
        dev.lib.vrtxDeviceSetParameter(dev.h, b"vrtx.failFrameAllocations", L.INT32, C.byref(k))
        frame, world, keep = S.build_on_device(dev, spec)
        # the frame commit used up the injected failures
        assert any("frame buffer allocation failed" in m for m in dev.errors())
        frame.render()
        frame.wait()
        assert any("invalid frame buffers" in m for m in dev.errors())
        assert frame.map("channel.color") is None
        dev.messages.clear()
        frame.commit()
        frame.render()
        frame.wait()
        assert not dev.errors(), dev.errors()
        for ch in ("color", "depth", "primitiveId", "objectId", "instanceId"):
            assert np.array_equal(frame.map("channel." + ch), ref[ch]), (fail_at, ch)
        for o in keep + [frame]:
            o.release()


def test_device_colour_write_against_reference_glm(device):
    """The colour write every render kernel ends with, run on the GPU
    (vrtxDebugWriteColors), against writeOutputColor's glm calls computed on
    the host from the glm the reference vendors (tests/golden/
    color_golden.npz): bit-exact in both formats on all 3269 colours after 1
    and 7 samples, including sRGB, whose powf runs on the device here and on
    the host in the fixtures."""
    import os

    import numpy as np

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "color_golden.npz"))
    for frames in (1, 7):
        acc = np.ascontiguousarray(z[f"accum_{frames}"], np.float32)
        for fmt in (0, 1):
            out = np.zeros(len(acc), np.uint32)
            rc = device.lib.vrtxDebugWriteColors(device.h, acc.ctypes.data, len(acc), frames - 1,
                                                 fmt, out.ctypes.data)
            assert rc == 0, device.errors()
            ref = z[f"packed_{frames}_{fmt}"]
            diff = np.abs(out.view(np.uint8).astype(np.int32).reshape(-1, 4)
                          - ref.view(np.uint8).astype(np.int32).reshape(-1, 4))
            exact = float(np.mean(out == ref))
            print("frames", frames, "format", fmt, "exact", exact, "max step", int(diff.max()))
            assert exact == 1.0, (frames, fmt, int(diff.max()))
