"""vrtxDMForwardNoAlloc, the forward pass for callers that cannot allocate
device memory (their memory comes from an allocator that is not CUDA's, or
they run where cudaMalloc must not be called): called through the C ABI, it
must give the same image and state as vrtxDMForward, twice in a row (its
fixed scratch array is reused, so the second call must not see the first
call's leftovers), and reject requests beyond its fixed limits.

Collected last on purpose (file name), so a stop-at-first-failure run has
already run every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest
import torch

from visrtx_gb300 import _lib as L, dm, scenes as S

pytestmark = pytest.mark.gpu


def _volume(seed, n=(20, 18, 22)):
    d = S.gaussian_blobs(n, n_blobs=4, seed=seed, sigma_scale=0.12)
    color, op = S.tf_knots(seed, max_opacity=0.6)
    tf = S.tf_table(color, op, 256)
    return dm.VolumeInput(torch.tensor(d, device="cuda").half().contiguous(),
                          torch.tensor(tf, device="cuda").contiguous(),
                          torch.tensor([1.2], device="cuda"), step=0.5, unit=1.0,
                          value_range=(-0.5, 1.5))


def _run(fn_name, batch):
    lib = L.load()
    image = torch.full((batch.pixels, 3), -7.0, device="cuda")
    state = torch.full((batch.pixels, 2), -7.0, device="cuda")
    vols, views = batch.descriptors()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = getattr(lib, fn_name)(dm._device().h, vols, len(vols), views, len(views),
                               C.c_void_p(image.data_ptr()), C.c_void_p(state.data_ptr()),
                               batch.tile[0], batch.tile[1], stream)
    torch.cuda.synchronize()
    return rc, image, state


def test_no_alloc_forward_matches_allocating_forward():
    batches = []
    for call in range(2):  # two calls in a row, different workloads
        vols = [_volume(10 + call), _volume(20 + call, n=(16, 24, 12))]
        views = []
        for i, res in enumerate([(24, 16), (16, 32), (40, 24)]):
            vi = i % 2
            views.append(dm.look_at_view(vi, vols[vi].dims, 2.0 * S.fibonacci_sphere(3)[i],
                                         50.0, res[0], res[1], (0.1, 0.1, 0.1)))
        batches.append((vols, views))
    for vols, views in batches:
        b = dm.Batch(vols, views, tile=(16, 8))
        rc0, img0, st0 = _run("vrtxDMForward", b)
        rc1, img1, st1 = _run("vrtxDMForwardNoAlloc", b)
        assert rc0 == 0 and rc1 == 0
        torch.testing.assert_close(img1, img0, rtol=0, atol=1e-6)
        torch.testing.assert_close(st1, st0, rtol=0, atol=1e-6)
        assert float(img1.mean()) > 0.0


def test_no_alloc_rejects_oversized_requests():
    v = _volume(3)
    views = [dm.look_at_view(0, v.dims, (0.0, 0.0, 2.0), 50.0, 4, 4)] * 4097
    b = dm.Batch([v], views, tile=(8, 4))
    rc, _, _ = _run("vrtxDMForwardNoAlloc", b)
    assert rc < 0
    assert any("4096 views" in m for m in dm._device().errors())


def test_no_alloc_rejects_a_capturing_stream():
    """Each call copies its descriptors from host memory that it frees on
    return, so it refuses a stream under capture (a captured copy would
    read freed memory at every replay) and leaves the capture usable."""
    v = _volume(5)
    views = [dm.look_at_view(0, v.dims, (0.0, 0.0, 2.0), 50.0, 8, 8)]
    b = dm.Batch([v], views, tile=(8, 4))
    rc, _, _ = _run("vrtxDMForwardNoAlloc", b)  # set-up call, outside capture
    assert rc == 0
    lib = L.load()
    image = torch.zeros((b.pixels, 3), device="cuda")
    state = torch.zeros((b.pixels, 2), device="cuda")
    x = torch.zeros(4, device="cuda")
    vols, vws = b.descriptors()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            x.add_(1.0)
            rc = lib.vrtxDMForwardNoAlloc(dm._device().h, vols, len(vols), vws, len(vws),
                                          C.c_void_p(image.data_ptr()),
                                          C.c_void_p(state.data_ptr()), 8, 4,
                                          C.c_void_p(s.cuda_stream))
    assert rc < 0
    assert any("capturing" in m for m in dm._device().errors())
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0  # capture records the add, the one replay runs it
