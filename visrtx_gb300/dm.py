"""Differentiable emission-absorption volume rendering on the GPU.

Forward and adjoint run in libvrtx (vrtxDMForward / vrtxDMBackward /
vrtxDMPlan*; model stated in include/vrtx.h), called through the C ABI with
torch tensors' device pointers on torch's current stream. torch is the
plumbing (memory, streams, autograd bookkeeping); no tensor op here
computes the rendering.

    batch = Batch([VolumeInput(density, tf, scale)], views)
    image = VolumeRender.apply(batch, density, tf, scale)   # (pixels, 3)

Many views of many volumes render in one launch; Plan keeps the launch
descriptors on the device so forward + backward can be captured in a CUDA
graph, and Plan.step_l2 runs forward, L2 loss gradient and backward of a
training step in one persistent launch; autotune() picks the tile shape,
autotune_launch() the tile shape, resident blocks per SM and tiles per
queue fetch.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L

_DT = {torch.float32: L.FLOAT32, torch.float16: L.FLOAT16, torch.bfloat16: L.BFLOAT16}
TILES = [(8, 8), (16, 8), (8, 16), (16, 16), (32, 4), (32, 8)]

_dev = None


def _device():
    """A libvrtx device used as the status-callback sink of DM calls."""
    global _dev
    if _dev is None:
        from .anari import Device

        _dev = Device(0)
    return _dev


def _check(rc: int, what: str):
    if rc != 0:
        msgs = _device().errors()
        raise RuntimeError(f"{what} failed ({rc}): {msgs[-1] if msgs else 'see status callback'}")


@dataclass
class View:
    """A pinhole view of one volume in voxel space (voxel i's centre at i)."""
    volume: int
    width: int
    height: int
    eye: tuple
    d00: tuple
    du: tuple
    dv: tuple
    background: tuple = (0.0, 0.0, 0.0)


def look_at_view(volume: int, dims, eye_unit, fovy_deg: float, width: int, height: int,
                 background=(0.0, 0.0, 0.0)) -> View:
    """A view of a volume whose box maps to [-1, 1]^3: eye_unit is the
    camera in that frame, looking at the centre."""
    nx, ny, nz = dims
    scale = np.array([(nx - 1) / 2.0, (ny - 1) / 2.0, (nz - 1) / 2.0])
    center = scale.copy()
    eye = center + np.asarray(eye_unit, np.float64) * scale
    d = center - eye
    d /= np.linalg.norm(d)
    up = np.array([0.0, 1.0, 0.0])
    if abs(np.dot(d, up)) > 0.99:
        up = np.array([1.0, 0.0, 0.0])
    right = np.cross(d, up)
    right /= np.linalg.norm(right)
    tup = np.cross(right, d)
    # the view frustum in voxel units: scale the basis by the box half-size
    h = 2.0 * math.tan(math.radians(fovy_deg) / 2.0)
    w = h * width / height
    du = right * (w / width)
    dv = -tup * (h / height)
    d00 = d - 0.5 * w * right + 0.5 * h * tup
    return View(volume, width, height, tuple(eye), tuple(d00), tuple(du), tuple(dv),
                tuple(background))


@dataclass
class VolumeInput:
    density: torch.Tensor  # (nz, ny, nx) fp32 / fp16 / bf16, CUDA
    tf: torch.Tensor  # (N, 4) fp32 / fp16 / bf16, CUDA
    scale: torch.Tensor  # () or (1,) fp32, CUDA (opacity scale)
    step: float = 0.5
    unit: float = 1.0
    value_range: tuple = (0.0, 1.0)
    # one atomic per gradient term (no per-thread run-length accumulation)
    plain: bool = False

    @property
    def dims(self):
        nz, ny, nx = self.density.shape
        return (nx, ny, nz)


class Batch:
    """Volumes and views of one launch, with the image layout (views
    concatenated row-major, 3 floats per pixel)."""

    def __init__(self, volumes: list[VolumeInput], views: list[View], tile=(16, 8)):
        self.volumes = volumes
        self.views = views
        self.tile = tuple(tile)
        self.offsets = []
        off = 0
        for v in views:
            self.offsets.append(off)
            off += v.width * v.height
        self.pixels = off
        dts = {v.density.dtype for v in volumes}
        if len(dts) != 1:
            raise ValueError("all volumes of a batch share one density dtype")

    def descriptors(self, grads: list | None = None):
        vols = (L.VRTXDMVolume * len(self.volumes))()
        for i, v in enumerate(self.volumes):
            o = vols[i]
            if not v.density.is_contiguous() or not v.tf.is_contiguous():
                raise ValueError("density and tf must be contiguous")
            o.density = v.density.data_ptr()
            o.densityType = _DT[v.density.dtype]
            o.dims = (C.c_int * 3)(*v.dims)
            o.tf = v.tf.data_ptr()
            o.tfType = _DT[v.tf.dtype]
            o.tfSize = v.tf.shape[0]
            o.opacityScale = 1.0
            o.opacityScaleDevice = v.scale.data_ptr()
            o.step = v.step
            o.unitDistance = v.unit
            o.valueLo, o.valueHi = v.value_range
            o.flags = L.DM_PLAIN if v.plain else 0
            if grads is not None:
                gd, gt, gs = grads[i]
                o.gradDensity = gd.data_ptr() if gd is not None else None
                o.gradTf = gt.data_ptr() if gt is not None else None
                o.gradOpacityScale = gs.data_ptr() if gs is not None else None
        views = (L.VRTXDMView * len(self.views))()
        for i, w in enumerate(self.views):
            o = views[i]
            o.volume = w.volume
            o.width, o.height = w.width, w.height
            o.eye = (C.c_float * 3)(*map(float, w.eye))
            o.d00 = (C.c_float * 3)(*map(float, w.d00))
            o.du = (C.c_float * 3)(*map(float, w.du))
            o.dv = (C.c_float * 3)(*map(float, w.dv))
            o.background = (C.c_float * 3)(*map(float, w.background))
            o.pixelOffset = self.offsets[i]
        return vols, views

    def new_grads(self):
        return [(torch.zeros(v.density.shape, dtype=torch.float32, device=v.density.device),
                 torch.zeros(v.tf.shape, dtype=torch.float32, device=v.tf.device),
                 torch.zeros(1, dtype=torch.float32, device=v.tf.device)) for v in self.volumes]


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def forward(batch: Batch):
    """Renders every view: image (pixels, 3) fp32 and state (pixels, 2)."""
    dev = batch.volumes[0].density.device
    image = torch.empty((batch.pixels, 3), dtype=torch.float32, device=dev)
    state = torch.empty((batch.pixels, 2), dtype=torch.float32, device=dev)
    vols, views = batch.descriptors()
    lib = L.load()
    rc = lib.vrtxDMForward(_device().h, vols, len(vols), views, len(views),
                           C.c_void_p(image.data_ptr()), C.c_void_p(state.data_ptr()),
                           batch.tile[0], batch.tile[1], _stream())
    _check(rc, "vrtxDMForward")
    return image, state


def backward(batch: Batch, state: torch.Tensor, grad_image: torch.Tensor, grads=None):
    """Accumulates fp32 gradients (density, tf, scale) per volume."""
    grads = grads if grads is not None else batch.new_grads()
    g = grad_image.contiguous().float()
    vols, views = batch.descriptors(grads)
    lib = L.load()
    rc = lib.vrtxDMBackward(_device().h, vols, len(vols), views, len(views), None,
                            C.c_void_p(state.data_ptr()), C.c_void_p(g.data_ptr()),
                            batch.tile[0], batch.tile[1], _stream())
    _check(rc, "vrtxDMBackward")
    return grads


class VolumeRender(torch.autograd.Function):
    """image = VolumeRender.apply(batch, d0, tf0, s0, d1, tf1, s1, ...)"""

    @staticmethod
    def forward(ctx, batch: Batch, *tensors):
        image, state = forward(batch)
        ctx.batch = batch
        ctx.save_for_backward(state)
        return image

    @staticmethod
    def backward(ctx, grad_image):
        (state,) = ctx.saved_tensors
        batch = ctx.batch
        grads = backward(batch, state, grad_image)
        out = [None]
        for v, (gd, gt, gs) in zip(batch.volumes, grads):
            out += [gd.to(v.density.dtype), gt.to(v.tf.dtype), gs.reshape(v.scale.shape)]
        return tuple(out)


def render(batch: Batch) -> torch.Tensor:
    ts = []
    for v in batch.volumes:
        ts += [v.density, v.tf, v.scale]
    return VolumeRender.apply(batch, *ts)


class Plan:
    """Descriptors on the device; forward()/backward() issue a counter reset
    and one kernel each, on torch's current stream (CUDA-graph capturable).
    Owns image/state/gradient buffers."""

    def __init__(self, batch: Batch, with_grads: bool = True):
        self.batch = batch
        dev = batch.volumes[0].density.device
        self.image = torch.empty((batch.pixels, 3), dtype=torch.float32, device=dev)
        self.state = torch.empty((batch.pixels, 2), dtype=torch.float32, device=dev)
        self.grads = batch.new_grads() if with_grads else None
        self._vols, self._views = batch.descriptors(self.grads)
        lib = L.load()
        self.h = lib.vrtxDMPlanCreate(_device().h, self._vols, len(self._vols), self._views,
                                      len(self._views), batch.tile[0], batch.tile[1], _stream())
        if not self.h:
            _check(-1, "vrtxDMPlanCreate")

    def forward(self):
        _check(L.load().vrtxDMPlanForward(C.c_void_p(self.h), C.c_void_p(self.image.data_ptr()),
                                          C.c_void_p(self.state.data_ptr()), _stream()),
               "vrtxDMPlanForward")
        return self.image

    def backward(self, grad_image: torch.Tensor):
        _check(L.load().vrtxDMPlanBackward(C.c_void_p(self.h), C.c_void_p(self.state.data_ptr()),
                                           C.c_void_p(grad_image.data_ptr()), _stream()),
               "vrtxDMPlanBackward")
        return self.grads

    def step_l2(self, target: torch.Tensor, loss_scale: float = 1.0, image: bool = True,
                loss: torch.Tensor | None = None):
        """One fused training step of the L2 loss loss_scale * sum((image -
        target)^2): forward, loss gradient and backward in one launch,
        gradients added into self.grads. Writes self.image when `image`;
        adds the loss into `loss` (a one-element fp32 CUDA tensor) when
        given."""
        if target.dtype != torch.float32 or not target.is_contiguous() \
                or target.numel() != self.image.numel():
            raise ValueError("target must be a contiguous fp32 tensor shaped like the image")
        _check(L.load().vrtxDMPlanStepL2(
            C.c_void_p(self.h), C.c_void_p(target.data_ptr()), float(loss_scale),
            C.c_void_p(self.image.data_ptr()) if image else None,
            C.c_void_p(loss.data_ptr()) if loss is not None else None, _stream()),
            "vrtxDMPlanStepL2")
        return self.grads

    def set_launch(self, blocks_per_sm: int = 0, tiles_per_fetch: int = 1):
        """Launch shape of both kernels: resident blocks per SM (0: as many
        as fit) and tiles taken from the work queue per fetch."""
        _check(L.load().vrtxDMPlanSetLaunch(C.c_void_p(self.h), int(blocks_per_sm),
                                            int(tiles_per_fetch)), "vrtxDMPlanSetLaunch")
        self.launch = (int(blocks_per_sm), int(tiles_per_fetch))

    def release(self):
        if self.h:
            L.load().vrtxDMPlanRelease(C.c_void_p(self.h))
            self.h = None


BLOCKS_PER_SM = (0, 1, 2)
TILES_PER_FETCH = (1, 2, 8)


@dataclass
class Launch:
    """A tuned launch: tile shape, resident blocks per SM (0: as many as
    fit) and tiles per queue fetch."""
    tile: tuple
    blocks_per_sm: int = 0
    tiles_per_fetch: int = 1


def _time_plan(volumes, views, tile, shape, reps, fused=False):
    p = Plan(Batch(volumes, views, tile))
    p.set_launch(*shape)
    g = torch.ones_like(p.image)

    def step():
        if fused:
            p.step_l2(g, image=False)
        else:
            p.forward()
            p.backward(g)

    step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        step()
    torch.cuda.synchronize()
    p.release()
    return (time.perf_counter() - t0) / reps


def autotune_launch(volumes: list[VolumeInput], views: list[View], tiles=TILES,
                    blocks_per_sm=BLOCKS_PER_SM, tiles_per_fetch=TILES_PER_FETCH, reps: int = 2,
                    cache: str | None = None, fused: bool = False) -> Launch:
    """Times forward + backward of this workload (with `fused`, the one-launch
    L2 training step, Plan.step_l2) over the tile shapes, then, for the
    fastest tile, over resident blocks per SM x tiles per queue fetch;
    returns the fastest Launch. Cached in a JSON file keyed by the
    workload's shape when `cache` is given."""
    key = "launch:" + json.dumps({"fused": fused, "dtype": str(volumes[0].density.dtype),
                                  "dims": sorted({v.dims for v in volumes}),
                                  "res": sorted({(w.width, w.height) for w in views}),
                                  "views": len(views), "volumes": len(volumes)}, default=list)
    table = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            table = json.load(f)
        if key in table:
            e = table[key]
            return Launch(tuple(e["tile"]), e["blocks_per_sm"], e["tiles_per_fetch"])
    times = {tile: _time_plan(volumes, views, tile, (0, 1), reps, fused) for tile in tiles}
    tile = min(times, key=times.get)
    shapes = {(b, f): _time_plan(volumes, views, tile, (b, f), reps, fused)
              for b in blocks_per_sm for f in tiles_per_fetch}
    b, f = min(shapes, key=shapes.get)
    best = Launch(tuple(tile), b, f)
    if cache:
        table[key] = {"tile": list(tile), "blocks_per_sm": b, "tiles_per_fetch": f,
                      "ms_tiles": {f"{a}x{c}": 1e3 * t for (a, c), t in times.items()},
                      "ms_shapes": {f"{a}/{c}": 1e3 * t for (a, c), t in shapes.items()}}
        os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
        with open(cache, "w") as fh:
            json.dump(table, fh, indent=1)
    return best


def autotune(volumes: list[VolumeInput], views: list[View], candidates=TILES, reps: int = 3,
             cache: str | None = None) -> tuple:
    """Times forward + backward for each tile shape on this workload and
    returns the fastest; results are cached in a JSON file keyed by the
    workload's shape when `cache` is given."""
    key = json.dumps({"dtype": str(volumes[0].density.dtype),
                      "dims": sorted({v.dims for v in volumes}),
                      "res": sorted({(w.width, w.height) for w in views}),
                      "views": len(views), "volumes": len(volumes)}, default=list)
    table = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            table = json.load(f)
        if key in table:
            return tuple(table[key]["tile"])
    times = {}
    for tile in candidates:
        b = Batch(volumes, views, tile)
        p = Plan(b)
        g = torch.ones_like(p.image)
        p.forward()
        p.backward(g)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            p.forward()
            p.backward(g)
        torch.cuda.synchronize()
        times[tile] = (time.perf_counter() - t0) / reps
        p.release()
    best = min(times, key=times.get)
    if cache:
        table[key] = {"tile": list(best), "ms": {f"{a}x{b}": 1e3 * t for (a, b), t in times.items()}}
        os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
        with open(cache, "w") as f:
            json.dump(table, f, indent=1)
    return best
