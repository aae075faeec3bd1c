"""The benchmark workloads beside bench.py's headline (instanced geometry +
AO). bench.py puts each one's measurement into its JSON line under
"workloads"; `python bench.py --workload <name>` prints one of them alone.

  soup     100k-triangle FP32 soup, one instance, 512x384 pinhole camera,
           1 spp, one directional light, matte, renderer "default"; Mrays/s
           (primary + shadow rays) and primary Mrays/s.
  volume   structured-regular 512^3 FP32 volume (64 Gaussian blobs), 256-entry
           TF from 8-knot ramps, 16^3 macrocells, 0.5-voxel steps, 1920x1080
           orbit camera, 1 spp, raycast renderer; Msamples/s (march
           positions, the reference's samples) and Mrays/s.
  nanovdb  the same 512^3 field as a sparse NanoVDB grid (voxels >= 0.02 set;
           --nvdb-type float|fp4|fp8|fp16|fpn, default fp16) through the
           "nanovdb" spatial field, same TF, camera, steps and renderer;
           Msamples/s (opt-in only).
  dm       differentiable marcher: 256^3 FP16 density (32 blobs), 128 views
           of 512x512 on a Fibonacci sphere of radius 2, L2 loss against a
           target rendered from a second volume; forward + backward views/s,
           batched (one graph-captured launch pair, autotuned tiles) against
           the FP32 one-view-per-launch form, both with staged gradient
           accumulation and with one atomic per gradient term.
  batched  64 volumes with edges U[64,384] (BF16, own TFs), 4-32 views each
           at {256,512,1024}^2; forward + backward views/s, one
           graph-captured launch pair against FP32 one launch per view.

Every figure is device time (CUDA events on the launching stream) with L2
flushed between steps; `e2e` is the same metric through the public API
with host inputs copied in and the result read back inside the timed
region; `cpu_baseline` is the CPU oracle (a restatement of the reference's
algorithm) on the host's cores over a bounded sample of the workload.
"""
from __future__ import annotations

import json
import os
import statistics
import time

import numpy as np
import torch

from bench import ClockSampler, algorithmic_bytes, measured_peaks
from visrtx_gb300 import anari, dm, scenes as S

L2_FLUSH_BYTES = 256 * 1024 * 1024


def _flush(buf):
    buf.zero_()
    torch.cuda.synchronize()


def _cores() -> int:
    return os.cpu_count() or 1


def _frames(frame, steps, warmup, flush, before=None):
    """Renders warmup + steps frames; returns per-frame (duration s, stats,
    kernel launches, integrator-kernel ms) of the timed ones."""
    out = []
    for i in range(warmup + steps):
        if before:
            before()
        _flush(flush)
        frame.render()
        frame.wait()
        if i >= warmup:
            out.append((frame.get_property("duration", 240), frame.stats(),
                        frame.kernel_launches(), frame.kernel_ms()))
    return out


def _roofline(bytes_, seconds, peaks, bound="hbm", traffic=None, **extra):
    ach = bytes_ / seconds / 1e9
    r = {"bound": bound, "achieved": round(ach, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
         "frac": round(ach / peaks["hbm_gbs"], 4), "traffic": traffic,
         "peak_source": peaks["source"]}
    r.update(extra)
    return r


# ---------------------------------------------------------------------------
# config 1: the plain 100k-triangle soup, renderer "default"
# ---------------------------------------------------------------------------

def measure_soup(local=0, steps=20, warmup=5, with_cpu=True):
    dev = anari.Device(local)
    spec = S.soup_spec(renderer="default")
    chans = ("color", "depth", "primitiveId")
    frame, world, keep = S.build_on_device(dev, spec, channels=chans)
    ren = frame._keep["renderer"]
    ren.set("sampleLimit", 0)
    ren.commit()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    res = _frames(frame, steps, warmup, flush)
    assert not dev.errors(), dev.errors()
    secs = sum(r[0] for r in res)
    rays = sum(r[1]["rays"] for r in res)
    prim = spec.width * spec.height * steps
    assert all(r[1]["error_flags"] == 0 for r in res)
    build_ms = float(dev.lib.vrtxWorldBuildMilliseconds(dev.h, world.handle))
    kms = statistics.mean(r[3] for r in res)
    # counting pass (untimed): nodes and primitive tests of one frame
    frame.set("vrtx.countTraversal", True)
    frame.commit()
    frame.render()
    frame.wait()
    cst = frame.stats()
    frame.set("vrtx.countTraversal", False)
    frame.commit()
    peaks = measured_peaks()
    fbytes = algorithmic_bytes(cst)
    # end to end through the C ABI: scene from host arrays, BVH build,
    # render, the three channels read back
    e2e, h2d, d2h = [], 0, 0
    for i in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fr2, w2, k2 = S.build_on_device(dev, spec, channels=chans)
        r2 = fr2._keep["renderer"]
        r2.set("sampleLimit", 0)
        r2.commit()
        fr2.render()
        outs = [fr2.map("channel." + c) for c in chans]
        t1 = time.perf_counter()
        st2 = fr2.stats()
        if i:  # the first one warms the allocator
            e2e.append(st2["rays"] / (t1 - t0) / 1e6)
        h2d = int(spec.surfaces[0].vertices.nbytes)
        d2h = sum(int(o.nbytes) for o in outs)
        for o in k2 + [fr2]:
            o.release()
    line = {
        "metric": "Mrays/s", "value": round(rays / secs / 1e6, 2), "unit": "Mrays/s",
        "steps": steps, "warmup": warmup, "ms_per_step": round(1000 * secs / steps, 4),
        "dtype": "f32",
        "config": {"workload": "soup100k_512x384_default_1spp", "renderer": "default",
                   "l2": "flushed between frames (256 MiB)", "bvh_build_ms": round(build_ms, 2)},
        "primary_mrays_per_s": round(prim / secs / 1e6, 2),
        "rays_per_frame": rays / steps,
        "gpu_launches": sum(r[2] for r in res),
        "roofline": _roofline(fbytes, kms / 1e3, peaks, kernel="k_render<default>",
                              algorithmic_bytes_per_launch=fbytes,
                              launch_ms=round(kms, 4),
                              nodes_per_ray=round(cst["nodes"] / max(cst["rays"], 1), 2)),
        "e2e": {"value": round(statistics.median(e2e), 2), "unit": "Mrays/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "includes": "array upload, BVH build, frame, colour/depth/primitiveId read-back"},
    }
    for o in keep + [frame]:
        o.release()
    dev.release()
    if with_cpu:
        line["cpu_baseline"] = cpu_soup()
    return line


def cpu_soup():
    """The oracle's tracer on the full soup frame, all host threads."""
    from oracle import oracle as O

    spec = S.soup_spec(renderer="default")
    sc = O.OracleScene(spec)
    cores = _cores()
    sc.render(threads=cores)
    t0 = time.perf_counter()
    reps = 0
    rays = 0
    while reps < 3 or time.perf_counter() - t0 < 2.0:
        o = sc.render(threads=cores)
        rays += o["rays"]
        reps += 1
    dt = time.perf_counter() - t0
    sc.release()
    return {"value": round(rays / dt / 1e6, 3), "unit": "Mrays/s", "cores": cores,
            "kind": "port", "sample": f"the full 512x384 frame x {reps} ({dt:.1f} s)"}


# ---------------------------------------------------------------------------
# config 3: the 512^3 structured-regular volume
# ---------------------------------------------------------------------------

VOLUME_WORKLOAD = "volume512_blobs64_tf256_step0.5_1920x1080_1spp_raycast"


def measure_volume(local=0, steps=20, warmup=5, with_cpu=True, cpu_seconds=6.0):
    dev = anari.Device(local)
    field = S.gaussian_blobs((512, 512, 512), 64, 0, device="cuda")
    spec = S.volume_spec(field=field, renderer="raycast", sampling_rate=1.0)
    frame, world, keep = S.build_on_device(dev, spec, channels=("color", "depth"))
    cam = frame._keep["camera"]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler(local)
    clocks.start()
    res = _frames(frame, steps, warmup, flush, before=cam.commit)
    clk = clocks.stop()
    kms = statistics.mean(r[3] for r in res)
    assert not dev.errors(), dev.errors()
    secs = sum(r[0] for r in res)
    samples = sum(r[1]["volume_samples"] for r in res)
    fetches = sum(r[1]["volume_fetches"] for r in res)
    rays = sum(r[1]["rays"] for r in res)
    peaks = measured_peaks()
    n = 512
    compulsory = n ** 3 * 4 + (n // 16) ** 3 * 4 + 256 * 16 + 1920 * 1080 * 8
    # end to end: the field from pinned host memory through a new array,
    # commit (texture upload, grids), render, colour read-back
    host = field.cpu().pin_memory()
    spec_h = S.volume_spec(field=host.numpy(), renderer="raycast", sampling_rate=1.0)
    e2e = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fr2, w2, k2 = S.build_on_device(dev, spec_h, channels=("color",))
        fr2.render()
        col = fr2.map("channel.color")
        t1 = time.perf_counter()
        st2 = fr2.stats()
        if i:
            e2e.append(st2["volume_samples"] / (t1 - t0) / 1e6)
        for o in k2 + [fr2]:
            o.release()
    line = {
        "metric": "Msamples/s", "value": round(samples / secs / 1e6, 1), "unit": "Msamples/s",
        "steps": steps, "warmup": warmup, "ms_per_step": round(1000 * secs / steps, 4),
        "dtype": "f32",
        "config": {"workload": VOLUME_WORKLOAD, "l2": "flushed between frames (256 MiB)"},
        "mrays_per_s": round(rays / secs / 1e6, 2),
        "samples_per_frame": samples / steps,
        "fetched_fraction": round(fetches / max(samples, 1), 4),
        "gpu_launches": sum(r[2] for r in res),
        "roofline": _roofline(compulsory, kms / 1e3, peaks, kernel="k_render<raycast, volumes>",
                              algorithmic_bytes_per_launch=compulsory, launch_ms=round(kms, 4),
                              note="compulsory bytes (the field once, grids, TF, framebuffer)"
                                   "; the march is texture- and issue-bound"),
        "e2e": {"value": round(statistics.median(e2e), 1), "unit": "Msamples/s",
                "h2d_bytes_per_step": int(host.numel() * 4), "d2h_bytes_per_step": int(col.nbytes),
                "includes": "field upload (pinned host), texture + grid build, frame, read-back"},
        "clocks": clk,
    }
    for o in keep + [frame]:
        o.release()
    dev.release()
    del field, host
    torch.cuda.empty_cache()
    if with_cpu:
        line["cpu_baseline"] = cpu_volume(spec_h, cpu_seconds)
    return line


def cpu_volume(spec, seconds):
    """The oracle's parity-mode marcher (FP32, the texture unit's filter
    restated) on a band of rows through the middle of the frame."""
    from oracle import oracle as O

    sc = O.OracleScene(spec)
    cores = _cores()
    mid = spec.height // 2
    t0 = time.perf_counter()
    sc.render(rows=(mid - 2, mid + 2), threads=cores)
    per_row = (time.perf_counter() - t0) / 4
    band = int(min(spec.height, max(4, seconds / max(per_row, 1e-6))))
    r0 = max(0, mid - band // 2)
    r1 = min(spec.height, r0 + band)
    t0 = time.perf_counter()
    o = sc.render(rows=(r0, r1), threads=cores)
    dt = time.perf_counter() - t0
    sc.release()
    return {"value": round(o["volume_samples"] / dt / 1e6, 3), "unit": "Msamples/s",
            "cores": cores, "kind": "port",
            "sample": f"rows {r0}-{r1} of 1920x1080 ({o['volume_samples']} samples, {dt:.1f} s)"}


# ---------------------------------------------------------------------------
# NanoVDB (opt-in)
# ---------------------------------------------------------------------------

def measure_nanovdb(local=0, steps=5, warmup=3, nvdb_type="fp16"):
    from visrtx_gb300 import nanovdb as NV

    dev = anari.Device(local)
    field = S.gaussian_blobs((512, 512, 512), 64, 0, device="cuda").cpu().numpy()
    t0 = time.time()
    grid = NV.build_grid(field, field >= 0.02, grid_type=nvdb_type)
    build_s = time.time() - t0
    info = NV.grid_info(grid)
    del field
    spec = S.nanovdb_volume_spec(grid, renderer="raycast", sampling_rate=1.0)
    frame, world, keep = S.build_on_device(dev, spec, channels=("color", "depth"))
    cam = frame._keep["camera"]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler(local)
    clocks.start()
    res = _frames(frame, steps, warmup, flush, before=cam.commit)
    clk = clocks.stop()
    kms = statistics.mean(r[3] for r in res)
    secs = sum(r[0] for r in res)
    samples = sum(r[1]["volume_samples"] for r in res)
    rays = sum(r[1]["rays"] for r in res)
    peaks = measured_peaks()
    compulsory = int(grid.size) + 256 * 16 + 1920 * 1080 * 8
    line = {
        "metric": "Msamples/s", "value": round(samples / secs / 1e6, 2), "unit": "Msamples/s",
        "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": round(1000 * secs / steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"nanovdb512_{nvdb_type}_blobs64_tf256_step0.5_1920x1080"
                               "_1spp_raycast",
                   "grid_bytes": int(grid.size), "active_voxels": info["voxels"],
                   "leaves": info["leaves"], "grid_build_s": round(build_s, 1),
                   "l2": "flushed between frames (256 MiB)"},
        "mrays_per_s": round(rays / secs / 1e6, 2),
        "samples_per_frame": samples / steps,
        "roofline": _roofline(compulsory, kms / 1e3, peaks, algorithmic_bytes_per_launch=compulsory),
        "clocks": clk,
    }
    for o in keep + [frame]:
        o.release()
    dev.release()
    return line


# ---------------------------------------------------------------------------
# configs 4 and 5: the differentiable marcher
# ---------------------------------------------------------------------------

def _dm_problem(n=256, views=128, res=512, dtype=torch.float16, seed=0):
    d = S.gaussian_blobs((n, n, n), 32, seed, device="cuda")
    color, op = S.tf_knots(seed, max_opacity=0.25)
    tf = torch.tensor(S.tf_table(color, op, 256), device="cuda")
    scale = torch.tensor([1.0], device="cuda")
    vol = dm.VolumeInput(d.to(dtype).contiguous(), tf, scale,
                         step=0.5, unit=1.0, value_range=(0.0, 1.0))
    tgt = dm.VolumeInput(S.gaussian_blobs((n, n, n), 32, seed + 1, device="cuda"), tf, scale,
                         step=0.5, unit=1.0, value_range=(0.0, 1.0))
    dirs = S.fibonacci_sphere(views)
    vws = [dm.look_at_view(0, vol.dims, 2.0 * dirs[i], 45.0, res, res) for i in range(views)]
    return vol, d, tgt, vws


def _time_steps(fn, steps, warmup, flush):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        _flush(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    return ts


def _batched_step(vols, views, tile, target, shape=(0, 1), fused=True):
    """One training step of the L2 loss through a plan (launch shape:
    blocks per SM, tiles per queue fetch), captured in a CUDA graph: with
    `fused` the one-launch step (forward, loss gradient and backward in one
    persistent kernel), else a forward launch, the loss gradient in torch
    and a backward launch."""
    b = dm.Batch(vols, views, tile)
    p = dm.Plan(b)
    p.set_launch(*shape)
    grad = torch.empty_like(p.image)

    def body():
        for gd, gt, gs in p.grads:
            gd.zero_()
            gt.zero_()
            gs.zero_()
        if fused:
            p.step_l2(target)
            return
        img = p.forward()
        torch.sub(img, target, out=grad)
        grad.mul_(2.0)
        p.backward(grad)

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        body()
    torch.cuda.current_stream().wait_stream(s)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        body()
    # the graph writes into `grad` at every replay: keep it alive with the plan
    p.graph_buffers = (grad, target)
    return p, graph


def _per_view_fp32_step(vols32, views, target):
    """The FP32 one-view-per-launch form: a forward and a backward launch
    per view, gradients into one set of buffers per volume."""
    targets, off = [], 0
    for w in views:
        targets.append(target[off:off + w.width * w.height])
        off += w.width * w.height
    grads = [(torch.zeros(v.density.shape, device="cuda"), torch.zeros(v.tf.shape, device="cuda"),
              torch.zeros(1, device="cuda")) for v in vols32]
    batches = [dm.Batch([vols32[w.volume]], [dm.View(0, w.width, w.height, w.eye, w.d00, w.du,
                                                      w.dv, w.background)], (16, 8))
               for w in views]

    def body():
        for gd, gt, gs in grads:
            gd.zero_()
            gt.zero_()
            gs.zero_()
        for i, w in enumerate(views):
            img, st = dm.forward(batches[i])
            dm.backward(batches[i], st, 2.0 * (img - targets[i]), grads=[grads[w.volume]])
    return body, grads


def _per_view_fp32_fused_step(vols32, views, target):
    """The FP32 one-launch-per-view form of the fused step: one plan per
    view, one Plan.step_l2 launch each."""
    plans, off = [], 0
    for w in views:
        b = dm.Batch([vols32[w.volume]], [dm.View(0, w.width, w.height, w.eye, w.d00, w.du, w.dv,
                                                   w.background)], (16, 8))
        p = dm.Plan(b)
        plans.append((p, target[off:off + w.width * w.height].contiguous()))
        off += w.width * w.height

    def body():
        for p, t in plans:
            for gd, gt, gs in p.grads:
                gd.zero_()
                gt.zero_()
                gs.zero_()
            p.step_l2(t, image=False)

    def release():
        for p, _ in plans:
            p.release()
    return body, release


def _targets(target_vols, views):
    """Target images of the L2 loss: every view rendered (FP32) from the
    second seeded volume of its slot."""
    img, _ = dm.forward(dm.Batch(target_vols, views, (16, 8)))
    return img


def _dm_measure(workload, vols, dens32, targets, views, steps, warmup, fp32_steps,
                with_cpu=True):
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    target = _targets(targets, views)
    # the launch search (tile shape, then blocks per SM x tiles per queue
    # fetch) times a forward + backward of about 96 views spread over the
    # whole set (every k-th view), two repetitions each
    sub = views[::max(1, len(views) // 96)]
    launch = dm.autotune_launch(vols, [dm.View(w.volume, w.width, w.height, w.eye, w.d00, w.du,
                                               w.dv, w.background) for w in sub], reps=2,
                                fused=True)
    tile = launch.tile
    shape = (launch.blocks_per_sm, launch.tiles_per_fetch)
    p, graph = _batched_step(vols, views, tile, target, shape)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    tb = _time_steps(graph.replay, steps, warmup, flush)
    clk = clocks.stop()
    nviews = len(views)
    vps = nviews / statistics.median(tb)
    # the same batched step as two launches (forward, torch loss gradient,
    # backward) in one graph, same tile and launch shape
    p2, graph2 = _batched_step(vols, views, tile, target, shape, fused=False)
    t2 = _time_steps(graph2.replay, max(1, min(steps, 5)), 1, flush)
    p2.release()
    del graph2
    # the FP32 one-view-per-launch forms on the same views, from the FP32
    # fields the low-precision copies were made from: forward + torch loss
    # gradient + backward per view with staged gradient accumulation (the
    # library's default) and with one atomic per term, and the fused step
    # as one launch per view
    out = {}
    for name, plain in (("staged", False), ("plain", True)):
        v32 = [dm.VolumeInput(d, v.tf, v.scale, v.step, v.unit, v.value_range, plain=plain)
               for d, v in zip(dens32, vols)]
        body, _ = _per_view_fp32_step(v32, views, target)
        t32 = _time_steps(body, fp32_steps, 1, flush)
        out[name] = nviews / statistics.median(t32)
    v32 = [dm.VolumeInput(d, v.tf, v.scale, v.step, v.unit, v.value_range)
           for d, v in zip(dens32, vols)]
    body, release = _per_view_fp32_fused_step(v32, views, target)
    t32 = _time_steps(body, fp32_steps, 1, flush)
    out["fused"] = nviews / statistics.median(t32)
    release()
    # image and gradient error of the batched low-precision form against
    # the FP32 form (same views, same loss)
    v32 = [dm.VolumeInput(d, v.tf, v.scale, v.step, v.unit, v.value_range)
           for d, v in zip(dens32, vols)]
    b32 = dm.Batch(v32, views, tile)
    img32, st32 = dm.forward(b32)
    g32 = dm.backward(b32, st32, 2.0 * (img32 - target))
    graph.replay()
    torch.cuda.synchronize()
    rms = float(torch.sqrt(torch.mean((p.image - img32) ** 2)))
    gnum = sum(float(torch.sum((a[0] - b[0]) ** 2)) for a, b in zip(p.grads, g32))
    gden = sum(float(torch.sum(b[0] ** 2)) for b in g32)
    grel = (gnum / max(gden, 1e-30)) ** 0.5
    dens_bytes = sum(v.density.numel() * v.density.element_size() for v in vols)
    peaks = measured_peaks()
    # compulsory bytes per step: the density read by the forward and again
    # by the backward, the FP32 density gradient written, the image written
    # and the target read
    comp = 2 * dens_bytes + sum(v.density.numel() * 4 for v in vols) + p.image.numel() * 4 * 2
    line = {
        "metric": "views/s (fwd+bwd)", "value": round(vps, 2), "unit": "views/s",
        "steps": steps, "warmup": warmup, "ms_per_step": round(1000 * statistics.median(tb), 3),
        "dtype": {torch.float16: "f16", torch.bfloat16: "bf16"}.get(vols[0].density.dtype, "f32"),
        "config": {"workload": workload, "tile": list(tile),
                   "blocks_per_sm": launch.blocks_per_sm,
                   "tiles_per_fetch": launch.tiles_per_fetch, "pixels": int(p.batch.pixels),
                   "views": nviews, "l2": "flushed between steps (256 MiB)"},
        "step": "one launch: forward, L2 loss gradient and backward fused (Plan.step_l2)",
        "batched_two_launch_views_per_s": round(nviews / statistics.median(t2), 2),
        "fp32_per_view_staged_views_per_s": round(out["staged"], 2),
        "fp32_per_view_plain_views_per_s": round(out["plain"], 2),
        "fp32_per_view_fused_views_per_s": round(out["fused"], 2),
        "speedup_vs_fp32_per_view_staged": round(vps / out["staged"], 2),
        "speedup_vs_fp32_per_view_plain": round(vps / out["plain"], 2),
        "speedup_vs_fp32_per_view_fused": round(vps / out["fused"], 2),
        "image_rms_vs_fp32": rms,
        "density_grad_rel_err_vs_fp32": grel,
        "gpu_launches": steps,
        "roofline": _roofline(comp, statistics.median(tb), peaks, kernel="k_dmBackward<T, fused>",
                              algorithmic_bytes_per_launch=comp,
                              note="compulsory bytes per step; the march is issue-bound"),
        "clocks": clk,
    }
    p.release()
    return line, target


def measure_dm(local=0, steps=10, warmup=3, views=128, with_cpu=True):
    torch.cuda.set_device(local)
    vol, d32, tgt, vws = _dm_problem(views=views)
    line, target = _dm_measure(f"dm256_fp16_{len(vws)}views_512x512", [vol], [d32], [tgt], vws,
                               steps, warmup, max(1, min(steps, 3)))
    # end to end through the autograd API: FP16 density and TF copied from
    # pinned host memory, forward + loss + backward, the loss and the
    # density gradient read back
    hd = vol.density.cpu().pin_memory()
    ht = vol.tf.cpu().pin_memory()
    tile = tuple(line["config"]["tile"])
    e2e = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d = hd.to("cuda", non_blocking=True).requires_grad_()
        tf = ht.to("cuda", non_blocking=True).requires_grad_()
        v = dm.VolumeInput(d, tf, vol.scale, 0.5, 1.0, (0.0, 1.0))
        img = dm.render(dm.Batch([v], vws, tile))
        loss = torch.sum((img - target) ** 2)
        loss.backward()
        lv = float(loss.item())
        gcpu = d.grad.cpu()
        t1 = time.perf_counter()
        if i:
            e2e.append(len(vws) / (t1 - t0))
    line["e2e"] = {"value": round(statistics.median(e2e), 2), "unit": "views/s",
                   "h2d_bytes_per_step": int(hd.numel() * 2 + ht.numel() * 4),
                   "d2h_bytes_per_step": int(gcpu.numel() * gcpu.element_size() + 4),
                   "includes": "density + TF upload, forward, loss, backward through the "
                               "autograd Function, loss and density-gradient read-back",
                   "loss": lv}
    if with_cpu:
        line["cpu_baseline"] = cpu_dm(vol, vws[0])
    return line


def cpu_dm(vol, view, rows=32):
    """The FP64 oracle forward + adjoint on a band of rows of one view,
    all host threads; views/s scaled from the band's pixels."""
    from oracle import oracle as O

    d = vol.density.float().cpu().numpy()
    tf = vol.tf.cpu().numpy()
    r0 = view.height // 2 - rows // 2
    d00 = tuple(np.asarray(view.d00) + r0 * np.asarray(view.dv))
    vw = {"width": view.width, "height": rows, "eye": view.eye, "d00": d00, "du": view.du,
          "dv": view.dv, "background": view.background}
    g = np.ones((rows, view.width, 3))
    cores = _cores()
    t0 = time.perf_counter()
    O.dm(d, tf, vw, 1.0, 0.5, 1.0, (0.0, 1.0), grad_image=g, threads=cores)
    dt = time.perf_counter() - t0
    frac = rows / view.height
    return {"value": round(frac / dt, 4), "unit": "views/s", "cores": cores, "kind": "port",
            "sample": f"FP64 forward + adjoint, rows {r0}-{r0 + rows} of one "
                      f"{view.width}x{view.height} view ({dt:.1f} s), scaled to the view"}


def measure_batched(local=0, steps=3, warmup=3, with_cpu=True):
    torch.cuda.set_device(local)
    rng = S.Rng(5, stream=17)
    vols, dens32, tgts, views = [], [], [], []
    res_choices = [256, 512, 1024]
    for i in range(64):
        dims = tuple(int(x) for x in rng.uniform(3, 64, 385).astype(int))
        d = S.gaussian_blobs(dims, 16, 100 + i, device="cuda", sigma_scale=max(dims) / 512)
        color, op = S.tf_knots(100 + i, max_opacity=0.25)
        tf = torch.tensor(S.tf_table(color, op, 256), device="cuda")
        scale = torch.tensor([1.0], device="cuda")
        vols.append(dm.VolumeInput(d.to(torch.bfloat16).contiguous(), tf, scale, 0.5, 1.0,
                                   (0.0, 1.0)))
        dens32.append(d)
        t = S.gaussian_blobs(dims, 16, 5000 + i, device="cuda", sigma_scale=max(dims) / 512)
        tgts.append(dm.VolumeInput(t, tf, scale, 0.5, 1.0, (0.0, 1.0)))
        nv = int(rng.uniform(1, 4, 33)[0])
        dirs = S.fibonacci_sphere(nv)
        for k in range(nv):
            w = res_choices[int(rng.uniform(1, 0, 3)[0])]
            h = res_choices[int(rng.uniform(1, 0, 3)[0])]
            views.append(dm.look_at_view(i, vols[-1].dims, 2.0 * dirs[k], 45.0, w, h))
    line, target = _dm_measure(f"batched64_bf16_{len(views)}views_uneven", vols, dens32, tgts,
                               views, steps, warmup, 1)
    del dens32, tgts
    torch.cuda.empty_cache()
    # end to end through the autograd API: the 64 BF16 densities and TFs
    # copied from pinned host memory, forward + loss + backward over all
    # views in one batch, the loss and every density gradient read back
    hds = [v.density.cpu().pin_memory() for v in vols]
    hts = [v.tf.cpu().pin_memory() for v in vols]
    tile = tuple(line["config"]["tile"])
    e2e = []
    for i in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ins, ts = [], []
        for hd, ht, v in zip(hds, hts, vols):
            d = hd.to("cuda", non_blocking=True).requires_grad_()
            tf = ht.to("cuda", non_blocking=True).requires_grad_()
            ins.append(dm.VolumeInput(d, tf, v.scale, 0.5, 1.0, (0.0, 1.0)))
            ts += [d, tf]
        img = dm.render(dm.Batch(ins, views, tile))
        loss = torch.sum((img - target) ** 2)
        loss.backward()
        lv = float(loss.item())
        grads = [t.grad.cpu() for t in ts[0::2]]
        t1 = time.perf_counter()
        if i:
            e2e.append(len(views) / (t1 - t0))
        del ins, ts, img, loss
    line["e2e"] = {"value": round(statistics.median(e2e), 2), "unit": "views/s",
                   "h2d_bytes_per_step": int(sum(h.numel() * 2 for h in hds)
                                             + sum(h.numel() * 4 for h in hts)),
                   "d2h_bytes_per_step": int(sum(g.numel() * g.element_size() for g in grads) + 4),
                   "includes": "64 densities + TFs uploaded, forward, loss, backward through the "
                               "autograd Function, loss and density-gradient read-back",
                   "loss": lv}
    if with_cpu:
        v0 = next(w for w in views if w.volume == 0)
        line["cpu_baseline"] = cpu_dm(vols[0], v0, rows=min(32, v0.height))
    del vols, grads, hds, hts
    torch.cuda.empty_cache()
    return line


# ---------------------------------------------------------------------------
# `python bench.py --workload <name>`: one workload's line alone
# ---------------------------------------------------------------------------

def _print(line, ws):
    full = {"n_gpus": ws, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic"}
    full.update(line)
    print(json.dumps(full), flush=True)


def run(name, args, ws, rank, local):
    torch.cuda.set_device(local)
    import __graft_entry__ as g

    g.build()
    if rank != 0:
        return
    if name == "soup":
        _print(measure_soup(local, args.steps, args.warmup), ws)
    elif name == "volume":
        _print(measure_volume(local, args.steps, args.warmup), ws)
    elif name == "nanovdb":
        _print(measure_nanovdb(local, args.steps, args.warmup, args.nvdb_type), ws)
    elif name == "dm":
        _print(measure_dm(local, args.steps, args.warmup, args.dm_views), ws)
    elif name == "batched":
        _print(measure_batched(local, args.steps, args.warmup), ws)
