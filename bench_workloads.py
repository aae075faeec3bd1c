"""Opt-in benchmark workloads beside bench.py's default line (run as
`python bench.py --workload volume|dm|batched`); each prints one JSON line.

  volume   structured-regular 512^3 FP32 volume (64 Gaussian blobs), 256-entry
           TF from 8-knot ramps, 16^3 macrocells, 0.5-voxel steps, 1920x1080
           orbit camera, 1 spp, raycast renderer; Msamples/s (march
           positions, the reference's samples) and Mrays/s.
  nanovdb  the same 512^3 field as a sparse NanoVDB grid (voxels >= 0.02 set;
           --nvdb-type float|fp4|fp8|fp16|fpn, default fp16) through the
           "nanovdb" spatial field, same TF, camera, steps and renderer;
           Msamples/s.
  dm       differentiable marcher: 256^3 FP16 density (32 blobs), 128 views
           of 512x512 on a Fibonacci sphere of radius 2, L2 loss against a
           target rendered from a second volume; forward + backward views/s,
           batched (one graph-captured launch pair, autotuned tiles) against
           the plain FP32 one-view-per-launch form.
  batched  64 volumes with edges U[64,384] (BF16, own TFs), 4-32 views each
           at {256,512,1024}^2; forward + backward views/s, one
           graph-captured launch pair against FP32 one launch per view.
"""
from __future__ import annotations

import json
import math
import os
import statistics
import time

import numpy as np
import torch

from bench import ClockSampler, measured_peaks
from visrtx_gb300 import anari, dm, scenes as S

L2_FLUSH_BYTES = 256 * 1024 * 1024


def _flush(buf):
    buf.zero_()
    torch.cuda.synchronize()


def run_volume(args, ws, rank, local):
    torch.cuda.set_device(local)
    import __graft_entry__ as g

    g.build()
    dev = anari.Device(local)
    field = S.gaussian_blobs((512, 512, 512), 64, 0, device="cuda")
    spec = S.volume_spec(field=field, renderer="raycast", sampling_rate=1.0)
    frame, world, keep = S.build_on_device(dev, spec, channels=("color", "depth"))
    cam = frame._keep["camera"]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def one():
        cam.commit()  # raycast renders one sample per reset (sampleLimit 1)
        _flush(flush)
        frame.render()
        frame.wait()
        return frame.get_property("duration", 240), frame.stats(), frame.kernel_ms()

    for _ in range(args.warmup):
        one()
    clocks = ClockSampler(local)
    clocks.start()
    durs, kms, samples, fetches, rays = [], [], 0, 0, 0
    for _ in range(args.steps):
        d, st, km = one()
        durs.append(d)
        kms.append(km)
        samples += st["volume_samples"]
        fetches += st["volume_fetches"]
        rays += st["rays"]
    clk = clocks.stop()
    secs = sum(durs)
    peaks = measured_peaks()
    # compulsory bytes per frame: the field once (upper bound: every brick
    # touched), majorants, TF, framebuffer writes
    n = 512
    compulsory = n ** 3 * 4 + (n // 16) ** 3 * 4 + 256 * 16 + 1920 * 1080 * 8
    kmean = statistics.mean(kms) / 1e3
    line = {
        "metric": "Msamples/s", "value": round(samples / secs / 1e6, 2), "unit": "Msamples/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "volume512_blobs64_tf256_step0.5_1920x1080_1spp_raycast",
                   "l2": "flushed between frames (256 MiB)"},
        "mrays_per_s": round(rays / secs / 1e6, 2),
        "samples_per_frame": samples / args.steps,
        "fetched_fraction": round(fetches / max(samples, 1), 4),
        "roofline": {"bound": "hbm", "achieved": round(compulsory / kmean / 1e9, 1),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(compulsory / kmean / 1e9 / peaks["hbm_gbs"], 4),
                     "traffic": None, "algorithmic_bytes_per_launch": compulsory},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    dev.release()


def run_nanovdb(args, ws, rank, local):
    torch.cuda.set_device(local)
    import __graft_entry__ as g

    from visrtx_gb300 import nanovdb as NV

    g.build()
    dev = anari.Device(local)
    field = S.gaussian_blobs((512, 512, 512), 64, 0, device="cuda").cpu().numpy()
    t0 = time.time()
    grid = NV.build_grid(field, field >= 0.02, grid_type=args.nvdb_type)
    build_s = time.time() - t0
    info = NV.grid_info(grid)
    del field
    spec = S.nanovdb_volume_spec(grid, renderer="raycast", sampling_rate=1.0)
    frame, world, keep = S.build_on_device(dev, spec, channels=("color", "depth"))
    cam = frame._keep["camera"]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def one():
        cam.commit()
        _flush(flush)
        frame.render()
        frame.wait()
        return frame.get_property("duration", 240), frame.stats(), frame.kernel_ms()

    for _ in range(args.warmup):
        one()
    clocks = ClockSampler(local)
    clocks.start()
    durs, kms, samples, rays = [], [], 0, 0
    for _ in range(args.steps):
        d, st, km = one()
        durs.append(d)
        kms.append(km)
        samples += st["volume_samples"]
        rays += st["rays"]
    clk = clocks.stop()
    secs = sum(durs)
    peaks = measured_peaks()
    compulsory = int(grid.size) + 256 * 16 + 1920 * 1080 * 8  # the grid once, TF, framebuffer
    kmean = statistics.mean(kms) / 1e3
    line = {
        "metric": "Msamples/s", "value": round(samples / secs / 1e6, 2), "unit": "Msamples/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"nanovdb512_{args.nvdb_type}_blobs64_tf256_step0.5_1920x1080"
                               "_1spp_raycast",
                   "grid_bytes": int(grid.size), "active_voxels": info["voxels"],
                   "leaves": info["leaves"], "grid_build_s": round(build_s, 1),
                   "l2": "flushed between frames (256 MiB)"},
        "mrays_per_s": round(rays / secs / 1e6, 2),
        "samples_per_frame": samples / args.steps,
        "roofline": {"bound": "hbm", "achieved": round(compulsory / kmean / 1e9, 1),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(compulsory / kmean / 1e9 / peaks["hbm_gbs"], 4),
                     "traffic": None, "algorithmic_bytes_per_launch": compulsory},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    dev.release()


def _dm_problem(n=256, views=128, res=512, dtype=torch.float16, seed=0):
    d = S.gaussian_blobs((n, n, n), 32, seed, device="cuda")
    color, op = S.tf_knots(seed, max_opacity=0.25)
    tf = torch.tensor(S.tf_table(color, op, 256), device="cuda")
    scale = torch.tensor([1.0], device="cuda")
    vol = dm.VolumeInput(d.to(dtype).contiguous(), tf, scale,
                         step=0.5, unit=1.0, value_range=(0.0, 1.0))
    vol32 = dm.VolumeInput(d, tf, scale, step=0.5, unit=1.0, value_range=(0.0, 1.0), plain=True)
    tgt = dm.VolumeInput(S.gaussian_blobs((n, n, n), 32, seed + 1, device="cuda"), tf, scale,
                         step=0.5, unit=1.0, value_range=(0.0, 1.0))
    dirs = S.fibonacci_sphere(views)
    vws = [dm.look_at_view(0, vol.dims, 2.0 * dirs[i], 45.0, res, res) for i in range(views)]
    return vol, vol32, tgt, vws


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


def _batched_step(vols, views, tile, target):
    """One forward + L2 loss gradient + backward through a plan, captured
    in a CUDA graph."""
    b = dm.Batch(vols, views, tile)
    p = dm.Plan(b)
    grad = torch.empty_like(p.image)

    def body():
        for gd, gt, gs in p.grads:
            gd.zero_()
            gt.zero_()
            gs.zero_()
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
    return p, graph, target


def _per_view_fp32_step(vols32, views, target):
    targets, off = [], 0
    for w in views:
        targets.append(target[off:off + w.width * w.height])
        off += w.width * w.height

    def body():
        for i, w in enumerate(views):
            v = vols32[w.volume]
            b = dm.Batch([v], [dm.View(0, w.width, w.height, w.eye, w.d00, w.du, w.dv,
                                       w.background)], (16, 8))
            img, st = dm.forward(b)
            dm.backward(b, st, 2.0 * (img - targets[i]))
    return body


def _targets(target_vols, views):
    """Target images of the L2 loss: every view rendered (FP32) from the
    second seeded volume of its slot."""
    img, _ = dm.forward(dm.Batch(target_vols, views, (16, 8)))
    return img


def _dm_line(name, workload, vols, vols32, targets, views, args, local):
    torch.cuda.set_device(local)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    target = _targets(targets, views)
    cache = os.path.join(os.path.expanduser("~"), ".cache", "vrtx", "dm_tune.json")
    tile = dm.autotune(vols, views, reps=1, cache=cache)
    p, graph, _ = _batched_step(vols, views, tile, target)
    clocks = ClockSampler(local)
    clocks.start()
    tb = _time_steps(graph.replay, args.steps, args.warmup, flush)
    clk = clocks.stop()
    # the plain FP32 one-view-per-launch form on the same views (the FP32
    # fields the low-precision copies were made from, direct atomics)
    body32 = _per_view_fp32_step(vols32, views, target)
    t32 = _time_steps(body32, max(1, args.steps // 2), 1, flush)
    # image error of the batched low-precision form against FP32
    b32 = dm.Batch(vols32, views, tile)
    img32, _ = dm.forward(b32)
    rms = float(torch.sqrt(torch.mean((p.image - img32) ** 2)))
    nviews = len(views)
    vps = nviews / statistics.median(tb)
    vps32 = nviews / statistics.median(t32)
    dens_bytes = sum(v.density.numel() * v.density.element_size() for v in vols)
    line = {
        "metric": "views/s (fwd+bwd)", "value": round(vps, 2), "unit": "views/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * statistics.median(tb), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {torch.float16: "f16", torch.bfloat16: "bf16"}.get(vols[0].density.dtype, "f32"),
        "data": "synthetic", "config": {"workload": workload, "tile": list(tile),
                                        "pixels": int(p.batch.pixels),
                                        "l2": "flushed between steps (256 MiB)"},
        "fp32_one_view_per_launch_views_per_s": round(vps32, 2),
        "speedup_vs_fp32_per_view": round(vps / vps32, 2),
        "rms_vs_fp32": rms,
        "density_bytes": dens_bytes,
        "clocks": clk,
        "gpu_launches": 2 * 1,
    }
    print(json.dumps(line), flush=True)
    p.release()


def run_dm(args, ws, rank, local):
    torch.cuda.set_device(local)
    import __graft_entry__ as g

    g.build()
    vol, vol32, tgt, views = _dm_problem(views=args.dm_views)
    _dm_line("dm", f"dm256_fp16_{len(views)}views_512x512", [vol], [vol32], [tgt], views, args,
             local)


def run_batched(args, ws, rank, local):
    torch.cuda.set_device(local)
    import __graft_entry__ as g

    g.build()
    rng = S.Rng(5, stream=17)
    vols, vols32, tgts, views = [], [], [], []
    res_choices = [256, 512, 1024]
    for i in range(64):
        dims = tuple(int(x) for x in rng.uniform(3, 64, 385).astype(int))
        d = S.gaussian_blobs(dims, 16, 100 + i, device="cuda", sigma_scale=max(dims) / 512)
        color, op = S.tf_knots(100 + i, max_opacity=0.25)
        tf = torch.tensor(S.tf_table(color, op, 256), device="cuda")
        scale = torch.tensor([1.0], device="cuda")
        vols.append(dm.VolumeInput(d.to(torch.bfloat16).contiguous(), tf, scale, 0.5, 1.0,
                                   (0.0, 1.0)))
        vols32.append(dm.VolumeInput(d, tf, scale, 0.5, 1.0, (0.0, 1.0), plain=True))
        t = S.gaussian_blobs(dims, 16, 5000 + i, device="cuda", sigma_scale=max(dims) / 512)
        tgts.append(dm.VolumeInput(t, tf, scale, 0.5, 1.0, (0.0, 1.0)))
        nv = int(rng.uniform(1, 4, 33)[0])
        dirs = S.fibonacci_sphere(nv)
        for k in range(nv):
            w = res_choices[int(rng.uniform(1, 0, 3)[0])]
            h = res_choices[int(rng.uniform(1, 0, 3)[0])]
            views.append(dm.look_at_view(i, vols[-1].dims, 2.0 * dirs[k], 45.0, w, h))
    _dm_line("batched", f"batched64_bf16_{len(views)}views_uneven", vols, vols32, tgts, views,
             args, local)
