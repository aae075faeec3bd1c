"""Benchmark of the hot path on one GB300 (or N, one process per GPU).

Headline workload (one "step" = one frame): 64 instances of a 1.31M-triangle
displaced icosphere (subdivision 8) + 1M spheres, 1920x1080, 64 samples per
pixel, 16 AO rays per hit, renderer "ao", FP32 -- the instanced-geometry +
AO configuration. Metric: Mrays/s (primary + AO rays traced, counted on the
device).

At N=1 the same JSON line also carries, under "workloads", the other
configurations' metrics measured in the same run (bench_workloads.py): the
100k-triangle soup with the "default" renderer (Mrays/s), the 512^3 volume
(Msamples/s), the differentiable marcher on 128 views of a 256^3 FP16
volume and the batched uneven 64-volume set (forward + backward views/s
against the FP32 one-view-per-launch forms), each with its roofline,
end-to-end figure and CPU-oracle baseline. --headline-only skips them.

Arms:
  ours (default)     libvrtx through its C ABI; `value` from the device
                     duration of each frame (CUDA events on the library's
                     stream), L2 flushed between frames; `e2e` re-creates
                     the scene from host arrays every step (upload, BVH
                     builds, render, colour read-back).
  --impl reference   the reference's algorithm on the host cores: the CPU
                     oracle (a restatement of VisRTX's integrator; VisRTX
                     itself needs OptiX + the ANARI-SDK and cannot be built
                     here), each step the band of rows REF_ROWS at 1 spp --
                     the same sample as the `cpu_baseline` leg of ours.

Multi-GPU (torchrun): every rank renders its own frame of the same workload
(weak scaling, no collective on the data path); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s"
WORKLOAD = "instanced64_icosphere_s8_1Mspheres_1920x1080_64spp_ao16"
# the CPU sample of the headline workload: these rows of the 1920x1080
# frame at 1 spp (16 AO rays per hit), for the reference arm and the
# cpu_baseline leg alike
REF_ROWS = (476, 604)


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--spp", type=int, default=64)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workload", default="instanced",
                   choices=["instanced", "soup", "volume", "nanovdb", "dm", "batched"],
                   help="instanced (default line) | soup | volume | nanovdb | dm | batched")
    p.add_argument("--headline-only", action="store_true",
                   help="skip the other workloads in the N=1 line")
    p.add_argument("--nvdb-type", default="fp16", choices=["float", "fp4", "fp8", "fp16", "fpn"])
    p.add_argument("--dm-views", type=int, default=128)
    p.add_argument("--size", default="1920x1080",
                   help="frame size of the default line's scene (a smaller frame for profiling)")
    p.add_argument("--lib", default=None,
                   help="libvrtx.so to load (a tuning variant from python -m visrtx_gb300.build --lib)")
    return p.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(name: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/<name>.json), scaled to one full frame there."""
    p = os.path.join(ROOT, "profiles", name + ".json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f).get("dram_bytes_per_launch")


def trace_bytes(st: dict) -> float:
    """Demand bytes of the AO any-hit kernel: per ray its 32-byte queue
    record read and a 4-byte weighted result written, then the same
    per-node / per-primitive / per-BLAS-entry bytes as algorithmic_bytes."""
    return (st["rays"] * 36.0 + st["nodes"] * 80.0 + st["tri_tests"] * 36.0
            + st["sphere_tests"] * 16.0 + st["blas_entries"] * 48.0)


def algorithmic_bytes(st: dict) -> float:
    """Demand bytes of one frame: per ray a 32-byte ray + 20 bytes of output,
    80 bytes per BVH8 node visited, 36 per triangle tested (3 vertices), 16
    per sphere tested (centre + radius), 48 per BLAS entry (instance
    transform)."""
    return (st["rays"] * 52.0 + st["nodes"] * 80.0 + st["tri_tests"] * 36.0
            + st["sphere_tests"] * 16.0 + st["blas_entries"] * 48.0)


def cpu_sample(sc, spec, cores):
    """Renders REF_ROWS of the 1-spp oracle scene; returns (rays, seconds)."""
    t0 = time.perf_counter()
    o = sc.render(rows=REF_ROWS, threads=cores)
    return o["rays"], time.perf_counter() - t0


def ref_sample_text(steps: int) -> str:
    return (f"rows {REF_ROWS[0]}-{REF_ROWS[1]} of 1920x1080 at 1 spp (AO 16) per step, "
            f"oracle BVH prebuilt; the workload's 64 spp scale linearly")


def run_reference(args, ws, rank):
    """The CPU restatement of the reference integrator, all host threads,
    each step the rows REF_ROWS at 1 spp (AO 16) of the same workload."""
    if rank != 0:
        return
    from oracle import oracle as O
    from visrtx_gb300 import scenes as S

    spec = S.instanced_spec(spp=1)
    sc = O.OracleScene(spec)
    cores = os.cpu_count() or 1
    for _ in range(max(0, args.warmup)):
        sc.render(rows=(REF_ROWS[0], REF_ROWS[0] + 8), threads=cores)
    rays = 0
    secs = 0.0
    for _ in range(args.steps):
        r, dt = cpu_sample(sc, spec, cores)
        rays += r
        secs += dt
    sc.release()
    value = rays / secs / 1e6
    sample = ref_sample_text(args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": METRIC,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "renderer": "ao", "sample": sample},
        "cpu_baseline": {"value": round(value, 4), "unit": METRIC, "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def build_scene(dev, spec):
    from visrtx_gb300 import _lib as L
    from visrtx_gb300 import scenes as S

    frame, world, keep = S.build_on_device(dev, spec, channels=("color", "depth"))
    ren = frame._keep["renderer"]
    ren.set("sampleLimit", 0)
    ren.commit()
    return frame, world, keep


def main():
    args = _args()
    ws, rank, local = _dist()
    if args.workload != "instanced":
        import bench_workloads as BW

        BW.run(args.workload, args, ws, rank, local)
        return
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import torch

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as g

    if args.lib is None and (
            rank == 0 or not os.path.exists(os.path.join(ROOT, "visrtx_gb300", "lib", "libvrtx.so"))):
        g.build()  # a --lib variant is built beforehand (python -m visrtx_gb300.build --lib)
    if ws > 1:
        torch.distributed.barrier()
    from visrtx_gb300 import anari
    from visrtx_gb300 import scenes as S

    width, height = (int(v) for v in args.size.split("x"))
    spec = S.instanced_spec(spp=args.spp, width=width, height=height)
    dev = anari.Device(local, lib_path=args.lib)
    assert dev.is_valid(), dev.errors()
    frame, world, keep = build_scene(dev, spec)

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def one_frame():
        flush.zero_()
        torch.cuda.synchronize()
        frame.render()
        frame.wait()
        return frame.get_property("duration", 240), frame.stats(), frame.kernel_ms(), \
            frame.kernel_launches(), frame.ao_trace()["ms"]

    for _ in range(args.warmup):
        one_frame()
    if dev.errors():
        raise RuntimeError("; ".join(dev.errors()))
    # the world (BLASes + TLAS) is built on the first render after commit
    build_ms = float(dev.lib.vrtxWorldBuildMilliseconds(dev.h, world.handle))

    clocks = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    durs, rays, kms, tms, launches = [], 0, [], [], 0
    for _ in range(args.steps):
        d, st, km, nl, tm = one_frame()
        durs.append(d)
        rays += st["rays"]
        kms.append(km)
        tms.append(tm)
        launches += nl
        assert st["error_flags"] == 0, st
    torch.cuda.synchronize()
    clk = clocks.stop()
    secs = float(sum(durs))
    if ws > 1:
        t = torch.tensor([secs, float(rays)], device="cuda", dtype=torch.float64)
        mx = t.clone()
        torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
        secs_max, rays_all = float(mx[0]), float(t[1])
    else:
        secs_max, rays_all = secs, float(rays)
    value = rays_all / secs_max / 1e6

    # counting pass (untimed): node visits / primitive tests of one frame
    frame.set("vrtx.countTraversal", True)
    frame.commit()
    frame.render()
    frame.wait()
    cst = frame.stats()
    tst = frame.ao_trace()
    frame.set("vrtx.countTraversal", False)
    frame.commit()

    # roofline of the dominant kernel, the AO any-hit kernel (one launch per
    # sample over the compacted AO ray queue), timed with CUDA events around
    # each of its launches on the library stream
    peaks = measured_peaks()
    k_ms = statistics.mean(kms)
    trace_launch_ms = statistics.mean(tms) / args.spp
    trace_launch_bytes = trace_bytes(tst) / args.spp
    achieved = trace_launch_bytes / (trace_launch_ms / 1e3) / 1e9
    traffic = profile_traffic("k_aoTrace_" + WORKLOAD)
    frame_bytes = algorithmic_bytes(cst) * (rays / args.steps) / max(cst["rays"], 1)
    roofline = {"bound": "hbm", "kernel": "k_aoTrace", "achieved": round(achieved, 1),
                "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / peaks["hbm_gbs"], 4),
                "traffic": traffic, "peak_source": peaks["source"],
                "algorithmic_bytes_per_launch": trace_launch_bytes,
                "launch_ms": round(trace_launch_ms, 4),
                "share_of_frame_kernel_time": round(statistics.mean(tms) / k_ms, 4),
                "nodes_per_ray": round(tst["nodes"] / max(tst["rays"], 1), 2),
                "per_launch": {k: tst[k] / args.spp for k in ("rays", "nodes", "tri_tests",
                                                              "sphere_tests", "blas_entries")},
                "frame": {"achieved": round(frame_bytes / (k_ms / 1e3) / 1e9, 1),
                          "algorithmic_bytes": frame_bytes, "kernel_ms": round(k_ms, 3)}}

    # end to end through the C ABI with host buffers
    e2e_vals, h2d, d2h = [], 0, 0
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev2 = dev  # same device; every object re-created from host arrays
        fr2, w2, keep2 = build_scene(dev2, spec)
        fr2.render()
        col = fr2.map("channel.color")
        t1 = time.perf_counter()
        st2 = fr2.stats()
        e2e_vals.append(st2["rays"] / (t1 - t0) / 1e6)
        h2d = sum(int(np.asarray(a).nbytes) for a in (
            spec.surfaces[0].vertices, spec.surfaces[0].indices, spec.surfaces[1].vertices,
            spec.surfaces[1].radii)) + 64 * 64
        d2h = int(col.nbytes)
        for o in keep2 + [fr2]:
            o.release()
    e2e = {"value": round(statistics.median(e2e_vals), 3), "unit": METRIC,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "includes": "array upload, BVH builds, 64-spp frame, colour read-back"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline()
    for o in keep + [frame]:
        o.release()
    del flush
    torch.cuda.empty_cache()

    # the other configurations, measured in the same run (N=1 only)
    workloads = None
    if ws == 1 and not args.headline_only:
        import bench_workloads as BW

        n = min(args.steps, 10)
        w = max(3, min(args.warmup, 5))
        workloads = {}
        for name, fn in (("soup100k_512x384_default", lambda: BW.measure_soup(local, n, w)),
                         ("volume512_raycast", lambda: BW.measure_volume(local, n, w)),
                         ("dm256_fp16_128views", lambda: BW.measure_dm(local, n, w)),
                         ("batched64_bf16_uneven", lambda: BW.measure_batched(local, 2, 3))):
            t0 = time.perf_counter()
            workloads[name] = fn()
            workloads[name]["wall_s"] = round(time.perf_counter() - t0, 1)
            torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * secs_max / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD.replace("1920x1080", args.size), "renderer": "ao",
                       "spp": args.spp, "ao_samples": 16, "width": width, "height": height,
                       "l2": "flushed between frames (256 MiB)",
                       "bvh_build_ms": round(build_ms, 2)},
            "rays_per_frame": rays / args.steps,
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": e2e,
            "roofline": roofline,
            "cpu_baseline": cpu,
        }
        if workloads:
            line["workloads"] = workloads
        print(json.dumps(line), flush=True)
    dev.release()
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline():
    """The oracle's multithreaded C++ tracer on the rows REF_ROWS at 1 spp
    (AO 16), all host threads: the same sample as the reference arm."""
    from oracle import oracle as O
    from visrtx_gb300 import scenes as S

    s1 = S.instanced_spec(spp=1)
    sc = O.OracleScene(s1)
    cores = os.cpu_count() or 1
    sc.render(rows=(REF_ROWS[0], REF_ROWS[0] + 8), threads=cores)
    rays, dt = cpu_sample(sc, s1, cores)
    sc.release()
    return {"value": round(rays / dt / 1e6, 4), "unit": METRIC, "cores": cores,
            "kind": "port", "sample": ref_sample_text(1) + f" ({rays} rays, {dt:.1f} s)"}


if __name__ == "__main__":
    main()
