"""Sharding logic on CPU: view partitioning, row bands, and the gradient
all-reduce across two gloo ranks giving the single-process sum (per-view
gradients from the FP64 oracle adjoint)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from visrtx_gb300 import shard


def test_partition_views_balanced_and_complete():
    counts = [256 * 256, 512 * 512, 1024 * 1024, 256 * 512, 1024 * 256, 512 * 512, 64 * 64]
    for ws in (1, 2, 3, 4):
        parts = shard.partition_views(counts, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(counts)))
        loads = [sum(counts[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(counts)


def test_row_bands_cover_frame():
    for h in (1, 7, 1080):
        for ws in (1, 2, 3, 8):
            bands = [shard.row_band(h, ws, r) for r in range(ws)]
            assert bands[0][0] == 0 and bands[-1][1] == h
            for (a0, a1), (b0, b1) in zip(bands, bands[1:]):
                assert a1 == b0
            assert max(b - a for a, b in bands) - min(b - a for a, b in bands) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _views():
    from visrtx_gb300 import dm

    out = []
    dirs = [(0.0, 0.0, 2.2), (2.0, 0.5, 0.5), (-1.0, 1.5, 1.0), (0.3, -2.0, 0.4)]
    res = [(10, 8), (6, 12), (12, 10), (8, 8)]
    for d, r in zip(dirs, res):
        v = dm.look_at_view(0, (9, 8, 10), d, 55.0, r[0], r[1], (0.1, 0.2, 0.3))
        out.append({"width": v.width, "height": v.height, "eye": v.eye, "d00": v.d00,
                    "du": v.du, "dv": v.dv, "background": v.background})
    return out


def _problem():
    from visrtx_gb300 import scenes as S

    d = S.gaussian_blobs((9, 8, 10), n_blobs=3, seed=5, sigma_scale=0.1).astype(np.float64)
    c, o = S.tf_knots(5, max_opacity=0.5)
    tf = S.tf_table(c, o, 16).astype(np.float64)
    return d, tf


def _grad_for(views_idx):
    from oracle import oracle as O

    d, tf = _problem()
    views = _views()
    gd = np.zeros_like(d)
    gt = np.zeros_like(tf)
    for i in views_idx:
        v = views[i]
        g = np.full((v["height"], v["width"], 3), 0.25)
        _, a, b, _ = O.dm(d, tf, v, 1.2, 0.5, 1.0, (-0.5, 1.5), grad_image=g, threads=1)
        gd += a
        gt += b
    return gd, gt


def _worker(rank, ws, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    views = _views()
    parts = shard.partition_views([v["width"] * v["height"] for v in views], ws)
    gd, gt = _grad_for(parts[rank])
    tensors = [torch.tensor(gd), torch.tensor(gt)]
    shard.allreduce_gradients(tensors)
    if rank == 0:
        out.put((tensors[0].numpy(), tensors[1].numpy()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gradient_allreduce_equals_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gd, gt = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    rd, rt = _grad_for(range(len(_views())))
    np.testing.assert_allclose(gd, rd, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(gt, rt, rtol=1e-12, atol=1e-15)
