"""Generates tests/golden/dda_golden.npz: the cells and intervals the
reference's own macrocell walk (devices/rtx/gpu/dda.h:43-122, dda3, the walk
of the delta-tracking march in gpu/volumeIntegration.h) visits, compiled on
the host with contraction on, as nvcc builds it (oracle/ref_dda.cpp).

Cases: a non-cubic grid over an off-centre box with random directions and
directions with one or two zero components (the walk's axis-aligned quirk:
a zero component walks that axis down to -1 at t = 0); a power-of-two grid
over the unit cube from exact face, edge and corner points along diagonals
(ties between axes, which step two or three axes at once); a one-cell grid;
a large grid with [tlo, thi] inside the box and negative tlo; origins just
outside the box (clamped by projectOnGrid); walks cut short by the
callback (maxCells 3).

Run in a tree that holds the reference (it builds oracle/_ref/libddaref.so
from the reference's headers):  python tests/golden/make_dda_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def _unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def cases(seed=11):
    rng = np.random.default_rng(seed)
    out = []

    # 1. non-cubic grid, off-centre box, random and partly axis-aligned rays
    dims = (13, 7, 29)
    box = np.array([-1.5, 0.25, -3.0, 2.0, 1.75, 4.5], np.float32)
    n = 600
    org = box[:3] + rng.uniform(0, 1, (n, 3)) * (box[3:] - box[:3])
    d = _unit(rng.normal(size=(n, 3)))
    d[:60, 0] = 0.0
    d[60:100, 1] = 0.0
    d[100:130, 2] = 0.0
    d[130:140, :2] = 0.0
    d[140:150, 1:] = 0.0
    d[:150] = _unit(np.where(np.abs(d[:150]).sum(1, keepdims=True) == 0, 1.0, d[:150]))
    t = np.stack([np.zeros(n), np.full(n, 1e30)], 1)
    out.append((dims, box, np.concatenate([org, d, t], 1), sum(dims) + 2))

    # 2. power-of-two grid over the unit cube: exact faces, edges, corners,
    # diagonal and axis-pair directions (ties between axes)
    dims = (16, 16, 16)
    box = np.array([0, 0, 0, 1, 1, 1], np.float32)
    grid = np.array([0.0, 0.0625, 0.25, 0.5, 0.9375, 1.0])
    pts = np.array(np.meshgrid(grid, grid, grid, indexing="ij")).reshape(3, -1).T
    signs = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)], float)
    dirs = np.concatenate([signs, signs * [1, 1, 0], signs * [1, 0, 1], signs * [2, 1, 1]])
    dirs = _unit(np.unique(dirs, axis=0))
    pick = rng.integers(0, len(dirs), len(pts))
    pts2 = np.repeat(pts, 2, axis=0)
    d2 = np.concatenate([dirs[pick], dirs[(pick + 7) % len(dirs)]])
    d2 = np.stack([d2[:len(pts)], d2[len(pts):]], 1).reshape(-1, 3)
    t = np.stack([np.zeros(len(pts2)), np.full(len(pts2), 1e30)], 1)
    out.append((dims, box, np.concatenate([pts2, d2, t], 1), sum(dims) + 2))

    # 3. one cell
    dims = (1, 1, 1)
    box = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    n = 64
    org = rng.uniform(-1, 1, (n, 3))
    d = _unit(rng.normal(size=(n, 3)))
    t = np.stack([np.zeros(n), np.full(n, 1e30)], 1)
    out.append((dims, box, np.concatenate([org, d, t], 1), 4))

    # 4. large grid, [tlo, thi] inside the box, negative tlo
    dims = (64, 48, 32)
    box = np.array([10.0, -20.0, 0.5, 74.0, 28.0, 32.5], np.float32)
    n = 300
    org = box[:3] + rng.uniform(0, 1, (n, 3)) * (box[3:] - box[:3])
    d = _unit(rng.normal(size=(n, 3)))
    tlo = np.where(rng.uniform(size=n) < 0.3, -rng.uniform(0, 5, n), rng.uniform(0, 10, n))
    thi = tlo + rng.uniform(0.5, 40, n)
    out.append((dims, box, np.concatenate([org, d, np.stack([tlo, thi], 1)], 1), sum(dims) + 2))

    # 5. origins just outside the box (clamped to the border cells)
    dims = (8, 12, 5)
    box = np.array([-2, -3, -1, 2, 3, 1], np.float32)
    n = 200
    org = box[:3] + rng.uniform(-0.2, 1.2, (n, 3)) * (box[3:] - box[:3])
    d = _unit(rng.normal(size=(n, 3)))
    t = np.stack([np.zeros(n), np.full(n, 1e30)], 1)
    out.append((dims, box, np.concatenate([org, d, t], 1), sum(dims) + 2))

    # 6. walks cut short by the callback
    dims = (32, 32, 32)
    box = np.array([0, 0, 0, 4, 4, 4], np.float32)
    n = 200
    org = rng.uniform(0, 4, (n, 3))
    d = _unit(rng.normal(size=(n, 3)))
    t = np.stack([np.zeros(n), np.full(n, 1e30)], 1)
    out.append((dims, box, np.concatenate([org, d, t], 1), 3))
    return [(np.array(dm, np.int32), bx, r.astype(np.float32), mc) for dm, bx, r, mc in out]


def walk(lib, dims, box, rays, max_cells):
    n = len(rays)
    counts = np.zeros(n, np.int32)
    cells = np.full((n, max_cells), -1, np.int64)
    t01 = np.zeros((n, max_cells, 2), np.float32)
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    lib.ddaref_walk(P(rays), C.c_int(n), P(dims), P(box), C.c_int(max_cells),
                    P(counts), P(cells), P(t01))
    keep = np.arange(max_cells)[None, :] < counts[:, None]
    return counts, cells[keep].astype(np.int32), t01[keep]


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_DDA_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_DDA_LIB)
    lib.ddaref_walk.restype = C.c_int
    arrays = {}
    total = 0
    for i, (dims, box, rays, mc) in enumerate(cases()):
        counts, cells, t01 = walk(lib, dims, box, np.ascontiguousarray(rays), mc)
        arrays.update({f"c{i}_dims": dims, f"c{i}_box": box, f"c{i}_rays": rays,
                       f"c{i}_max_cells": np.int32(mc), f"c{i}_counts": counts,
                       f"c{i}_cells": cells, f"c{i}_t01": t01})
        total += int(counts.sum())
    arrays["num_cases"] = np.int32(len(cases()))
    np.savez_compressed(os.path.join(HERE, "dda_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "dda_golden.npz"), total, "cells")


if __name__ == "__main__":
    main()
