"""Generates tests/golden/box_golden.npz: the ray/box intervals of the
reference's own intersectBox (devices/rtx/gpu/gpu_math.h:278-290, the
volume's entry interval in the scivis and dpt marches), compiled on the host
by oracle/ref_tf.cpp (oracle/_ref/libtfref.so).

Rays per box: random origins inside and around the box with random
directions; axis-aligned directions (one or two zero components, +0 and -0,
so 1 / d is +-inf) from inside, outside and exactly on the box's planes
(where (lo - org) * inf is NaN); origins on faces, edges and corners; and
directions pointing away. Five boxes, including a flat one and one with
negative coordinates.

Run in a tree that holds the reference:  python tests/golden/make_box_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

BOXES = np.array([[0, 0, 0, 1, 1, 1],
                  [-3.5, -2.0, -1.25, 4.0, 0.5, 7.75],
                  [10.0, 20.0, 30.0, 10.5, 21.0, 30.25],
                  [-1, -1, 0, 1, 1, 0],  # flat in z
                  [0.1, 0.2, 0.3, 512.0, 384.0, 256.0]], np.float32)


def rays_for(box, rng, n=400):
    lo, hi = box[:3].astype(np.float64), box[3:].astype(np.float64)
    ext = np.maximum(hi - lo, 1e-3)
    org = lo - ext + rng.uniform(0, 3, (n, 3)) * ext
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # axis-aligned directions, +0 and -0 components
    k = n // 4
    d[:k] = 0.0
    axis = rng.integers(0, 3, k)
    d[np.arange(k), axis] = rng.choice([-1.0, 1.0], k)
    d[k:k + 40, 0] = -0.0
    d[k + 40:k + 80, 1] = 0.0
    d[k + 40:k + 80, 2] = -0.0
    # origins exactly on the box's planes, and on faces / edges / corners
    on = slice(2 * k, 2 * k + 60)
    corners = np.stack([np.where(rng.uniform(size=60) < 0.5, lo[a], hi[a]) for a in range(3)], 1)
    mix = rng.uniform(size=(60, 3)) < 0.5
    org[on] = np.where(mix, corners, org[on])
    org[:k][np.arange(k) % 3 == 0, 0] = lo[0]
    org[:k][np.arange(k) % 3 == 1, 1] = hi[1]
    d[2 * k:2 * k + 60][rng.uniform(size=60) < 0.3] *= -1.0
    return np.concatenate([org, d], 1).astype(np.float32)


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_TF_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_TF_LIB)
    lib.mathref_intersect_box.restype = None
    rng = np.random.default_rng(29)
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    arrays = {"boxes": BOXES}
    for i, box in enumerate(BOXES):
        rays = rays_for(box, rng)
        hit = np.zeros(len(rays), np.int32)
        t01 = np.zeros((len(rays), 2), np.float32)
        lib.mathref_intersect_box(P(rays), C.c_int(len(rays)), P(np.ascontiguousarray(box)),
                                  P(hit), P(t01))
        arrays.update({f"b{i}_rays": rays, f"b{i}_hit": hit, f"b{i}_t01": t01})
    np.savez_compressed(os.path.join(HERE, "box_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "box_golden.npz"))


if __name__ == "__main__":
    main()
