"""Generates tests/golden/volume_interval_golden.npz: the volume entry
intervals of the reference's intersectVolume
(devices/rtx/scene/Intersectors_ptx.cu:248-274), its glm and gpu_math.h
calls compiled on the host by oracle/ref_tf.cpp (oracle/_ref/libtfref.so).

Local rays per box, with a ray interval [tmin, tmax]: random origins inside
and around the box with random directions; axis-aligned directions (one or
two zero components, +0 and -0, so 1 / d is +-inf) from inside, outside and
exactly on each of the box's six planes (where (bound - org) * inf is NaN,
in every axis position of the slab vectors); origins on faces, edges and
corners; directions pointing away; intervals that start inside the box or
end before it. Five boxes, including a flat one and one with negative
coordinates.

Run in a tree that holds the reference:
    python tests/golden/make_volume_interval_golden.py
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


def rays_for(box, rng, n=480):
    lo, hi = box[:3].astype(np.float64), box[3:].astype(np.float64)
    ext = np.maximum(hi - lo, 1e-3)
    org = lo - ext + rng.uniform(0, 3, (n, 3)) * ext
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # axis-aligned and plane-parallel directions, +0 and -0 components
    k = n // 4
    d[:k] = 0.0
    d[np.arange(k), rng.integers(0, 3, k)] = rng.choice([-1.0, 1.0], k)
    d[k:k + 40, 0] = -0.0
    d[k + 40:k + 80, 1] = 0.0
    d[k + 40:k + 80, 2] = -0.0
    # origins on each of the six planes, with the direction parallel to it
    # (a NaN slab in that axis), inside the box's extent on the other axes
    m = 2 * k
    for j in range(96):
        a, side = j % 3, (j // 3) % 2
        i = m + j
        org[i] = lo + rng.uniform(0.1, 0.9, 3) * ext
        org[i, a] = (lo if side == 0 else hi)[a]
        dd = rng.normal(size=3)
        dd[a] = 0.0 if j % 4 else -0.0
        d[i] = dd / np.linalg.norm(dd)
    # origins on faces, edges and corners
    on = slice(m + 96, m + 156)
    corners = np.stack([np.where(rng.uniform(size=60) < 0.5, lo[a], hi[a]) for a in range(3)], 1)
    org[on] = np.where(rng.uniform(size=(60, 3)) < 0.5, corners, org[on])
    tmin = np.zeros(n)
    tmax = np.full(n, np.float32(3.4028235e38))
    # intervals that start inside the box or end before it
    tmin[m + 156:m + 200] = rng.uniform(0, 2, 44) * ext.max()
    tmax[m + 200:m + 240] = rng.uniform(0, 1, 40) * ext.max()
    return np.concatenate([org, d, tmin[:, None], tmax[:, None]], 1).astype(np.float32)


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_TF_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_TF_LIB)
    lib.mathref_volume_interval.restype = None
    rng = np.random.default_rng(29)
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    arrays = {"boxes": BOXES}
    for i, box in enumerate(BOXES):
        rays = rays_for(box, rng)
        hit = np.zeros(len(rays), np.int32)
        t01 = np.zeros((len(rays), 2), np.float32)
        lib.mathref_volume_interval(P(rays), C.c_int(len(rays)), P(np.ascontiguousarray(box)),
                                    P(hit), P(t01))
        arrays.update({f"b{i}_rays": rays, f"b{i}_hit": hit, f"b{i}_t01": t01})
    np.savez_compressed(os.path.join(HERE, "volume_interval_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "volume_interval_golden.npz"))


if __name__ == "__main__":
    main()
