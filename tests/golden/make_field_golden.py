"""Generates tests/golden/field_golden.npz: the texture coordinates at which
the reference's own structured-regular field sampler
(devices/rtx/gpu/sampleSpatialField.h:54-78, with StructuredRegularField's
invSpacing) reads its field texture, compiled on the host by
oracle/ref_field.cpp, for world points inside and around six fields:
unit and non-unit spacings, negative and off-grid origins, one-voxel and
elongated grids, the bench field's 512^3 layout; points on voxel centres,
voxel boundaries, the field's bounds and outside them.

Run in a tree that holds the reference:  python tests/golden/make_field_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

FIELDS = [  # origin, spacing, dims
    ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (48, 48, 48)),
    ((-1.0, -1.0, -1.0), (2.0 / 511, 2.0 / 511, 2.0 / 511), (512, 512, 512)),
    ((10.25, -3.5, 0.125), (0.37, 1.9, 0.05), (13, 7, 29)),
    ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (1, 1, 1)),
    ((-100.0, 50.0, -0.001), (3.0, 0.25, 7.5), (2, 300, 5)),
    ((0.5, 0.5, 0.5), (0.1, 0.1, 0.1), (64, 32, 16)),
]


def points_for(origin, spacing, dims, rng, n=600):
    o = np.asarray(origin, np.float64)
    s = np.asarray(spacing, np.float64)
    d = np.asarray(dims, np.float64)
    hi = o + (d - 1) * s
    pts = [o + rng.uniform(-0.2, 1.2, (n // 3, 3)) * np.maximum(hi - o, s)]
    centres = rng.integers(0, np.maximum(d, 1), (n // 6, 3))
    pts.append(o + centres * s)
    pts.append(o + (centres + 0.5) * s)
    pts.append(np.stack([o, hi, o - s, hi + s]))
    return np.concatenate(pts).astype(np.float32)


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_FIELD_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_FIELD_LIB)
    lib.fieldref_coords.restype = None
    rng = np.random.default_rng(31)
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    arrays = {"num_fields": np.int32(len(FIELDS))}
    for i, (o, s, d) in enumerate(FIELDS):
        o32 = np.asarray(o, np.float32)
        s32 = np.asarray(s, np.float32)
        d32 = np.asarray(d, np.int32)
        pts = points_for(o32, s32, d32, rng)
        out = np.zeros_like(pts)
        lib.fieldref_coords(P(o32), P(s32), P(d32), P(pts), C.c_int(len(pts)), P(out))
        arrays.update({f"f{i}_origin": o32, f"f{i}_spacing": s32, f"f{i}_dims": d32,
                       f"f{i}_points": pts, f"f{i}_coords": out})
    np.savez_compressed(os.path.join(HERE, "field_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "field_golden.npz"))


if __name__ == "__main__":
    main()
