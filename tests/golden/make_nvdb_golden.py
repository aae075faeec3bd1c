"""Generates tests/golden/nvdb_golden.npz: NanoVDB grids built by NanoVDB's
own builder (the library the reference vendors in external/nanovdb) and the
values NanoVDB's first-order sampler returns for them at seeded world-space
points, through the same call sequence the reference's field sampler makes
(gpu/sampleSpatialField.h:80-109).

Run in a tree that holds the reference (it builds oracle/_ref/libnvdbref.so
from the vendored headers):  python tests/golden/make_nvdb_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

# the block every grid is built from: voxel (x, y, z) of `dense` sits at
# index ORIGIN + (x, y, z); it straddles a lower-node boundary in x (128) and
# has negative y indices
DIMS = (23, 14, 19)  # nz, ny, nx
ORIGIN = (118, -5, 40)
VOXEL = 0.25
TRANSLATION = (0.5, -1.0, 2.0)
TYPES = {"float": 1, "fp4": 13, "fp8": 14, "fp16": 15, "fpn": 16}


def block(seed=5):
    """Smooth blobs plus noise in [0, 1]; voxels under 0.15 are left unset."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = DIMS
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    v = np.zeros(DIMS)
    for _ in range(5):
        c = rng.uniform(0, 1, 3) * (nx, ny, nz)
        s = rng.uniform(2.0, 6.0)
        v += rng.uniform(0.3, 1.0) * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
                                            / (2 * s * s))
    v = np.clip(v + rng.normal(0, 0.02, DIMS), 0, 1).astype(np.float32)
    # one constant leaf region, so FpN has 1-bit leaves too
    v[:8, :8, :8] = 0.5
    return v, v >= 0.15


def points(seed=6, n=3000):
    rng = np.random.default_rng(seed)
    nz, ny, nx = DIMS
    lo = np.array(ORIGIN, np.float64) * VOXEL + TRANSLATION
    hi = (np.array(ORIGIN) + (nx, ny, nz)) * VOXEL + np.array(TRANSLATION)
    p = rng.uniform(lo - 2 * VOXEL, hi + 2 * VOXEL, (n, 3))
    # a few exactly on voxel centres
    ijk = rng.integers(0, (nx, ny, nz), (200, 3)) + np.array(ORIGIN)
    p[:200] = ijk * VOXEL + np.array(TRANSLATION)
    return p.astype(np.float32)


def load_ref():
    from oracle import build as ob

    path = ob.build_ref()
    if path is None:
        raise SystemExit("the reference tree is not present")
    lib = C.CDLL(path)
    lib.nvdbref_build.restype = C.c_size_t
    lib.nvdbref_build.argtypes = [C.c_int, C.c_void_p, C.c_void_p] + [C.c_int] * 6 + [
        C.c_float, C.c_double, C.c_void_p, C.c_void_p, C.c_size_t]
    lib.nvdbref_sample.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_int, C.c_void_p]
    lib.nvdbref_validate.argtypes = [C.c_void_p, C.c_size_t]
    return lib


def ref_build(lib, gtype, dense, active):
    a8 = np.ascontiguousarray(active, np.uint8)
    d = np.ascontiguousarray(dense, np.float32)
    t = np.array(TRANSLATION, np.float64)
    nz, ny, nx = d.shape
    args = (gtype, d.ctypes.data, a8.ctypes.data, nx, ny, nz, *ORIGIN, 0.0, VOXEL, t.ctypes.data)
    n = lib.nvdbref_build(*args, None, 0)
    out = np.zeros(n, np.uint8)
    lib.nvdbref_build(*args, out.ctypes.data, n)
    return out


def ref_sample(lib, buf, pts):
    out = np.zeros(len(pts), np.float32)
    p = np.ascontiguousarray(pts, np.float32)
    b = np.ascontiguousarray(buf, np.uint8)
    if lib.nvdbref_sample(b.ctypes.data, b.size, p.ctypes.data, len(p), out.ctypes.data) != 0:
        raise RuntimeError("sampling failed")
    return out


def main():
    lib = load_ref()
    dense, active = block()
    pts = points()
    out = {"dense": dense, "active": active, "points": pts,
           "origin": np.array(ORIGIN), "voxel": np.array(VOXEL),
           "translation": np.array(TRANSLATION)}
    for name, t in TYPES.items():
        buf = ref_build(lib, t, dense, active)
        out[f"grid_{name}"] = buf
        out[f"values_{name}"] = ref_sample(lib, buf, pts)
    np.savez_compressed(os.path.join(HERE, "nvdb_golden.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
