"""Generates tests/golden/math_golden.npz: the reference's own gpu_math.h
helpers on the thin-lens and HDRI paths, compiled unchanged on the host
(oracle/ref_tf.cpp): uniformSampleDisk (gpu/gpu_math.h:292-297, the
aperture sample of cameraCreateRay.h:52) on seeded (radius, s0, s1) and
sphericalCoordsFromDirection (gpu/gpu_math.h:254-261, the HDRI lookup of
gpu_util.h:283) on seeded unit directions plus the poles, the axes and
directions on the phi = 0 seam from both sides, and uniformSampleCone
(gpu/gpu_math.h:299-312, the physically based material's next ray,
PhysicallyBasedShader_ptx.cu:75) on seeded (cosThetaMax, s0, s1, s2), and
projectOnGrid (gpu/uniformGrid.h:43-50, the macrocell projection of the
delta-tracking grid and its DDA) of points inside seeded boxes, faces
included, onto grids of 1 to 40 cells per axis.

Run in a tree that holds the reference (it builds oracle/_ref/libtfref.so
from the reference's headers):  python tests/golden/make_math_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def inputs(seed=7):
    rng = np.random.default_rng(seed)
    disk = np.stack([rng.uniform(0.0, 2.0, 2000), rng.uniform(0.0, 1.0, 2000),
                     rng.uniform(0.0, 1.0, 2000)], axis=1)
    disk = np.concatenate([disk, [[1.0, 0.0, 0.0], [1.0, 1.0, 0.5], [0.5, 0.25, 1.0]]])
    d = rng.normal(size=(2000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    edge = np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
                     [1, 1e-7, 0], [1, -1e-7, 0], [-1, 1e-7, 0], [-1, -1e-7, 0],
                     [0.6, 0.0, 0.8], [0.6, -0.0, -0.8]], np.float64)
    cone = np.stack([rng.uniform(-1.0, 1.0, 2000), rng.uniform(0.0, 1.0, 2000),
                     rng.uniform(0.0, 1.0, 2000), rng.uniform(0.0, 1.0, 2000)], axis=1)
    cone = np.concatenate([cone, [[1.0, 0.0, 0.0, 0.0], [0.0, 0.5, 1.0, 1.0]]])
    grids = []
    for _ in range(40):
        dims = rng.integers(1, 41, 3).astype(np.int32)
        lo = rng.uniform(-50, 50, 3)
        hi = lo + rng.uniform(0.5, 100, 3)
        pts = lo + rng.uniform(0, 1, (50, 3)) * (hi - lo)
        pts = np.concatenate([pts, [lo, hi, np.where([1, 0, 1], lo, hi)]])
        grids.append((dims, np.concatenate([lo, hi]).astype(np.float32), pts.astype(np.float32)))
    return (disk.astype(np.float32), np.concatenate([d, edge]).astype(np.float32),
            cone.astype(np.float32), grids)


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_TF_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_TF_LIB)
    for f in (lib.mathref_uniform_sample_disk, lib.mathref_spherical_from_dir,
              lib.mathref_uniform_sample_cone):
        f.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        f.restype = None
    disk, dirs, cone, grids = inputs()
    d_out = np.zeros((len(disk), 2), np.float32)
    s_out = np.zeros((len(dirs), 2), np.float32)
    lib.mathref_uniform_sample_disk(disk.ctypes.data, len(disk), d_out.ctypes.data)
    lib.mathref_spherical_from_dir(dirs.ctypes.data, len(dirs), s_out.ctypes.data)
    c_out = np.zeros((len(cone), 3), np.float32)
    lib.mathref_uniform_sample_cone(cone.ctypes.data, len(cone), c_out.ctypes.data)
    lib.mathref_project_on_grid.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_void_p]
    lib.mathref_project_on_grid.restype = None
    g_arr = {}
    for k, (dims, box, pts) in enumerate(grids):
        cells = np.zeros((len(pts), 3), np.int32)
        lib.mathref_project_on_grid(pts.ctypes.data, len(pts), dims.ctypes.data, box.ctypes.data,
                                    cells.ctypes.data)
        g_arr[f"grid{k}_dims"] = dims
        g_arr[f"grid{k}_box"] = box
        g_arr[f"grid{k}_points"] = pts
        g_arr[f"grid{k}_cells"] = cells
    np.savez_compressed(os.path.join(HERE, "math_golden.npz"), disk_in=disk, disk_out=d_out,
                        dir_in=dirs, dir_out=s_out, cone_in=cone, cone_out=c_out,
                        grids=np.asarray([len(grids)]), **g_arr)
    print("wrote", os.path.join(HERE, "math_golden.npz"), len(disk), "disk samples,",
          len(dirs), "directions,", len(cone), "cone samples")


if __name__ == "__main__":
    main()
