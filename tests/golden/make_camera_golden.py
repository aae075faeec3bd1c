"""Generates tests/golden/camera_golden.npz: primary rays (origin, direction
and screen position) from the reference's own makePrimaryRay /
cameraCreateRay (devices/rtx/gpu/cameraCreateRay.h:38-81), compiled on the
host by oracle/ref_camera.cpp twice: without floating-point contraction
(each operation rounded once, the form the oracle and the library's kernels
compute) and with it (the kind of rounding an nvcc build with its default
-fmad=true gives), so that the gap between the two is on record.

Cases: pinhole perspective cameras, thin-lens cameras (aperture > 0, the
focus distance folded into dir_00 / dir_du / dir_dv) and orthographic
cameras, over the full image region and sub-regions, at 1920x1080, 512x384
and 7x5 frames, with and without the pixel-centre flag; pixels include the
frame's first and last rows and columns, and the uniform draws include
values next to 0 and exactly 1 (curand_uniform's range is (0, 1]).

Run in a tree that holds the reference (it builds oracle/_ref/libcamref.so
and libcamref_fused.so from the reference's headers):
    python tests/golden/make_camera_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

FRAMES = ((1920, 1080), (512, 384), (7, 5))


def camera_record(rng, kind):
    """30 floats: region, pos, dir, dir_00, dir_du, dir_dv, scaledAperture,
    aspect, pos_00, pos_du, pos_dv, for kind 0 pinhole, 1 thin lens,
    2 orthographic."""
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    up = rng.normal(size=3)
    du = np.cross(d, up)
    du /= np.linalg.norm(du)
    dv = np.cross(du, d)
    aspect = rng.uniform(0.5, 2.5)
    ipy = 2.0 * np.tan(0.5 * rng.uniform(0.2, 2.0))
    ipx = ipy * aspect
    pdu, pdv = du * ipx, dv * ipy
    d00 = d - 0.5 * pdu - 0.5 * pdv
    aperture = 0.0
    if kind == 1:
        focus = rng.uniform(0.5, 40.0)
        aperture = rng.uniform(0.01, 2.0) / (ipx * focus)
        pdu, pdv, d00 = pdu * focus, pdv * focus, d00 * focus
    if rng.uniform() < 0.5:
        region = [0.0, 0.0, 1.0, 1.0]
    else:
        x = np.sort(rng.uniform(0, 1, 2))
        y = np.sort(rng.uniform(0, 1, 2))
        region = [x[0], y[0], x[1], y[1]]
    pos = rng.uniform(-100, 100, 3)
    h = rng.uniform(0.5, 20.0)
    odu, odv = du * h * aspect, dv * h
    p00 = pos - 0.5 * odu - 0.5 * odv
    return np.concatenate([region, pos, d, d00, pdu, pdv, [aperture, aspect],
                           p00, odu, odv]).astype(np.float32)


def samples(rng, w, h, n):
    px = rng.integers(0, w, n)
    py = rng.integers(0, h, n)
    px[:4] = [0, w - 1, 0, w - 1]
    py[:4] = [0, 0, h - 1, h - 1]
    r = rng.uniform(0, 1, (n, 4))
    r[4:8] = 1.0
    r[8:12] = np.float32(2.0 ** -24)
    r[r == 0] = 1.0
    return np.concatenate([px[:, None], py[:, None], r], 1).astype(np.float32)


def cases(seed=17, n=220):
    rng = np.random.default_rng(seed)
    out = []
    for kind in (0, 1, 2):
        for w, h in FRAMES:
            for center in (0, 1):
                cam = camera_record(rng, kind)
                out.append((cam, 1 if kind == 2 else 0, w, h, center, samples(rng, w, h, n)))
    return out


def run(lib, cam, typ, w, h, center, s):
    out = np.zeros((len(s), 8), np.float32)
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    lib.camref_primary_rays(P(cam), C.c_int(typ), P(s), C.c_int(len(s)),
                            C.c_float(np.float32(1.0) / np.float32(w)),
                            C.c_float(np.float32(1.0) / np.float32(h)), C.c_int(center), P(out))
    return out


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_CAM_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    exact = C.CDLL(B.REF_CAM_LIB)
    fused = C.CDLL(B.REF_CAM_FUSED_LIB)
    arrays = {}
    cs = cases()
    for i, (cam, typ, w, h, center, s) in enumerate(cs):
        arrays.update({f"c{i}_cam": cam, f"c{i}_meta": np.array([typ, w, h, center], np.int32),
                       f"c{i}_samples": s,
                       f"c{i}_rays": run(exact, cam, typ, w, h, center, s),
                       f"c{i}_rays_fused": run(fused, cam, typ, w, h, center, s)})
    arrays["num_cases"] = np.int32(len(cs))
    np.savez_compressed(os.path.join(HERE, "camera_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "camera_golden.npz"), sum(len(c[5]) for c in cs), "rays")


if __name__ == "__main__":
    main()
