"""Generates tests/golden/color_golden.npz: packed frame colours computed by
the reference's output encoding (gpu/gpu_util.h:370-389, writeOutputColor)
with the glm the reference vendors (glm::convertLinearToSRGB,
glm::packUnorm4x8), for accumulated RGBA values after 1 and 7 samples, in
the sRGB and linear rgba8 formats. The values cover [0, 2] with
out-of-range, zero and negative entries, the sRGB curve's linear segment
below 0.0031308 and its edge, and values next to every 8-bit rounding
boundary.

Run in a tree that holds the reference (it builds oracle/_ref/libglmref.so
from the reference's glm headers):  python tests/golden/make_color_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def accumulations(seed=3):
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-0.1, 2.0, (2000, 4)),
             rng.uniform(0.0, 0.01, (500, 4)),
             np.repeat(np.array([[0.0031308, 0.00313, 0.0031309, 0.0]]), 4, axis=0)]
    # next to each rounding boundary (k + 0.5) / 255 of the linear format
    k = (np.arange(255) + 0.5) / 255.0
    for d in (-1e-6, 0.0, 1e-6):
        parts.append(np.stack([k + d, k, k - d, np.clip(k + 2 * d, 0, 1)], axis=1))
    a = np.concatenate(parts).astype(np.float32)
    return a


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_GLM_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_GLM_LIB)
    lib.glmref_write_color.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
    lib.glmref_write_color.restype = None
    acc = accumulations()
    arrays = {"accum": acc}
    for frames in (1, 7):
        a = (acc * frames).astype(np.float32)  # the accumulation of `frames` equal samples
        arrays[f"accum_{frames}"] = a
        for fmt in (0, 1):
            out = np.zeros(len(a), np.uint32)
            lib.glmref_write_color(a.ctypes.data, len(a), frames - 1, fmt, out.ctypes.data)
            arrays[f"packed_{frames}_{fmt}"] = out
    np.savez_compressed(os.path.join(HERE, "color_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "color_golden.npz"), len(acc), "colours")


if __name__ == "__main__":
    main()
