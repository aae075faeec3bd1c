"""Generates tests/golden/tf_golden.npz: 256-entry transfer-function tables
computed by the reference's own helpers (devices/rtx/utility/
colorMapHelpers.h: generateLinearPositions, getInterpolatedValue), through
the call sequence of TransferFunction1D::discritizeTFData
(TransferFunction1D.cpp:101-150), for seeded knot arrays: vec3 and vec4
colours, opacity arrays of 2 to 17 knots, colour or opacity absent (the
uniform colour / opacity then), unit, offset, negative and narrow value
ranges.

Run in a tree that holds the reference (it builds oracle/_ref/libtfref.so
from the reference's headers):  python tests/golden/make_tf_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

RANGES = [(0.0, 1.0), (-2.0, 3.5), (0.25, 0.3), (-1.0, -0.5), (10.0, 1000.0)]


def cases(seed=11):
    """(color or None, opacity or None, value range, uniform colour, uniform
    opacity) tuples."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(40):
        comps = 3 if k % 2 == 0 else 4
        nc = int(rng.integers(2, 18))
        no = int(rng.integers(2, 18))
        color = rng.uniform(0.0, 1.0, (nc, comps)).astype(np.float32)
        opacity = rng.uniform(0.0, 1.0, no).astype(np.float32)
        if k % 7 == 3:
            color = None
        if k % 5 == 4:
            opacity = None
        rng_v = RANGES[k % len(RANGES)]
        uc = rng.uniform(0.0, 1.0, 4).astype(np.float32)
        uo = np.float32(rng.uniform(0.0, 1.0))
        out.append((color, opacity, rng_v, uc, uo))
    return out


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_TF_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_TF_LIB)
    fp = C.POINTER(C.c_float)
    lib.tfref_discretize.argtypes = [fp, C.c_int, C.c_int, fp, C.c_int, C.c_float, C.c_float,
                                     fp, C.c_float, C.c_int, fp]
    lib.tfref_discretize.restype = None
    arrays = {}
    for i, (color, opacity, vr, uc, uo) in enumerate(cases()):
        out = np.zeros((256, 4), np.float32)
        cptr = color.ctypes.data_as(fp) if color is not None else None
        optr = opacity.ctypes.data_as(fp) if opacity is not None else None
        lib.tfref_discretize(cptr, 0 if color is None else len(color),
                             0 if color is None else color.shape[1], optr,
                             0 if opacity is None else len(opacity), vr[0], vr[1],
                             uc.ctypes.data_as(fp), float(uo), 256, out.ctypes.data_as(fp))
        if color is not None:
            arrays[f"c{i}_color"] = color
        if opacity is not None:
            arrays[f"c{i}_opacity"] = opacity
        arrays[f"c{i}_range"] = np.asarray(vr, np.float32)
        arrays[f"c{i}_uniform_color"] = uc
        arrays[f"c{i}_uniform_opacity"] = np.asarray([uo], np.float32)
        arrays[f"c{i}_table"] = out
    arrays["count"] = np.asarray([len(cases())])
    np.savez_compressed(os.path.join(HERE, "tf_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "tf_golden.npz"), len(cases()), "tables")


if __name__ == "__main__":
    main()
