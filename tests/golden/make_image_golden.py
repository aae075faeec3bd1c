"""Generates tests/golden/image_golden.npz: image texels as the reference's
own staging writes them into CUDA arrays (devices/rtx/utility/
CudaImageTexture.cpp:43-111, transformToStagingBufferUint8 / Float with
convertComponentUint8 / Float), compiled on the host by
oracle/ref_image.cpp, for every image element type this library's samplers
and background take:

  * image samplers (sampler/Image1D/2D/3D.cpp: float element types staged
    as float, every other as 8-bit read as normalised float, by the
    reference's own isFloat): UFIXED8 x1 and x4 over all 256 byte values,
    UFIXED8_RGBA_SRGB over all 256 values in every channel (alpha too),
    UFIXED16 over all 65536 values, FLOAT32 x1..x4;
  * the renderer's background image (Renderer.cpp:173-179, always 8-bit):
    FLOAT32 x3 / x4 in [0, 1] (0, 1, every k / 255 and the floats next to
    it), UFIXED8 x4 and UFIXED8_RGBA_SRGB over all 256 values.

Each case keeps the reference's own layout (nc components per texel, a
fourth added for three): `staged`, with `channels` = nc.

Run in a tree that holds the reference (it builds oracle/_ref/libimgref.so
from the reference's sources):  python tests/golden/make_image_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

# this library's element type codes (include/vrtx.h)
UFIXED8, UFIXED16, FLOAT32, UFIXED8_VEC4, UFIXED8_RGBA_SRGB = 221, 223, 240, 260, 261
# the harness's kinds: 0 float32, 1 ufixed8, 2 ufixed16, 3 ufixed32, 4 sRGB
KIND = {UFIXED8: 1, UFIXED16: 2, UFIXED8_VEC4: 1, UFIXED8_RGBA_SRGB: 4,
        FLOAT32: 0, FLOAT32 + 1: 0, FLOAT32 + 2: 0, FLOAT32 + 3: 0}


def _all_bytes_x4():
    i = np.arange(256)
    return np.stack([i, (i + 64) % 256, (i + 128) % 256, (i + 192) % 256], 1).astype(np.uint8)


def _unit_floats(nc, rng):
    k = np.arange(256, dtype=np.float32) / np.float32(255)
    v = np.concatenate([k, np.nextafter(k, np.float32(0)), np.nextafter(k, np.float32(1)),
                        rng.uniform(0, 1, 256).astype(np.float32), np.float32([0, 1])])
    v = np.clip(v, 0, 1).astype(np.float32)
    n = len(v) // nc * nc
    return v[:n].reshape(-1, nc)


def cases(seed=23):
    rng = np.random.default_rng(seed)
    out = []  # (name, et, background, texels (n, nc) or (n,))
    out.append(("sampler_ufixed8", UFIXED8, 0, np.arange(256, dtype=np.uint8)))
    out.append(("sampler_ufixed8x4", UFIXED8_VEC4, 0, _all_bytes_x4()))
    out.append(("sampler_srgb8x4", UFIXED8_RGBA_SRGB, 0, _all_bytes_x4()))
    out.append(("sampler_ufixed16", UFIXED16, 0, np.arange(65536, dtype=np.uint16)))
    for nc in (1, 2, 3, 4):
        v = rng.normal(0, 2, (97, nc)).astype(np.float32)
        v[0] = 0.0
        v[1] = -0.0
        v[2] = 1.0
        out.append((f"sampler_float32x{nc}", FLOAT32 + nc - 1, 0, v[:, 0] if nc == 1 else v))
    out.append(("background_float32x3", FLOAT32 + 2, 1, _unit_floats(3, rng)))
    out.append(("background_float32x4", FLOAT32 + 3, 1, _unit_floats(4, rng)))
    out.append(("background_ufixed8x4", UFIXED8_VEC4, 1, _all_bytes_x4()))
    out.append(("background_srgb8x4", UFIXED8_RGBA_SRGB, 1, _all_bytes_x4()))
    return out


def stage(lib, et, background, texels):
    t = np.ascontiguousarray(texels)
    n = t.shape[0]
    nc = 1 if t.ndim == 1 else t.shape[1]
    kind = KIND[et]
    uses_float = (not background) and lib.imgref_sampler_uses_float(C.c_int(kind)) == 1
    width = 4 if nc == 3 else nc
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    if uses_float:
        out = np.zeros((n, width), np.float32)
        r = lib.imgref_stage_float(C.c_int(kind), C.c_int(nc), P(t), C.c_size_t(n), P(out))
    else:
        out = np.zeros((n, width), np.uint8)
        r = lib.imgref_stage_uint8(C.c_int(kind), C.c_int(nc), P(t), C.c_size_t(n), P(out))
    assert r == 0
    return out, nc, int(uses_float)


def main():
    from oracle import build as B

    if B.build_ref() is None or not os.path.exists(B.REF_IMG_LIB):
        raise SystemExit("the reference tree is needed to generate the fixtures")
    lib = C.CDLL(B.REF_IMG_LIB)
    arrays = {}
    cs = cases()
    for name, et, bg, tex in cs:
        staged, nc, uf = stage(lib, et, bg, tex)
        arrays.update({f"{name}_texels": tex, f"{name}_staged": staged,
                       f"{name}_meta": np.array([et, bg, nc, uf], np.int32)})
    arrays["names"] = np.array([c[0] for c in cs])
    np.savez_compressed(os.path.join(HERE, "image_golden.npz"), **arrays)
    print("wrote", os.path.join(HERE, "image_golden.npz"), len(cs), "cases")


if __name__ == "__main__":
    main()
