"""Generates tests/golden/tex_sweep.npz on a machine with a GPU: compiles
tex_sweep.cu (sm_103a), runs it, and stores every record (texture header,
texels, coordinates and the texture unit's results) as arrays r<i>_hdr,
r<i>_tex, r<i>_coords, r<i>_vals.

    python tests/golden/gen_tex_sweep.py [out.npz]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ELEM = {0: np.float32, 1: np.uint8, 2: np.uint16, 3: np.int8, 4: np.int16}


def parse(raw: bytes) -> list[dict]:
    recs, o = [], 0
    while o < len(raw):
        hdr = np.frombuffer(raw, np.int32, 16, o).copy()
        o += 64
        dim, nx, ny, nz, ch, fmt = (int(v) for v in hdr[:6])
        k = int(hdr[10])
        dt = np.dtype(ELEM[fmt])
        n = nx * ny * nz * ch
        tex = np.frombuffer(raw, dt, n, o).copy()
        o += n * dt.itemsize
        coords = np.frombuffer(raw, np.float32, k * dim, o).copy().reshape(k, dim)
        o += 4 * k * dim
        oc = 1 if ch == 1 else 4
        vals = np.frombuffer(raw, np.float32, k * oc, o).copy().reshape(k, oc)
        o += 4 * k * oc
        recs.append({"hdr": hdr, "tex": tex, "coords": coords, "vals": vals})
    return recs


def main(out: str = os.path.join(HERE, "tex_sweep.npz")) -> None:
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "tex_sweep")
        binf = os.path.join(tmp, "tex_sweep.bin")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                        os.path.join(HERE, "tex_sweep.cu"), "-o", exe], check=True)
        subprocess.run([exe, binf], check=True)
        with open(binf, "rb") as f:
            recs = parse(f.read())
    arrays = {}
    for i, r in enumerate(recs):
        for key in ("hdr", "tex", "coords", "vals"):
            arrays[f"r{i}_{key}"] = r[key]
    np.savez_compressed(out, **arrays)
    print(f"{len(recs)} records -> {out}")


if __name__ == "__main__":
    main(*sys.argv[1:])
