"""Generates tests/golden/curand_philox.json and tests/golden/tex_filter.json
on a machine with a GPU: compiles cuda_fixtures.cu (sm_103a), runs it, and
records the GPU's curand draws and hardware-filtered texture values. For the
texture it also records how closely the oracle's filter emulation (weights
with 8 fractional bits, truncated or rounded) reproduces the hardware, and
picks the rounding that does.

    python tests/golden/gen_cuda_fixtures.py [out_dir]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main(out_dir: str = HERE) -> None:
    from oracle import oracle as O

    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "fixtures")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2",
                        os.path.join(HERE, "cuda_fixtures.cu"), "-o", exe], check=True)
        raw = json.loads(subprocess.run([exe], check=True, capture_output=True,
                                        text=True).stdout)
    cases = []
    for c in raw["curand"]:
        bits = np.array(c["bits"], np.uint32)
        values = bits.tolist() if c["kind"] == 0 else bits.view(np.float32).tolist()
        cases.append({"seed": c["seed"], "subsequence": c["subsequence"], "offset": c["offset"],
                      "kind": c["kind"], "values": values})
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, "curand_philox.json"), "w") as f:
        json.dump({"source": "curand_init + curand/curand_uniform/curand_uniform4 on a GB300",
                   "cases": cases}, f)

    t3 = raw["tex3"]
    vox = np.array(t3["volume"], np.float32).reshape(t3["dims"][::-1])
    errs = {}
    for mode in (0, 1):
        e = [abs(O.tex3d(vox, c, mode) - v) for c, v in zip(t3["coords"], t3["values"])]
        errs[mode] = float(max(e))
    mode = min(errs, key=errs.get)
    t1 = raw["tex1"]
    table = np.array(t1["table"], np.float32).reshape(-1, 4)
    e1 = {}
    for m in (0, 1):
        e1[m] = float(max(np.abs(O.tex1d(table, c, m) - np.array(t1["values"][4 * i:4 * i + 4])).max()
                          for i, c in enumerate(t1["coords"])))
    with open(os.path.join(out_dir, "tex_filter.json"), "w") as f:
        json.dump({"source": "tex3D<float> / tex1D<float4>, linear, clamp, normalised, on a GB300",
                   "dims": t3["dims"], "volume": t3["volume"], "coords": t3["coords"],
                   "values": t3["values"], "round_mode": mode,
                   "max_error_by_round_mode": errs,
                   "tolerance": errs[mode] * 1.01 + 1e-7,
                   "tex1": {"table": t1["table"], "coords": t1["coords"],
                            "values": t1["values"], "max_error_by_round_mode": e1}}, f)
    print("tex3 max error by rounding mode:", errs, "tex1:", e1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
