"""Generates tests/golden/curand_philox.json and tests/golden/tex_filter.json
on a machine with a GPU: compiles cuda_fixtures.cu (sm_103a), runs it, and
records the GPU's curand draws and hardware-filtered texture values, and
prints how many of them the oracle's texture-unit emulation misses.

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
    got = np.array([O.tex3d(vox, c, 1) for c in t3["coords"]], np.float32)
    t1 = raw["tex1"]
    table = np.array(t1["table"], np.float32).reshape(-1, 4)
    got1 = np.array([O.tex1d(table, c, 1) for c in t1["coords"]], np.float32).reshape(-1)
    with open(os.path.join(out_dir, "tex_filter.json"), "w") as f:
        json.dump({"source": "tex3D<float> / tex1D<float4>, linear, clamp, normalised, on a GB300",
                   "dims": t3["dims"], "volume": t3["volume"], "coords": t3["coords"],
                   "values": t3["values"],
                   "tex1": {"table": t1["table"], "coords": t1["coords"],
                            "values": t1["values"]}}, f)
    print("oracle texture emulation mismatches: 3D",
          int((got != np.array(t3["values"], np.float32)).sum()), "of", len(got),
          "1D", int((got1 != np.array(t1["values"], np.float32)).sum()), "of", len(got1))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
