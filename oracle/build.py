"""Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

The reference itself cannot be compiled here (its device path needs OptiX
headers fetched at configure time and the ANARI-SDK, neither present), so
there is no oracle/_ref build; see oracle.h for the parity status.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")


def build() -> str:
    src = [os.path.join(HERE, "oracle.cpp")]
    hdr = [os.path.join(HERE, "oracle.h")]
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(f) for f in src + hdr):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-o", tmp, *src, "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
