"""Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so,
and, where the reference tree is present, oracle/_ref/libnvdbref.so.

The reference's renderer cannot be compiled here (its device path needs
OptiX headers fetched at configure time and the ANARI-SDK, neither present);
see oracle.h for the parity status. The NanoVDB library it vendors
(external/nanovdb, header-only) does compile with g++ alone: ref_nvdb.cpp
drives its grid builder, sampler and validator, compiled from the headers
where they lie under the reference tree, with the output only in
oracle/_ref/. The GPU machine has no reference tree and never builds it.
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


# The VisRTX source tree: VISRTX_REFERENCE_TREE, or build_ref(tree=...);
# the default is where this recipe's build machine mounts it.
REF_TREE = os.environ.get("VISRTX_REFERENCE_TREE", "/root/reference")
REF_OUT = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_OUT, "libnvdbref.so")


def build_ref(tree: str | None = None) -> str | None:
    """oracle/_ref/libnvdbref.so from ref_nvdb.cpp and the reference's vendored
    NanoVDB headers under `tree` (default REF_TREE); None when the reference
    tree is absent."""
    inc = os.path.join(tree or REF_TREE, "external", "nanovdb", "include")
    if not os.path.isdir(inc):
        return None
    src = os.path.join(HERE, "ref_nvdb.cpp")
    os.makedirs(REF_OUT, exist_ok=True)
    if os.path.exists(REF_LIB) and os.path.getmtime(REF_LIB) >= os.path.getmtime(src):
        return REF_LIB
    tmp = REF_LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-I", inc, "-o", tmp, src, "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle/_ref build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    import sys

    print(build())
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None))
