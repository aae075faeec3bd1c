"""The BVH builder's Morton sort (a hand-written stable LSD radix sort,
visrtx_gb300/csrc/radix_sort.cu) against numpy's stable argsort, through
the C ABI: tile-edge sizes, the icosphere BLAS's primitive count, runs of
equal keys (which must keep their input order), and partial key widths."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,bits,distinct", [
    (1, 63, 0), (2, 63, 0), (2047, 63, 0), (2048, 63, 0), (2049, 63, 0),
    (100_003, 63, 0), (1_310_720, 63, 0), (70_000, 63, 37), (50_000, 12, 0),
    (40_000, 64, 0), (4096 * 5 + 17, 21, 1000)])
def test_radix_sort_matches_stable_argsort(device, n, bits, distinct):
    rng = np.random.default_rng(n + bits)
    if distinct:
        keys = rng.integers(0, distinct, n).astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    else:
        hi = 2 ** 63 if bits <= 63 else 2 ** 64
        keys = rng.integers(0, hi, n, dtype=np.uint64)
    keys = np.ascontiguousarray(keys)
    vals = np.arange(n, dtype=np.uint32)
    mask = np.uint64((1 << bits) - 1) if bits < 64 else np.uint64(2 ** 64 - 1)
    order = np.argsort(keys & mask, kind="stable")
    k = keys.copy()
    v = vals.copy()
    rc = device.lib.vrtxDebugRadixSort(device.h, k.ctypes.data_as(C.c_void_p),
                                       v.ctypes.data_as(C.c_void_p), n, bits)
    assert rc == 0, device.errors()
    assert np.array_equal(v, order.astype(np.uint32))
    assert np.array_equal(k, keys[order])


def test_radix_sort_rejects_bad_width(device):
    k = np.zeros(4, np.uint64)
    v = np.zeros(4, np.uint32)
    rc = device.lib.vrtxDebugRadixSort(device.h, k.ctypes.data_as(C.c_void_p),
                                       v.ctypes.data_as(C.c_void_p), 4, 65)
    assert rc < 0
    device.messages.clear()
