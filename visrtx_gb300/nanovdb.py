"""NanoVDB grid buffers from dense blocks, for the "nanovdb" spatial field.

The field (spatial_field/NvdbRegularField.cpp) takes one NanoVDB grid as an
Array1D of UINT8. This module writes such buffers (NanoVDB 32.7 layout,
the version the reference vendors in external/nanovdb) for float grids and
the quantised Fp4 / Fp8 / Fp16 / FpN leaf codecs the reference's marcher
dispatches (gpu/volumeIntegration.h:128-158):

  GridData (672 B) | TreeData (64 B) | RootData (64 B + 32 B per tile)
  | upper internal nodes (32^3 entries) | lower internal nodes (16^3)
  | leaves (8^3 voxels)

Nodes are stored breadth-first (root tile order, then child-mask order), so
NanoVDB's own validator accepts the buffers; child pointers are signed byte
offsets from the parent (from the RootData for root tiles). Voxels outside
the active set hold the background value, as NanoVDB's builder leaves them.
Quantised leaves store the leaf's minimum over all 512 values and the
quantum (max - min) / (2^bits - 1); codes round to nearest with the
builder's own arithmetic, so a grid written here holds the same codes as one
NanoVDB's builder makes from the same voxels. FpN picks, per leaf, the
narrowest of 1/2/4/8/16 bits whose error over the leaf's 512 values is
within `tolerance` (NanoVDB's default for fog volumes, 0.01). The checksum
is written as disabled (all bits set).
"""
from __future__ import annotations

import struct

import numpy as np

GRID_TYPES = {"float": 1, "fp4": 13, "fp8": 14, "fp16": 15, "fpn": 16}
MAGIC = 0x304244566F6E614E  # "NanoVDB0"
VERSION = (32 << 21) | (7 << 10) | 0
# IsBreadthFirst | HasBBox | HasMinMax | HasAverage | HasStdDeviation
GRID_FLAGS = 32 | 2 | 4 | 8 | 16
FOG_VOLUME = 2

GRID_SIZE, TREE_SIZE, ROOT_SIZE, TILE_SIZE = 672, 64, 64, 32
UPPER_SIZE, UPPER_TABLE = 270400, 8256
LOWER_SIZE, LOWER_TABLE = 33856, 1088
LEAF_HEADER = 96
_FIXED_LEAF = {"float": 96 + 4 * 512, "fp4": 96 + 256, "fp8": 96 + 512, "fp16": 96 + 1024}
_FIXED_BITS = {"fp4": 4, "fp8": 8, "fp16": 16}


def _root_key(x, y, z):
    u = lambda c: (np.asarray(c, np.int64) & 0xFFFFFFFF) >> 12  # noqa: E731
    return (u(z)) | (u(y) << 21) | (u(x) << 42)


_LEAF_HEADER = np.dtype([("bmin", "<i4", 3), ("dif", "u1", 3), ("flags", "u1"),
                         ("mask", "u1", 64), ("s", "<f4", 4)])
_LEAF_HEADER_FP = np.dtype([("bmin", "<i4", 3), ("dif", "u1", 3), ("flags", "u1"),
                            ("mask", "u1", 64), ("mn", "<f4"), ("q", "<f4"), ("st", "<u2", 4)])


def _encode_leaves(values, minimum, maximum, bits):
    """Codes (per leaf row) and the per-leaf quantum (max - min) / (2^bits - 1),
    with the arithmetic NanoVDB's builder uses (tools/CreateNanoGrid.h):
    encode = units / (max - min), code = trunc(encode * (v - min) + 0.5), in
    float32 below 16 bits and in float64 at 16 bits; a constant leaf gets
    code 0."""
    units = (1 << bits) - 1
    mn = np.asarray(minimum, np.float32)[:, None]
    mx = np.asarray(maximum, np.float32)[:, None]
    v = np.asarray(values, np.float32)
    span = (mx - mn).astype(np.float32)
    quantum = (span[:, 0] / np.float32(units)).astype(np.float32)
    ok = span > 0
    with np.errstate(divide="ignore", invalid="ignore"):
        if bits >= 16:
            enc = np.float64(units) / span.astype(np.float64)
            x = enc * (v - mn).astype(np.float64) + 0.5
        else:
            enc = (np.float32(units) / span).astype(np.float32)
            x = (enc * (v - mn)).astype(np.float32) + np.float32(0.5)
        codes = np.where(ok, np.trunc(np.where(ok, x, 0)), 0)
    return np.clip(codes, 0, units).astype(np.uint32), quantum


def _approx_leaves(codes, minimum, quantum):
    """code * decode + min in float32, separately rounded (the builder's
    bit-width test for FpN)."""
    q = np.asarray(quantum, np.float32)[:, None]
    return ((codes.astype(np.float32) * q).astype(np.float32)
            + np.asarray(minimum, np.float32)[:, None]).astype(np.float32)


def _pack_leaves(codes, bits):
    """Codes of each leaf row packed LSB-first (bit widths 1, 2, 4, 8, 16)."""
    n = codes.shape[0]
    if bits == 16:
        return codes.astype("<u2").view(np.uint8).reshape(n, -1)
    if bits == 8:
        return codes.astype(np.uint8)
    per = 8 // bits
    c = codes.astype(np.uint8).reshape(n, -1, per)
    out = np.zeros(c.shape[:2], np.uint8)
    for k in range(per):
        out |= (c[:, :, k] << (k * bits)).astype(np.uint8)
    return out


def build_grid(dense, active=None, index_origin=(0, 0, 0), voxel_size=1.0,
               translation=(0.0, 0.0, 0.0), background=0.0, grid_type="float",
               tolerance=0.01, name="density") -> np.ndarray:
    """One NanoVDB grid as a uint8 buffer.

    dense: (nz, ny, nx) float32 block whose voxel (x, y, z) sits at index
    coordinate index_origin + (x, y, z); active: bool block of the same shape
    (default: dense != background), the voxels that are set; the map is a
    uniform scale `voxel_size` plus `translation` (index -> world).
    """
    if grid_type not in GRID_TYPES:
        raise ValueError(f"grid_type must be one of {sorted(GRID_TYPES)}")
    dense = np.asarray(dense, np.float32)
    if dense.ndim != 3:
        raise ValueError("dense must be (nz, ny, nx)")
    bg = np.float32(background)
    act = (dense != bg) if active is None else np.asarray(active, bool)
    if act.shape != dense.shape:
        raise ValueError("active must match dense")
    ox, oy, oz = (int(c) for c in index_origin)
    nz, ny, nx = dense.shape
    # pad to leaf-aligned blocks
    lo = [(c // 8) * 8 for c in (ox, oy, oz)]
    pre = [o - l for o, l in zip((ox, oy, oz), lo)]
    ext = [-(-(p + n) // 8) * 8 for p, n in zip(pre, (nx, ny, nz))]
    vpad = np.full((ext[2], ext[1], ext[0]), bg, np.float32)
    apad = np.zeros((ext[2], ext[1], ext[0]), bool)
    vpad[pre[2]:pre[2] + nz, pre[1]:pre[1] + ny, pre[0]:pre[0] + nx] = dense
    apad[pre[2]:pre[2] + nz, pre[1]:pre[1] + ny, pre[0]:pre[0] + nx] = act
    nl = [e // 8 for e in ext]

    def leaves_of(a):
        # (z, y, x) -> leaves (lz, ly, lx) of [x][y][z], i.e. offset x<<6 | y<<3 | z
        return a.reshape(nl[2], 8, nl[1], 8, nl[0], 8).transpose(0, 2, 4, 5, 3, 1).reshape(-1, 512)

    lv = leaves_of(vpad)
    la = leaves_of(apad)
    keep = la.any(axis=1)
    lz, ly, lx = np.unravel_index(np.nonzero(keep)[0], (nl[2], nl[1], nl[0]))
    lv, la = lv[keep], la[keep]
    lv = np.where(la, lv, bg).astype(np.float32)
    org = np.stack([lo[0] + 8 * lx, lo[1] + 8 * ly, lo[2] + 8 * lz], axis=1).astype(np.int64)
    # breadth-first order: root key, then the lower's slot in its upper, then
    # the leaf's slot in its lower
    ukey = _root_key(org[:, 0], org[:, 1], org[:, 2])
    n_up = (((org[:, 0] & 4095) >> 7) << 10) | (((org[:, 1] & 4095) >> 7) << 5) | ((org[:, 2] & 4095) >> 7)
    n_lo = (((org[:, 0] & 127) >> 3) << 8) | (((org[:, 1] & 127) >> 3) << 4) | ((org[:, 2] & 127) >> 3)
    order = np.lexsort((n_lo, n_up, ukey))
    lv, la, org, ukey, n_up, n_lo = lv[order], la[order], org[order], ukey[order], n_up[order], n_lo[order]
    nleaf = len(lv)

    # leaf codecs (vectorised over leaves)
    if grid_type == "float":
        bits_of = np.full(nleaf, 32, np.int64)
        leaf_sizes = np.full(nleaf, _FIXED_LEAF["float"], np.int64)
    else:
        lmin = lv.min(axis=1) if nleaf else np.zeros(0, np.float32)
        lmax = lv.max(axis=1) if nleaf else np.zeros(0, np.float32)
        if grid_type == "fpn":
            bits_of = np.full(nleaf, 16, np.int64)
            undecided = np.ones(nleaf, bool)
            for bw in (1, 2, 4, 8):
                # the builder's AbsDiff oracle over all 512 values of the leaf
                codes, q = _encode_leaves(lv, lmin, lmax, bw)
                err = np.abs(lv - _approx_leaves(codes, lmin, q))
                ok = (err <= np.float32(tolerance)).all(axis=1)
                pick = undecided & ok
                bits_of[pick] = bw
                undecided &= ~pick
            leaf_sizes = 96 + 64 * bits_of
        else:
            bits_of = np.full(nleaf, _FIXED_BITS[grid_type], np.int64)
            leaf_sizes = np.full(nleaf, _FIXED_LEAF[grid_type], np.int64)

    # node grouping: a new lower node where (root key, upper slot) changes, a
    # new upper node where the root key changes
    if nleaf:
        new_low = np.r_[True, (ukey[1:] != ukey[:-1]) | (n_up[1:] != n_up[:-1])]
    else:
        new_low = np.zeros(0, bool)
    low_start = np.nonzero(new_low)[0]
    low_of_leaf = np.cumsum(new_low) - 1
    low_key, low_nup = ukey[low_start], n_up[low_start]
    new_up = np.r_[True, low_key[1:] != low_key[:-1]] if len(low_start) else np.zeros(0, bool)
    up_start = np.nonzero(new_up)[0]
    up_of_low = np.cumsum(new_up) - 1
    nlow, nup = len(low_start), len(up_start)

    root_off = GRID_SIZE + TREE_SIZE
    root_bytes = ROOT_SIZE + TILE_SIZE * nup
    up_off = root_off + root_bytes
    low_off = up_off + UPPER_SIZE * nup
    leaf_off0 = low_off + LOWER_SIZE * nlow
    leaf_offs = np.concatenate([[0], np.cumsum(leaf_sizes)]).astype(np.int64) + leaf_off0
    total = int(leaf_offs[-1])
    buf = bytearray(total)
    bg_word = np.frombuffer(struct.pack("<f", float(bg)), np.uint32)[0]

    # per-leaf aggregates of the active voxels: bbox, count, sums, min, max
    off = np.arange(512)
    loc = np.stack([off >> 6, (off >> 3) & 7, off & 7], axis=0)  # (3, 512)
    v64 = lv.astype(np.float64)
    cnt = la.sum(axis=1)
    if nleaf:
        bmin = np.stack([np.where(la, loc[k], 8).min(axis=1) for k in range(3)], axis=1)
        bmax = np.stack([np.where(la, loc[k], -1).max(axis=1) for k in range(3)], axis=1)
        s1 = np.where(la, v64, 0.0).sum(axis=1)
        s2 = np.where(la, v64 * v64, 0.0).sum(axis=1)
        amin = np.where(la, v64, np.inf).min(axis=1)
        amax = np.where(la, v64, -np.inf).max(axis=1)
    else:
        bmin = bmax = np.zeros((0, 3), np.int64)
        s1 = s2 = amin = amax = np.zeros(0)
    gmin, gmax = org + bmin, org + bmax

    def node_stats(starts, n_items, key_min, key_max, c, t1, t2, lo_, hi_):
        """Aggregates over contiguous runs [starts[i], starts[i+1])."""
        if not len(starts):
            z = np.zeros(0)
            return np.zeros((0, 3), np.int64), np.zeros((0, 3), np.int64), z, z, z, z
        bb_lo = np.minimum.reduceat(key_min, starts, axis=0)
        bb_hi = np.maximum.reduceat(key_max, starts, axis=0)
        cc = np.add.reduceat(c, starts)
        m1 = np.add.reduceat(t1, starts) / cc
        m2 = np.add.reduceat(t2, starts) / cc
        return (bb_lo, bb_hi, np.minimum.reduceat(lo_, starts), np.maximum.reduceat(hi_, starts),
                m1, np.sqrt(np.maximum(m2 - m1 * m1, 0.0)))

    # leaves: header (bbox of active voxels, flags, value mask, stats), then values
    hdr = np.zeros(nleaf, _LEAF_HEADER)
    if nleaf:
        hdr["bmin"] = gmin
        hdr["dif"] = (bmax - bmin).astype(np.uint8)
        hdr["mask"] = np.packbits(la, axis=1, bitorder="little")
        aavg = s1 / cnt
        astd = np.sqrt(np.maximum(s2 / cnt - aavg * aavg, 0.0))
        logb = np.round(np.log2(bits_of)).astype(np.uint8)
        hdr["flags"] = 2 | 16 | ((logb << 5) if grid_type == "fpn" else 0)
        if grid_type == "float":
            hdr["s"] = np.stack([amin, amax, aavg, astd], axis=1)
        else:
            hdr_fp = hdr.view(_LEAF_HEADER_FP)
            hdr_fp["mn"] = lmin
            qs = np.zeros(nleaf, np.float32)
            for bw in np.unique(bits_of):
                sel = bits_of == bw
                _, q = _encode_leaves(lv[sel], lmin[sel], lmax[sel], int(bw))
                qs[sel] = q
            hdr_fp["q"] = qs
            qq = np.where(qs > 0, qs, 1.0).astype(np.float64)
            st = [np.floor((x - lmin) / qq + 0.5) for x in (amin, amax, aavg)]
            st.append(np.floor(astd / qq + 0.5))
            hdr_fp["st"] = np.clip(np.stack(st, axis=1), 0, 65535).astype(np.uint16)
    leaf_block = np.zeros(total - leaf_off0, np.uint8)
    rel = (leaf_offs[:-1] - leaf_off0).astype(np.int64)
    hdr_bytes = hdr.view(np.uint8).reshape(nleaf, LEAF_HEADER)
    if grid_type != "fpn":
        if nleaf:
            rows = leaf_block.reshape(nleaf, int(leaf_sizes[0]))
            rows[:, :LEAF_HEADER] = hdr_bytes
            if grid_type == "float":
                rows[:, LEAF_HEADER:] = lv.astype("<f4").view(np.uint8).reshape(nleaf, -1)
            else:
                bw = _FIXED_BITS[grid_type]
                codes, _ = _encode_leaves(lv, lmin, lmax, bw)
                rows[:, LEAF_HEADER:] = _pack_leaves(codes, bw)
    else:
        for bw in np.unique(bits_of):
            sel = np.nonzero(bits_of == bw)[0]
            codes, _ = _encode_leaves(lv[sel], lmin[sel], lmax[sel], int(bw))
            packed = _pack_leaves(codes, int(bw))
            for r, i in enumerate(sel):
                o = rel[i]
                leaf_block[o:o + LEAF_HEADER] = hdr_bytes[i]
                leaf_block[o + LEAF_HEADER:o + LEAF_HEADER + packed.shape[1]] = packed[r]
    buf[leaf_off0:total] = leaf_block.tobytes()

    # lower nodes: bbox, child mask, stats, table (child offsets from the node,
    # background elsewhere)
    lb_lo, lb_hi, l_min, l_max, l_avg, l_std = node_stats(low_start, nleaf, gmin, gmax, cnt, s1, s2,
                                                          amin, amax)
    bounds = np.r_[low_start, nleaf]
    for j in range(nlow):
        o = low_off + LOWER_SIZE * j
        a_, b_ = bounds[j], bounds[j + 1]
        struct.pack_into("<6iQ", buf, o, *map(int, lb_lo[j]), *map(int, lb_hi[j]), 0)
        child = np.zeros(4096, bool)
        child[n_lo[a_:b_]] = True
        buf[o + 544:o + 1056] = np.packbits(child, bitorder="little").tobytes()
        struct.pack_into("<4f", buf, o + 1056, l_min[j], l_max[j], l_avg[j], l_std[j])
        table = np.zeros(4096, np.int64)
        table.view(np.uint32)[0::2] = bg_word
        table[n_lo[a_:b_]] = leaf_offs[a_:b_] - o
        buf[o + LOWER_TABLE:o + LOWER_SIZE] = table.astype("<i8").tobytes()

    # upper nodes
    leaf_up_start = low_start[up_start] if nup else np.zeros(0, np.int64)
    ub_lo, ub_hi, u_min, u_max, u_avg, u_std = node_stats(leaf_up_start, nleaf, gmin, gmax, cnt, s1,
                                                          s2, amin, amax)
    ubounds = np.r_[up_start, nlow]
    for k in range(nup):
        o = up_off + UPPER_SIZE * k
        a_, b_ = ubounds[k], ubounds[k + 1]
        struct.pack_into("<6iQ", buf, o, *map(int, ub_lo[k]), *map(int, ub_hi[k]), 0)
        child = np.zeros(32768, bool)
        child[low_nup[a_:b_]] = True
        buf[o + 4128:o + 8224] = np.packbits(child, bitorder="little").tobytes()
        struct.pack_into("<4f", buf, o + 8224, u_min[k], u_max[k], u_avg[k], u_std[k])
        table = np.zeros(32768, np.int64)
        table.view(np.uint32)[0::2] = bg_word
        table[low_nup[a_:b_]] = (low_off + LOWER_SIZE * np.arange(a_, b_)) - o
        buf[o + UPPER_TABLE:o + UPPER_SIZE] = table.astype("<i8").tobytes()

    # root: bbox of all active voxels, tile count, background, stats; tiles
    if nleaf:
        rb_lo, rb_hi, r_min, r_max, r_avg, r_std = node_stats(np.array([0]), nleaf, gmin, gmax, cnt,
                                                              s1, s2, amin, amax)
        rmin, rmax = rb_lo[0], rb_hi[0]
        stats = (r_min[0], r_max[0], r_avg[0], r_std[0])
    else:
        rmin, rmax = np.zeros(3, np.int64), np.zeros(3, np.int64)
        stats = (0.0, 0.0, 0.0, 0.0)
    struct.pack_into("<6iI5f", buf, root_off, *map(int, rmin), *map(int, rmax), nup, float(bg),
                     *stats)
    for k in range(nup):
        t = root_off + ROOT_SIZE + TILE_SIZE * k
        struct.pack_into("<QqIf", buf, t, int(low_key[up_start[k]]),
                         up_off + UPPER_SIZE * k - root_off, 0, 0.0)

    # tree
    tree = GRID_SIZE
    struct.pack_into("<4q3I3IQ", buf, tree, leaf_off0 - tree, low_off - tree, up_off - tree,
                     root_off - tree, nleaf, nlow, nup, 0, 0, 0, int(la.sum()))

    # grid
    dx = float(voxel_size)
    t = [float(c) for c in translation]
    inv = 1.0 / dx
    mat_f = [dx, 0, 0, 0, dx, 0, 0, 0, dx]
    inv_f = [inv, 0, 0, 0, inv, 0, 0, 0, inv]
    if nleaf:
        wlo = [float(rmin[k]) * dx + t[k] for k in range(3)]
        whi = [float(rmax[k] + 1) * dx + t[k] for k in range(3)]
    else:
        wlo, whi = [0.0] * 3, [0.0] * 3
    nm = name.encode()[:255]
    struct.pack_into("<QQIIIIQ", buf, 0, MAGIC, 0xFFFFFFFFFFFFFFFF, VERSION, GRID_FLAGS, 0, 1, total)
    buf[40:40 + len(nm)] = nm
    struct.pack_into("<9f9f3ff9d9d3dd", buf, 296, *mat_f, *inv_f, *t, 1.0, *mat_f, *inv_f, *t, 1.0)
    struct.pack_into("<6d3dIIqIIQQ", buf, 560, *wlo, *whi, dx, dx, dx, FOG_VOLUME,
                     GRID_TYPES[grid_type], total, 0, 0, 0, 0)
    return np.frombuffer(bytes(buf), np.uint8)


def grid_info(buf) -> dict:
    """Header fields of a grid buffer: type, voxel count, index and world bounds."""
    b = np.asarray(buf, np.uint8).tobytes()
    magic, = struct.unpack_from("<Q", b, 0)
    gtype, = struct.unpack_from("<I", b, 636)
    wb = struct.unpack_from("<6d", b, 560)
    vs = struct.unpack_from("<3d", b, 608)
    tree = GRID_SIZE
    offs = struct.unpack_from("<4q3I3IQ", b, tree)
    root = tree + offs[3]
    ib = struct.unpack_from("<6i", b, root)
    return {"magic": magic, "type": gtype, "world_bbox": (wb[:3], wb[3:]), "voxel_size": vs,
            "index_bbox": (ib[:3], ib[3:]), "leaves": offs[4], "lowers": offs[5], "uppers": offs[6],
            "voxels": offs[10]}
