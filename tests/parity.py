"""Comparison helpers for GPU-vs-oracle parity tests.

Tolerances follow the stated bar: primitiveId/objectId/instanceId
bit-exact except for at most `id_frac` of pixels (grazing or tied hits),
depth within 1e-5 relative on every pixel whose ids match, colour within
`color_tol`/255 per channel.
"""
from __future__ import annotations

import numpy as np

from visrtx_gb300 import anari, scenes

ID_FRAC = 1e-4
DEPTH_REL = 1e-5


def render_gpu(dev, spec: scenes.SceneSpec, frames: int = 1, channels: bool = False,
               float_color: bool = False):
    chans = ("color", "depth", "primitiveId", "objectId", "instanceId")
    if channels:
        chans += ("albedo", "normal")
    frame, world, keep = scenes.build_on_device(dev, spec, channels=chans,
                                                float_color=float_color)
    for _ in range(frames):
        frame.render()
    frame.wait()
    out = {ch: frame.map("channel." + ch) for ch in chans}
    out["frame"] = frame
    out["world"] = world
    out["keep"] = keep
    return out


def oracle_frame_ids(spec: scenes.SceneSpec, frames: int):
    """(frameID, checkerboardID) of each render call, as Frame::newFrame
    advances them (Frame.cu:590-660): with checkerboarding the frame id
    grows by one after checkerboard pass 3, else by pixelSamples."""
    r = spec.renderer
    out = []
    for f in range(frames):
        if r.checkerboard:
            out.append((f // 4, f % 4))
        elif r.subtype == "raycast":
            out.append((f, -1))
        else:
            out.append((f * max(1, r.pixel_samples), -1))
    return out


def render_oracle(spec: scenes.SceneSpec, frames: int = 1, channels: bool = False, **kw):
    """The oracle's frames; with `channels` the albedo and normal outputs are
    returned as the reference maps them (accumulation / (frameID + 1))."""
    from oracle import oracle as O

    sc = O.OracleScene(spec)
    prev = None
    out = None
    fid = 0
    try:
        for fid, cb in oracle_frame_ids(spec, frames):
            out = sc.render(frame_id=fid,
                            accum=None if prev is None else prev["accum"],
                            depth=None if prev is None else prev["depth"],
                            ids=prev, checkerboard_id=cb, channels=channels, **kw)
            prev = out
    finally:
        sc.release()
    if channels:
        out = dict(out)
        for ch in ("albedo", "normal"):
            out[ch] = out[ch] * np.float32(1.0 / (fid + 1))
    return out


def compare(gpu, ref, id_frac=ID_FRAC, depth_rel=DEPTH_REL, color_tol=1, allow_ids=0):
    """Returns a report dict; raises AssertionError with details on failure."""
    n = gpu["primitiveId"].size
    idm = np.zeros(gpu["primitiveId"].shape, bool)
    for ch in ("primitiveId", "objectId", "instanceId"):
        idm |= gpu[ch] != ref[ch]
    frac = idm.sum() / n
    same = ~idm
    hit = same & (ref["depth"] < 1e29)
    drel = np.abs(gpu["depth"][hit].astype(np.float64) - ref["depth"][hit]) / np.maximum(
        np.abs(ref["depth"][hit]), 1e-12)
    bg_ok = np.all(gpu["depth"][same & (ref["depth"] >= 1e29)] == ref["depth"][same & (ref["depth"] >= 1e29)])
    cg = anari.rgba8(gpu["color"]).astype(np.int32)
    cr = anari.rgba8(ref["color"]).astype(np.int32)
    cdiff = np.abs(cg - cr)[same]
    rep = {
        "pixels": n,
        "id_mismatch": int(idm.sum()),
        "id_frac": float(frac),
        "depth_rel_max": float(drel.max()) if drel.size else 0.0,
        "depth_rel_q999": float(np.quantile(drel, 0.999)) if drel.size else 0.0,
        "color_max": int(cdiff.max()) if cdiff.size else 0,
        "color_mean": float(cdiff.mean()) if cdiff.size else 0.0,
        "color_frac_over": float((cdiff > color_tol).any(axis=-1).mean()) if cdiff.size else 0.0,
    }
    ok = (idm.sum() <= max(allow_ids, int(id_frac * n))
          and rep["depth_rel_max"] <= depth_rel and bg_ok
          and rep["color_frac_over"] <= max(id_frac, allow_ids / n))
    assert ok, f"parity failure: {rep}"
    return rep


def inverse_tonemap(accum: np.ndarray, frames: int = 1) -> np.ndarray:
    """The frame's float colour from an oracle accumulation buffer, as
    accumResults writes FLOAT32_VEC4 colour (gpu_util.h:321-335,393-420):
    rgb / max(1e-12, 1 - max(rgb)) of accum / frames, in float64."""
    a = accum.astype(np.float64) / frames
    rgb = a[..., :3] / np.maximum(1e-12, 1.0 - a[..., :3].max(axis=-1, keepdims=True))
    return np.concatenate([rgb, a[..., 3:]], axis=-1)
