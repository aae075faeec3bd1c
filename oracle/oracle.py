"""Python binding of the CPU oracle (oracle.h). TEST INFRASTRUCTURE ONLY:
used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs as the checker, never by the product path.

render(spec) renders a visrtx_gb300.scenes.SceneSpec with the oracle's
restatement of the reference integrators; dm(...) runs the FP64
differentiable-marcher forward/adjoint.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        from . import build as _b  # noqa: F401  (package-relative when imported as oracle.oracle)
        path = _b.build()
        _lib = C.CDLL(path)
        _lib.orc_render.restype = C.c_int
        _lib.orc_tex3d.restype = C.c_float
    return _lib


class OrcAttr(C.Structure):
    _fields_ = [("data", C.c_void_p), ("type", C.c_int), ("channels", C.c_int)]


class OrcSampler(C.Structure):
    _fields_ = [("type", C.c_int), ("attribute", C.c_int), ("inT", C.c_float * 16),
                ("inO", C.c_float * 4), ("outT", C.c_float * 16), ("outO", C.c_float * 4),
                ("image", C.c_void_p), ("image8", C.c_void_p), ("dims", C.c_int * 3),
                ("filter", C.c_int),
                ("wrap", C.c_int * 3), ("prim", OrcAttr), ("primOffset", C.c_uint32)]


class OrcSurface(C.Structure):
    _fields_ = [("type", C.c_int), ("vertices", C.c_void_p), ("indices", C.c_void_p),
                ("numPrims", C.c_uint32), ("normals", C.c_void_p), ("primIds", C.c_void_p),
                ("radii", C.c_void_p), ("radius", C.c_float), ("cullBackfaces", C.c_int),
                ("id", C.c_uint32), ("color", C.c_float * 3), ("opacity", C.c_float),
                ("alphaMode", C.c_int), ("cutoff", C.c_float), ("caps", C.c_int),
                ("vattr", OrcAttr * 5), ("pattr", OrcAttr * 5), ("uattr", (C.c_float * 4) * 5),
                ("colorSrc", C.c_int), ("opacitySrc", C.c_int), ("colorW", C.c_float),
                ("colorSampler", OrcSampler), ("opacitySampler", OrcSampler),
                ("materialType", C.c_int), ("metallic", C.c_float), ("roughness", C.c_float),
                ("ior", C.c_float), ("metallicSrc", C.c_int), ("roughnessSrc", C.c_int),
                ("metallicSampler", OrcSampler), ("roughnessSampler", OrcSampler)]


_ATTR_SLOTS = ("attribute0", "attribute1", "attribute2", "attribute3", "color")
_PARAM_SOURCES = {"attribute0": 1, "attribute1": 2, "attribute2": 3, "attribute3": 4, "color": 5,
                  "worldPosition": 6, "worldNormal": 7, "objectPosition": 8, "objectNormal": 9}
_ATTR_CHANNELS = {240: 1, 241: 2, 242: 3, 243: 4, 221: 1, 223: 1, 260: 4, 261: 4}
_LIGHT_TYPES = {"directional": 0, "point": 1, "spot": 2, "hdri": 3}
_SAMPLER_TYPES = {"image1D": 1, "image2D": 2, "image3D": 3, "transform": 4, "primitive": 5}
_WRAP = {"clampToEdge": 0, "repeat": 1, "mirrorRepeat": 2}
_SAMPLER_SLOTS = {"attribute0": 0, "attribute1": 1, "attribute2": 2, "attribute3": 3, "color": 4}


def _column_major(m):
    m = np.eye(4, dtype=np.float32) if m is None else np.asarray(m, np.float32).reshape(4, 4)
    return (C.c_float * 16)(*np.ascontiguousarray(m.T).ravel().tolist())


def stage_image(et, texels):
    """An image sampler's texels as staged (orc_stage_image): (n, 4) float32
    for float element types, else (n, 4) uint8 read as normalised float."""
    lib = load()
    t = np.ascontiguousarray(texels)
    n = t.shape[0]
    f4 = np.zeros((n, 4), np.float32)
    u8 = np.zeros((n, 4), np.uint8)
    r = lib.orc_stage_image(C.c_int(et), _ptr(t), C.c_uint64(n), _ptr(f4), _ptr(u8))
    if r < 0:
        raise ValueError(f"image element type {et} is not supported")
    return f4 if r == 1 else u8


def stage_background(et, texels):
    """The renderer's background image staged as RGBA8 (orc_stage_background)."""
    lib = load()
    t = np.ascontiguousarray(texels)
    n = t.shape[0]
    out = np.zeros((n, 4), np.uint8)
    if lib.orc_stage_background(C.c_int(et), _ptr(t), C.c_uint64(n), _ptr(out)) < 0:
        raise ValueError(f"background element type {et} is not supported")
    return out


def _pack_sampler(o, sp, keep):
    """Fills an OrcSampler from a SamplerSpec, its image staged as the
    device stages it (stage_image)."""
    from visrtx_gb300.scenes import attr_type, sampler_image_type

    o.type = _SAMPLER_TYPES[sp.type]
    o.attribute = _SAMPLER_SLOTS[sp.attribute]
    o.inT = _column_major(sp.in_transform)
    o.outT = _column_major(sp.out_transform)
    o.inO = (C.c_float * 4)(*map(float, sp.in_offset))
    o.outO = (C.c_float * 4)(*map(float, sp.out_offset))
    nd = sp.image_dims
    if nd:
        tex, _ = sp.texels()
        img = np.asarray(sp.image)
        staged = stage_image(sampler_image_type(sp), tex)
        keep.append(staged)
        if staged.dtype == np.float32:
            o.image = _ptr(staged)
        else:
            o.image8 = _ptr(staged)
        shape = img.shape[:nd][::-1]
        o.dims = (C.c_int * 3)(*(list(shape) + [1] * (3 - nd)))
        o.filter = 0 if sp.filter == "nearest" else 1
        o.wrap = (C.c_int * 3)(*[_WRAP[w] for w in sp.wrap])
    elif sp.type == "primitive":
        a = np.ascontiguousarray(sp.array)
        keep.append(a)
        t = attr_type(a)
        o.prim.data = _ptr(a)
        o.prim.type = t
        o.prim.channels = _ATTR_CHANNELS[t]
        o.primOffset = int(sp.offset)


class OrcInstance(C.Structure):
    _fields_ = [("xfm", C.c_float * 12), ("userId", C.c_uint32), ("firstSurface", C.c_int),
                ("numSurfaces", C.c_int)]


class OrcLight(C.Structure):
    _fields_ = [("type", C.c_int), ("direction", C.c_float * 3), ("position", C.c_float * 3),
                ("radiance", C.c_float * 3), ("cosOuter", C.c_float), ("cosInner", C.c_float),
                ("hdri", C.c_void_p), ("hdriW", C.c_int), ("hdriH", C.c_int),
                ("hdriDirection", C.c_float * 3), ("hdriUp", C.c_float * 3),
                ("hdriScale", C.c_float), ("hdriVisible", C.c_int)]


class OrcVolume(C.Structure):
    _fields_ = [("field", C.c_void_p), ("dims", C.c_int * 3), ("origin", C.c_float * 3),
                ("spacing", C.c_float * 3), ("filterLinear", C.c_int), ("tf", C.c_void_p),
                ("valueRange", C.c_float * 2), ("unitDistance", C.c_float),
                ("uniformColor", C.c_float * 3), ("uniformOpacity", C.c_float),
                ("id", C.c_uint32), ("instId", C.c_uint32), ("xfm", C.c_float * 12),
                ("nvdb", C.c_void_p)]


class OrcScene(C.Structure):
    _fields_ = [("surfaces", C.c_void_p), ("numSurfaces", C.c_int), ("instances", C.c_void_p),
                ("numInstances", C.c_int), ("lights", C.c_void_p), ("numLights", C.c_int),
                ("volumes", C.c_void_p), ("numVolumes", C.c_int)]


class OrcCamera(C.Structure):
    _fields_ = [("type", C.c_int), ("position", C.c_float * 3), ("direction", C.c_float * 3),
                ("up", C.c_float * 3), ("fovy", C.c_float), ("aspect", C.c_float),
                ("height", C.c_float), ("imageRegion", C.c_float * 4),
                ("apertureRadius", C.c_float), ("focusDistance", C.c_float)]


class OrcRenderer(C.Structure):
    _fields_ = [("type", C.c_int), ("background", C.c_float * 4), ("ambientColor", C.c_float * 3),
                ("ambientRadiance", C.c_float), ("occlusionDistance", C.c_float),
                ("cullTriangleBackfaces", C.c_int), ("volumeSamplingRate", C.c_float),
                ("pixelSamples", C.c_int), ("ambientSamples", C.c_int), ("maxDepth", C.c_int),
                ("maxRayDepth", C.c_int), ("bgImage", C.c_void_p), ("bgType", C.c_int),
                ("bgW", C.c_int), ("bgH", C.c_int)]


class OrcFrame(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("frameID", C.c_int),
                ("colorFormat", C.c_int), ("rowBegin", C.c_int), ("rowEnd", C.c_int),
                ("accum", C.c_void_p), ("color", C.c_void_p), ("depth", C.c_void_p),
                ("primId", C.c_void_p), ("objId", C.c_void_p), ("instId", C.c_void_p),
                ("raysTraced", C.c_uint64), ("checkerboardID", C.c_int),
                ("albedo", C.c_void_p), ("normal", C.c_void_p),
                ("volumeSamples", C.c_uint64)]


class OrcDMVolume(C.Structure):
    _fields_ = [("density", C.c_void_p), ("dims", C.c_int * 3), ("tf", C.c_void_p),
                ("tfSize", C.c_int), ("opacityScale", C.c_double), ("step", C.c_double),
                ("unitDistance", C.c_double), ("valueLo", C.c_double), ("valueHi", C.c_double)]


class OrcDMView(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("eye", C.c_double * 3),
                ("d00", C.c_double * 3), ("du", C.c_double * 3), ("dv", C.c_double * 3),
                ("background", C.c_double * 3)]


_RENDERERS = {"default": 0, "directLight": 0, "raycast": 1, "ao": 2, "dpt": 3,
              "diffuse_pathtracer": 3}
_ALPHA = {"opaque": 0, "blend": 1, "mask": 2}
_SURFACE_TYPES = {"triangle": 0, "sphere": 1, "quad": 2, "cylinder": 3, "cone": 4, "curve": 5}


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _rows(m4):
    m = np.asarray(m4, np.float32)
    return (C.c_float * 12)(*[float(m[r, c]) for r in range(3) for c in range(4)])


def uniform_sample_disk(radius_s0_s1) -> np.ndarray:
    """(n, 3) of (radius, s0, s1) -> (n, 2) disk samples (the thin lens)."""
    lib = load()
    a = np.ascontiguousarray(radius_s0_s1, np.float32).reshape(-1, 3)
    out = np.zeros((len(a), 2), np.float32)
    lib.orc_uniform_sample_disk(_ptr(a), C.c_int(len(a)), _ptr(out))
    return out


def uniform_sample_cone(cos_s0_s1_s2) -> np.ndarray:
    """(n, 4) of (cosThetaMax, s0, s1, s2) -> (n, 3) cone samples."""
    lib = load()
    a = np.ascontiguousarray(cos_s0_s1_s2, np.float32).reshape(-1, 4)
    out = np.zeros((len(a), 3), np.float32)
    lib.orc_uniform_sample_cone(_ptr(a), C.c_int(len(a)), _ptr(out))
    return out


def project_on_grid(points, dims, box) -> np.ndarray:
    """(n, 3) points -> (n, 3) cells of a dims grid over box (lo, hi)."""
    lib = load()
    p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(dims, np.int32)
    b = np.ascontiguousarray(box, np.float32).reshape(6)
    out = np.zeros((len(p), 3), np.int32)
    lib.orc_project_on_grid(_ptr(p), C.c_int(len(p)), _ptr(d), _ptr(b), _ptr(out))
    return out


def primary_rays(cam, cam_type, samples, inv_w, inv_h, center_pixel=False):
    """Camera record (30 floats: region, pos, dir, dir_00, dir_du, dir_dv,
    scaledAperture, aspect, pos_00, pos_du, pos_dv), type 0 perspective /
    1 orthographic, (n, 6) samples (pixel x, pixel y, r0..r3) -> (n, 8)
    (org, dir, screen): the primary ray of each sample."""
    lib = load()
    c = np.ascontiguousarray(cam, np.float32).reshape(30)
    s = np.ascontiguousarray(samples, np.float32).reshape(-1, 6)
    out = np.zeros((len(s), 8), np.float32)
    lib.orc_primary_rays(_ptr(c), C.c_int(cam_type), _ptr(s), C.c_int(len(s)),
                         C.c_float(inv_w), C.c_float(inv_h), C.c_int(int(center_pixel)), _ptr(out))
    return out


def field_coords(origin, spacing, dims, points):
    """(n, 3) world points -> (n, 3) texture coordinates of a
    structured-regular field (origin, spacing, dims)."""
    lib = load()
    o = np.ascontiguousarray(origin, np.float32).reshape(3)
    s = np.ascontiguousarray(spacing, np.float32).reshape(3)
    d = np.ascontiguousarray(dims, np.int32).reshape(3)
    p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    out = np.zeros((len(p), 3), np.float32)
    lib.orc_field_coords(_ptr(o), _ptr(s), _ptr(d), _ptr(p), C.c_int(len(p)), _ptr(out))
    return out


def volume_interval(rays, box):
    """(n, 8) local rays (org, dir, tmin, tmax) against a volume's bounds
    (lo, hi) -> (hit (n,), t01 (n, 2)): the volume's entry interval."""
    lib = load()
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    b = np.ascontiguousarray(box, np.float32).reshape(6)
    hit = np.zeros(len(r), np.int32)
    t01 = np.zeros((len(r), 2), np.float32)
    lib.orc_volume_interval(_ptr(r), C.c_int(len(r)), _ptr(b), _ptr(hit), _ptr(t01))
    return hit, t01


def dda_walk(rays, dims, box, max_cells):
    """(n, 8) rays (org, dir, tlo, thi) -> (counts (n,), cells (n, max_cells),
    t01 (n, max_cells, 2)): the macrocell walk of the delta-tracking march."""
    lib = load()
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    d = np.ascontiguousarray(dims, np.int32)
    b = np.ascontiguousarray(box, np.float32).reshape(6)
    counts = np.zeros(len(r), np.int32)
    cells = np.full((len(r), max_cells), -1, np.int64)
    t01 = np.zeros((len(r), max_cells, 2), np.float32)
    lib.orc_dda_walk(_ptr(r), C.c_int(len(r)), _ptr(d), _ptr(b), C.c_int(max_cells),
                     _ptr(counts), _ptr(cells), _ptr(t01))
    return counts, cells, t01


def spherical_from_dir(dirs) -> np.ndarray:
    """(n, 3) directions -> (n, 2) (theta, phi) (the HDRI lookup)."""
    lib = load()
    a = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros((len(a), 2), np.float32)
    lib.orc_spherical_from_dir(_ptr(a), C.c_int(len(a)), _ptr(out))
    return out


def write_colors(accum, frame_id: int = 0, fmt: int = 0) -> np.ndarray:
    """The frame's packed colour (sRGB rgba8 for fmt 0, linear rgba8 for 1)
    of accumulated RGBA values after frame_id + 1 samples."""
    lib = load()
    a = np.ascontiguousarray(accum, np.float32).reshape(-1, 4)
    out = np.zeros(len(a), np.uint32)
    lib.orc_write_colors(_ptr(a), C.c_int(len(a)), C.c_int(frame_id), C.c_int(fmt), _ptr(out))
    return out


def discretize_tf(color, opacity, value_range=(0.0, 1.0), uniform_opacity=1.0,
                  uniform_color=(1.0, 1.0, 1.0, 1.0)) -> np.ndarray:
    """The reference's 256-entry TF table; uniform_color (3 or 4 floats, w 1
    when 3) and uniform_opacity stand in for an absent array."""
    lib = load()
    out = np.zeros((256, 4), np.float32)
    c = None if color is None else np.ascontiguousarray(color, np.float32)
    o = None if opacity is None else np.ascontiguousarray(opacity, np.float32)
    uc = np.ones(4, np.float32)
    uc[:len(uniform_color)] = uniform_color
    lib.orc_discretize_tf(_ptr(c), C.c_int(0 if c is None else len(c)),
                          C.c_int(0 if c is None else c.shape[1]), _ptr(o),
                          C.c_int(0 if o is None else len(o)), C.c_float(value_range[0]),
                          C.c_float(value_range[1]), _ptr(uc), C.c_float(uniform_opacity),
                          _ptr(out))
    return out


def render(spec, frame_id: int = 0, rows: tuple[int, int] | None = None, volume_mode: int = 0,
           tex_round: int = 1, threads: int = 0, accum=None, depth=None):
    """Renders `spec` on the CPU. Returns a dict of numpy outputs (color as
    packed sRGB uint32, depth, primitiveId, objectId, instanceId, accum)
    plus 'rays' (rays traced)."""
    sc = OracleScene(spec)
    try:
        return sc.render(frame_id, rows, volume_mode, tex_round, threads, accum, depth)
    finally:
        sc.release()


class OracleScene:
    """The oracle's acceleration structures for one spec, built once."""

    def __init__(self, spec):
        self.spec = spec
        self.lib = load()
        self._keep, self._scene = _scene_structs(spec)
        self.lib.orc_prepare.restype = C.c_void_p
        self.handle = C.c_void_p(self.lib.orc_prepare(C.byref(self._scene)))

    def release(self):
        if self.handle:
            self.lib.orc_release(self.handle)
            self.handle = None

    def render(self, frame_id=0, rows=None, volume_mode=0, tex_round=1, threads=0, accum=None,
               depth=None, spec=None, ids=None, checkerboard_id=-1, channels=False):
        """ids: a previous result dict whose id buffers (and colour, albedo
        and normal accumulations) carry over: ids are only rewritten where
        the depth improves, and a checkerboard pass leaves the other pixels'
        colour as it was. channels: also accumulate the albedo and normal
        channels."""
        return _render_prepared(self.lib, self.handle, spec or self.spec, frame_id, rows,
                                volume_mode, tex_round, threads, accum, depth, ids,
                                checkerboard_id, channels)


def _scene_structs(spec):
    keep = []
    surfs = (OrcSurface * max(1, len(spec.surfaces)))()
    for i, s in enumerate(spec.surfaces):
        o = surfs[i]
        o.type = _SURFACE_TYPES[s.type]
        v = np.ascontiguousarray(s.vertices, np.float32)
        keep.append(v)
        o.vertices = _ptr(v)
        if s.indices is not None:
            ix = np.ascontiguousarray(s.indices, np.uint32)
            keep.append(ix)
            o.indices = _ptr(ix)
        o.numPrims = s.num_prims
        for name, arr, dt in (("normals", s.normals, np.float32), ("primIds", s.prim_ids, np.uint32),
                              ("radii", s.radii, np.float32)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dt)
                keep.append(a)
                setattr(o, name, _ptr(a))
        o.radius = s.radius
        o.cullBackfaces = int(bool(s.cull))
        o.id = s.id & 0xFFFFFFFF
        from visrtx_gb300.scenes import SamplerSpec
        if isinstance(s.color, SamplerSpec):
            o.colorSrc = 10
            _pack_sampler(o.colorSampler, s.color, keep)
            o.color = (C.c_float * 3)(0.8, 0.8, 0.8)
            o.colorW = 1.0
        elif isinstance(s.color, str):
            o.colorSrc = _PARAM_SOURCES[s.color]
            o.color = (C.c_float * 3)(0.8, 0.8, 0.8)
            o.colorW = 1.0
        else:
            o.color = (C.c_float * 3)(*map(float, s.color[:3]))
            o.colorW = float(s.color[3]) if len(s.color) == 4 else 1.0
        if isinstance(s.opacity, SamplerSpec):
            o.opacitySrc = 10
            _pack_sampler(o.opacitySampler, s.opacity, keep)
            o.opacity = 1.0
        elif isinstance(s.opacity, str):
            o.opacitySrc = _PARAM_SOURCES[s.opacity]
            o.opacity = 1.0
        else:
            o.opacity = s.opacity
        o.materialType = 1 if s.material == "physicallyBased" else 0
        o.ior = float(s.ior)
        for name in ("metallic", "roughness"):
            val = getattr(s, name)
            if isinstance(val, SamplerSpec):
                setattr(o, name + "Src", 10)
                _pack_sampler(getattr(o, name + "Sampler"), val, keep)
                setattr(o, name, 1.0)
            elif isinstance(val, str):
                setattr(o, name + "Src", _PARAM_SOURCES[val])
                setattr(o, name, 1.0)
            else:
                setattr(o, name, float(val))
        from visrtx_gb300.scenes import attr_type
        for k, slot in enumerate(_ATTR_SLOTS):
            o.uattr[k] = (C.c_float * 4)(0.0, 0.0, 0.0, 1.0)
            for prefix, dst in (("vertex.", o.vattr), ("primitive.", o.pattr)):
                a = s.attrs.get(prefix + slot)
                if a is not None:
                    a = np.ascontiguousarray(a)
                    keep.append(a)
                    t = attr_type(a)
                    dst[k].data = _ptr(a)
                    dst[k].type = t
                    dst[k].channels = _ATTR_CHANNELS[t]
            if slot in s.attrs:
                o.uattr[k] = (C.c_float * 4)(*map(float, s.attrs[slot]))
        o.alphaMode = _ALPHA[s.alpha_mode]
        o.cutoff = s.cutoff
        o.caps = int(bool(s.caps))
    insts = []
    for ins in spec.instances:
        if not ins.surfaces:
            continue
        first = min(ins.surfaces)
        assert sorted(ins.surfaces) == list(range(first, first + len(ins.surfaces)))
        oi = OrcInstance()
        oi.xfm = _rows(np.eye(4) if ins.zero else ins.xfm)
        oi.userId = (spec.world_id if ins.zero else ins.id) & 0xFFFFFFFF
        oi.firstSurface = first
        oi.numSurfaces = len(ins.surfaces)
        insts.append(oi)
    inst_arr = (OrcInstance * max(1, len(insts)))(*insts)
    lights = (OrcLight * max(1, len(spec.lights)))()
    for i, l in enumerate(spec.lights):
        o = lights[i]
        o.type = _LIGHT_TYPES[l.type]
        o.direction = (C.c_float * 3)(*map(float, l.direction))
        o.position = (C.c_float * 3)(*map(float, l.position))
        level = np.float32(max(0.0, l.irradiance))
        rad = [float(np.float32(c) * level) for c in l.color]
        o.radiance = (C.c_float * 3)(*rad)
        if l.type == "spot":
            inner = np.float32(l.opening_angle) - np.float32(2.0) * np.float32(l.falloff_angle)
            o.cosOuter = float(np.cos(np.float32(l.opening_angle)))
            o.cosInner = float(np.cos(inner))
        if l.type == "hdri":
            img = np.ascontiguousarray(l.radiance, np.float32)
            keep.append(img)
            o.hdri = _ptr(img)
            o.hdriH, o.hdriW = img.shape[0], img.shape[1]
            o.hdriDirection = (C.c_float * 3)(*map(float, l.hdri_direction))
            o.hdriUp = (C.c_float * 3)(*map(float, l.hdri_up))
            o.hdriScale = float(l.scale)
            o.hdriVisible = int(bool(l.visible))
    vols = (OrcVolume * max(1, len(spec.volumes)))()
    for i, v in enumerate(spec.volumes):
        _pack_volume(v, vols[i], keep, spec.world_id)
    scene = OrcScene(C.cast(surfs, C.c_void_p), len(spec.surfaces), C.cast(inst_arr, C.c_void_p),
                     len(insts), C.cast(lights, C.c_void_p), len(spec.lights),
                     C.cast(vols, C.c_void_p), len(spec.volumes))
    keep += [surfs, inst_arr, lights, vols]
    return keep, scene


def _pack_volume(v, o, keep, world_id):
    if v.nvdb is not None:
        g = np.ascontiguousarray(v.nvdb, np.uint8)
        keep.append(g)
        o.nvdb = _ptr(g)
    else:
        f = np.ascontiguousarray(v.field, np.float32)
        keep.append(f)
        o.field = _ptr(f)
        o.dims = (C.c_int * 3)(f.shape[2], f.shape[1], f.shape[0])
    o.origin = (C.c_float * 3)(*map(float, v.origin))
    o.spacing = (C.c_float * 3)(*map(float, v.spacing))
    o.filterLinear = int(v.filter != "nearest")
    if v.color is not None or v.opacity is not None:
        tf = discretize_tf(v.color, v.opacity, v.value_range, v.uniform_opacity,
                           v.uniform_color)
        keep.append(tf)
        o.tf = _ptr(tf)
    o.valueRange = (C.c_float * 2)(*map(float, v.value_range))
    o.unitDistance = v.unit_distance
    o.uniformColor = (C.c_float * 3)(*map(float, v.uniform_color))
    o.uniformOpacity = v.uniform_opacity
    o.id = v.id & 0xFFFFFFFF
    o.instId = world_id & 0xFFFFFFFF
    o.xfm = _rows(np.eye(4))


def nvdb_sample(grid, xyz, fused: bool = True) -> np.ndarray:
    """Samples a NanoVDB grid buffer at world-space points (n, 3) the way the
    reference's field sampler does; fused=False rounds like NanoVDB compiled
    for the host, fused=True like the device build."""
    lib = load()
    g = np.ascontiguousarray(grid, np.uint8)
    p = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    out = np.zeros(len(p), np.float32)
    if lib.orc_nvdb_sample(_ptr(g), _ptr(p), C.c_int(len(p)), C.c_int(int(fused)), _ptr(out)) != 0:
        raise ValueError("not a NanoVDB grid this reader accepts")
    return out


def dpt_majorants(vspec, tex_round: int = 1) -> np.ndarray:
    """The reference's delta-tracking majorant grid of one volume (the dpt
    renderer's Woodcock bound), shape (ceil(nz/16), ceil(ny/16), ceil(nx/16))."""
    lib = load()
    keep = []
    o = OrcVolume()
    _pack_volume(vspec, o, keep, 0)
    if vspec.nvdb is not None:
        from visrtx_gb300.nanovdb import grid_info

        lo, hi = grid_info(vspec.nvdb)["index_bbox"]
        nx, ny, nz = (h - l + 1 for l, h in zip(lo, hi))
    else:
        nz, ny, nx = np.asarray(vspec.field).shape
    md = ((nz + 15) // 16, (ny + 15) // 16, (nx + 15) // 16)
    out = np.zeros(md, np.float32)
    lib.orc_dpt_majorants(C.byref(o), C.c_int(tex_round), _ptr(out))
    return out


def _render_prepared(lib, handle, spec, frame_id, rows, volume_mode, tex_round, threads, accum,
                     depth, ids=None, checkerboard_id=-1, channels=False):
    c = spec.camera
    cam = OrcCamera()
    cam.type = 0 if c.type == "perspective" else 1
    cam.position = (C.c_float * 3)(*map(float, c.position))
    cam.direction = (C.c_float * 3)(*map(float, c.direction))
    cam.up = (C.c_float * 3)(*map(float, c.up))
    cam.fovy = c.fovy
    cam.aspect = c.aspect
    cam.height = c.height
    cam.imageRegion = (C.c_float * 4)(*map(float, c.region))
    cam.apertureRadius = c.aperture
    cam.focusDistance = c.focus
    r = spec.renderer
    ren = OrcRenderer()
    ren.type = _RENDERERS[r.subtype]
    ren.background = (C.c_float * 4)(*map(float, r.background))
    ren.ambientColor = (C.c_float * 3)(*map(float, r.ambient_color))
    ren.ambientRadiance = r.resolved_ambient()
    ren.occlusionDistance = r.ao_distance
    ren.cullTriangleBackfaces = int(bool(r.cull))
    ren.volumeSamplingRate = r.volume_sampling_rate
    # checkerboarding forces one sample per pass (Renderer.cpp:168-169)
    ren.pixelSamples = 1 if r.checkerboard else r.pixel_samples
    ren.ambientSamples = r.ambient_samples if ren.type in (0, 2) else 0
    ren.maxDepth = r.max_depth
    ren.maxRayDepth = r.max_ray_depth
    bg_keep = None
    if r.background_image is not None:
        from visrtx_gb300.scenes import background_image_type
        bg_keep = np.ascontiguousarray(r.background_image)
        ren.bgImage = bg_keep.ctypes.data_as(C.c_void_p)
        ren.bgType = background_image_type(bg_keep, r.background_srgb)
        ren.bgH, ren.bgW = bg_keep.shape[0], bg_keep.shape[1]
    W, H = spec.width, spec.height
    out = {
        "accum": np.zeros((H, W, 4), np.float32) if accum is None else accum,
        "color": np.zeros((H, W), np.uint32),
        "depth": np.full((H, W), np.finfo(np.float32).max, np.float32) if depth is None else depth,
        "primitiveId": np.zeros((H, W), np.uint32) if ids is None else ids["primitiveId"],
        "objectId": np.zeros((H, W), np.uint32) if ids is None else ids["objectId"],
        "instanceId": np.zeros((H, W), np.uint32) if ids is None else ids["instanceId"],
    }
    if ids is not None and "color" in ids:
        out["color"] = ids["color"]
    if channels:
        for ch in ("albedo", "normal"):
            out[ch] = (ids[ch] if ids is not None and ch in ids
                       else np.zeros((H, W, 3), np.float32))
    fr = OrcFrame()
    fr.width, fr.height, fr.frameID, fr.colorFormat = W, H, frame_id, 0
    fr.rowBegin, fr.rowEnd = (0, H) if rows is None else rows
    fr.accum = _ptr(out["accum"])
    fr.color = _ptr(out["color"])
    fr.depth = _ptr(out["depth"])
    fr.primId = _ptr(out["primitiveId"])
    fr.objId = _ptr(out["objectId"])
    fr.instId = _ptr(out["instanceId"])
    fr.checkerboardID = checkerboard_id
    fr.albedo = _ptr(out.get("albedo"))
    fr.normal = _ptr(out.get("normal"))
    rc = lib.orc_render_prepared(handle, C.byref(cam), C.byref(ren), C.byref(fr),
                                 C.c_int(volume_mode), C.c_int(tex_round), C.c_int(threads))
    assert rc == 0
    out["rays"] = int(fr.raysTraced)
    out["volume_samples"] = int(fr.volumeSamples)
    return out


def philox_stream(seed: int, subsequence: int, offset: int, kind: int, n: int) -> np.ndarray:
    lib = load()
    out = np.zeros(n, np.uint32 if kind == 0 else np.float32)
    lib.orc_philox_stream(C.c_uint64(seed), C.c_uint64(subsequence), C.c_uint64(offset),
                          C.c_int(kind), C.c_int(n), _ptr(out))
    return out


def philox_block(ctr, key) -> np.ndarray:
    lib = load()
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib.orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def tex1d(table: np.ndarray, coord: float, round_mode: int = 1) -> np.ndarray:
    lib = load()
    t = np.ascontiguousarray(table, np.float32)
    comps = t.shape[1] if t.ndim == 2 else 1
    out = np.zeros(comps, np.float32)
    lib.orc_tex1d(_ptr(t), C.c_int(len(t)), C.c_int(comps), C.c_float(coord), C.c_int(round_mode),
                  _ptr(out))
    return out


def tex3d(vox: np.ndarray, coord, round_mode: int = 1) -> float:
    lib = load()
    v = np.ascontiguousarray(vox, np.float32)
    dims = np.array([v.shape[2], v.shape[1], v.shape[0]], np.int32)
    c = np.asarray(coord, np.float32)
    return float(lib.orc_tex3d(_ptr(v), _ptr(dims), _ptr(c), C.c_int(round_mode)))


def tex_float4(texels: np.ndarray, dims, filter_: int, wrap, coord) -> np.ndarray:
    """Float4 texture fetch (texels (..., 4) with x fastest; dims per axis;
    filter 0 point / 1 linear; wrap per axis 0 clamp / 1 repeat / 2 mirror)
    as the texture unit computes it."""
    lib = load()
    t = np.ascontiguousarray(texels, np.float32)
    nd = len(dims)
    d = np.array(list(dims) + [1] * (3 - nd), np.int32)
    w = np.array(list(wrap) + [0] * (3 - nd), np.int32)
    c = np.array(list(coord) + [0.0] * (3 - nd), np.float32)
    out = np.zeros(4, np.float32)
    lib.orc_tex_float4(_ptr(t), C.c_int(nd), _ptr(d), C.c_int(filter_), _ptr(w), _ptr(c),
                       _ptr(out))
    return out


def tex_unorm8(texels: np.ndarray, dims, filter_: int, wrap, coord) -> np.ndarray:
    """tex_float4's fetch from RGBA8 texels (..., 4) read as normalised float,
    as an 8-bit image sampler's texture is read."""
    lib = load()
    t = np.ascontiguousarray(texels, np.uint8)
    nd = len(dims)
    d = np.array(list(dims) + [1] * (3 - nd), np.int32)
    w = np.array(list(wrap) + [0] * (3 - nd), np.int32)
    c = np.array(list(coord) + [0.0] * (3 - nd), np.float32)
    out = np.zeros(4, np.float32)
    lib.orc_tex_unorm8(_ptr(t), C.c_int(nd), _ptr(d), C.c_int(filter_), _ptr(w), _ptr(c),
                       _ptr(out))
    return out


def tex_norm16(texels: np.ndarray, dims, filter_: int, wrap, coord, scale: int) -> float:
    """Read of a single-channel 16-bit normalised texture (integer texels, x
    fastest; scale 65535 unsigned / 32767 signed)."""
    lib = load()
    t = np.ascontiguousarray(texels, np.int32)
    nd = len(dims)
    d = np.array(list(dims) + [1] * (3 - nd), np.int32)
    w = np.array(list(wrap) + [0] * (3 - nd), np.int32)
    c = np.array(list(coord) + [0.0] * (3 - nd), np.float32)
    lib.orc_tex_norm16.restype = C.c_float
    return float(lib.orc_tex_norm16(_ptr(t), C.c_int(nd), _ptr(d), C.c_int(filter_), _ptr(w),
                                    _ptr(c), C.c_int(scale)))


def tex_rgba8(texels: np.ndarray, width: int, height: int, coord) -> np.ndarray:
    """Linear, clamped, normalised-float fetch of an RGBA8 image (the
    background image's texture)."""
    lib = load()
    t = np.ascontiguousarray(texels, np.uint8)
    c = np.asarray(coord, np.float32)
    out = np.zeros(4, np.float32)
    lib.orc_tex_rgba8(_ptr(t), C.c_int(width), C.c_int(height), _ptr(c), _ptr(out))
    return out


def bvh8_count(nodes: bytes, tris: bytes, rays: np.ndarray):
    lib = load()
    nb = np.frombuffer(nodes, np.uint8)
    tb = np.frombuffer(tris, np.uint8)
    r = np.ascontiguousarray(rays, np.float32)
    nv, pt = C.c_uint64(), C.c_uint64()
    th = np.zeros(len(r), np.float32)
    lib.orc_bvh8_count(_ptr(nb), _ptr(tb), _ptr(r), C.c_int(len(r)), C.byref(nv), C.byref(pt),
                       _ptr(th))
    return int(nv.value), int(pt.value), th


def dm(density: np.ndarray, tf: np.ndarray, view: dict, opacity_scale: float, step: float,
       unit: float = 1.0, value_range=(0.0, 1.0), grad_image: np.ndarray | None = None,
       threads: int = 0):
    """FP64 forward (and adjoint when grad_image is given) of the
    differentiable marcher for one view. density: (nz, ny, nx); view:
    width, height, eye, d00, du, dv, background (voxel space)."""
    lib = load()
    d = np.ascontiguousarray(density, np.float64)
    t = np.ascontiguousarray(tf, np.float64)
    ov = OrcDMVolume(_ptr(d), (C.c_int * 3)(d.shape[2], d.shape[1], d.shape[0]), _ptr(t), len(t),
                     opacity_scale, step, unit, value_range[0], value_range[1])
    vw = OrcDMView()
    vw.width, vw.height = view["width"], view["height"]
    for k in ("eye", "d00", "du", "dv", "background"):
        setattr(vw, k, (C.c_double * 3)(*map(float, view[k])))
    img = np.zeros((view["height"], view["width"], 3), np.float64)
    gD = gT = gS = None
    if grad_image is not None:
        g = np.ascontiguousarray(grad_image, np.float64)
        gD = np.zeros_like(d)
        gT = np.zeros_like(t)
        gS = np.zeros(1, np.float64)
        lib.orc_dm(C.byref(ov), C.byref(vw), _ptr(img), _ptr(g), _ptr(gD), _ptr(gT), _ptr(gS),
                   C.c_int(threads))
        return img, gD, gT, float(gS[0])
    lib.orc_dm(C.byref(ov), C.byref(vw), _ptr(img), None, None, None, None, C.c_int(threads))
    return img
