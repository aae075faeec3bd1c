"""Seeded synthetic scenes for the five benchmark workloads.

Random numbers come from a counter-based SplitMix64 (Steele, Lea, Flood,
"Fast splittable pseudorandom number generators", OOPSLA 2014) with
Box-Muller normals, so the same seed gives the same scene on every machine
and numpy version.

Workloads:
  soup      100k-triangle FP32 soup, centres U[0,1]^3, edge offsets
            N(0, 0.01^2), one instance, 512x384 pinhole camera at
            (0.5, 0.5, -1.5) looking +z, fovy 40 deg.
  instanced 64 instances of a displaced icosphere (subdivision 8,
            r = 1 + 0.05 * valueNoise(p)) under random rotation / scale
            [0.5, 2] / translation [-10, 10]^3, plus 1M spheres (centres
            U[-10,10]^3, radius U[0.001, 0.01]); 1920x1080, AO renderer.
  volume    512^3 FP32 clamped sum of 64 Gaussians, 256-entry TF from
            8-knot ramps, 16^3 macrocells, step 0.5 voxel, 1920x1080.
  dm        256^3 FP16 density (32 blobs), 128 Fibonacci-sphere cameras
            at radius 2, 512x512 each.
  batched   64 volumes with edges U[64,384], BF16, own TFs, 4-32 views
            each at {256,512,1024}^2.
"""
from __future__ import annotations

import math

import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)


class Rng:
    """Counter-based SplitMix64 stream: value i = mix(seed' + (i+1)*golden)."""

    def __init__(self, seed: int, stream: int = 0):
        with np.errstate(over="ignore"):
            s = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
            s = s * np.uint64(0x9FB21C651E98DF25) + np.uint64(stream) * _C1
        self.base = np.uint64(s)
        self.count = 0

    def u64(self, n: int) -> np.ndarray:
        i = np.arange(self.count + 1, self.count + n + 1, dtype=np.uint64)
        self.count += n
        with np.errstate(over="ignore"):
            z = self.base + i * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _C1
            z = (z ^ (z >> np.uint64(27))) * _C2
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """float64 in [lo, hi) from the top 53 bits."""
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def normal(self, n: int) -> np.ndarray:
        m = (n + 1) // 2
        u1 = self.uniform(m)
        u2 = self.uniform(m)
        r = np.sqrt(-2.0 * np.log1p(-u1))
        z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
        return z[:n]


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------

def triangle_soup(n: int = 100_000, seed: int = 0, sigma: float = 0.01) -> np.ndarray:
    """(n, 3, 3) float32: n independent triangles."""
    rng = Rng(seed)
    centers = rng.uniform(3 * n).reshape(n, 3)
    offs = rng.normal(9 * n).reshape(n, 3, 3) * sigma
    return (centers[:, None, :] + offs).astype(np.float32)


def icosphere(subdiv: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (V, 3) float64 vertices, (F, 3) uint32 faces, CCW
    seen from outside. F = 20 * 4^subdiv."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                 dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                  [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                  [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        es = np.sort(e, axis=1)
        uniq, inv = np.unique(es, axis=0, return_inverse=True)
        mids = v[uniq[:, 0]] + v[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mids])
        nf = len(f)
        m01 = base + inv[:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([m01, f[:, 1], m12], 1),
            np.stack([m20, m12, f[:, 2]], 1),
            np.stack([m01, m12, m20], 1)])
    return v, f.astype(np.uint32)


def value_noise(p: np.ndarray, seed: int, freq: float = 4.0, lattice: int = 32) -> np.ndarray:
    """Trilinear value noise in [-1, 1] on a seeded `lattice`^3 grid of
    U[-1,1] values, sampled at p * freq (wrapping)."""
    rng = Rng(seed, stream=7)
    g = rng.uniform(lattice ** 3, -1.0, 1.0).reshape(lattice, lattice, lattice)
    q = (p * freq) % lattice
    i0 = np.floor(q).astype(np.int64)
    f = q - i0
    i1 = (i0 + 1) % lattice
    out = np.zeros(len(p))
    for dx in (0, 1):
        wx = f[:, 0] if dx else 1 - f[:, 0]
        ix = i1[:, 0] if dx else i0[:, 0]
        for dy in (0, 1):
            wy = f[:, 1] if dy else 1 - f[:, 1]
            iy = i1[:, 1] if dy else i0[:, 1]
            for dz in (0, 1):
                wz = f[:, 2] if dz else 1 - f[:, 2]
                iz = i1[:, 2] if dz else i0[:, 2]
                out += wx * wy * wz * g[ix, iy, iz]
    return out


def displaced_icosphere(subdiv: int = 8, amp: float = 0.05, seed: int = 0):
    v, f = icosphere(subdiv)
    r = 1.0 + amp * value_noise(v, seed)
    return (v * r[:, None]).astype(np.float32), f


def random_instances(n: int = 64, seed: int = 0) -> np.ndarray:
    """(n, 4, 4) float32 row-major affine transforms: uniform rotation
    (normalised quaternion of 4 normals), scale U[0.5, 2], translation
    U[-10, 10]^3."""
    rng = Rng(seed, stream=3)
    q = rng.normal(4 * n).reshape(n, 4)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    s = rng.uniform(n, 0.5, 2.0)
    t = rng.uniform(3 * n, -10.0, 10.0).reshape(n, 3)
    w, x, y, z = q.T
    R = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], 1)
    M = np.zeros((n, 4, 4))
    M[:, :3, :3] = R * s[:, None, None]
    M[:, :3, 3] = t
    M[:, 3, 3] = 1.0
    return M.astype(np.float32)


def random_spheres(n: int = 1_000_000, seed: int = 0):
    rng = Rng(seed, stream=5)
    c = rng.uniform(3 * n, -10.0, 10.0).reshape(n, 3).astype(np.float32)
    r = rng.uniform(n, 0.001, 0.01).astype(np.float32)
    return c, r


# ---------------------------------------------------------------------------
# volumes and transfer functions
# ---------------------------------------------------------------------------

def blob_params(n_blobs: int, dims, seed: int):
    rng = Rng(seed, stream=11)
    dims = np.asarray(dims, np.float64)
    c = rng.uniform(3 * n_blobs).reshape(n_blobs, 3) * dims
    sig = rng.uniform(n_blobs, 8.0, 48.0)
    amp = rng.uniform(n_blobs, 0.2, 1.0)
    return c, sig, amp


def gaussian_blobs(dims=(512, 512, 512), n_blobs: int = 64, seed: int = 0,
                   device: str | None = None, sigma_scale: float = 1.0):
    """clamp(sum_k A_k exp(-|x - c_k|^2 / (2 sigma_k^2)), 0, 1) on the voxel
    centres; returns a (nz, ny, nx) float32 array (x fastest). Uses torch
    (on `device`) when given, numpy otherwise. sigma_scale shrinks blobs for
    small test grids."""
    nx, ny, nz = dims
    c, sig, amp = blob_params(n_blobs, dims, seed)
    sig = sig * sigma_scale
    if device is not None:
        import torch
        out = torch.zeros((nz, ny, nx), dtype=torch.float32, device=device)
        ax = [torch.arange(n, dtype=torch.float32, device=device) for n in (nx, ny, nz)]
        for k in range(n_blobs):
            s2 = 2.0 * sig[k] * sig[k]
            gx = torch.exp(-(ax[0] - float(c[k, 0])) ** 2 / s2)
            gy = torch.exp(-(ax[1] - float(c[k, 1])) ** 2 / s2)
            gz = torch.exp(-(ax[2] - float(c[k, 2])) ** 2 / s2)
            out.add_(float(amp[k]) * gz[:, None, None] * gy[None, :, None] * gx[None, None, :])
        return out.clamp_(0.0, 1.0)
    out = np.zeros((nz, ny, nx), np.float32)
    ax = [np.arange(n, dtype=np.float64) for n in (nx, ny, nz)]
    for k in range(n_blobs):
        s2 = 2.0 * sig[k] * sig[k]
        gx = np.exp(-(ax[0] - c[k, 0]) ** 2 / s2)
        gy = np.exp(-(ax[1] - c[k, 1]) ** 2 / s2)
        gz = np.exp(-(ax[2] - c[k, 2]) ** 2 / s2)
        out += (amp[k] * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]).astype(np.float32)
    return np.clip(out, 0.0, 1.0)


def tf_knots(seed: int = 0, n: int = 8, max_opacity: float = 0.2):
    """8 RGB knots U[0,1] and 8 opacity knots (first 0, rest U[0, max])."""
    rng = Rng(seed, stream=13)
    color = rng.uniform(3 * n).reshape(n, 3).astype(np.float32)
    op = rng.uniform(n, 0.0, max_opacity).astype(np.float32)
    op[0] = 0.0
    return color, op


def tf_table(color: np.ndarray, opacity: np.ndarray, n: int = 256) -> np.ndarray:
    """(n, 4) float32 table: knots spread uniformly, piecewise-linear."""
    x = np.linspace(0.0, 1.0, n)
    kc = np.linspace(0.0, 1.0, len(color))
    ko = np.linspace(0.0, 1.0, len(opacity))
    out = np.empty((n, 4), np.float32)
    for ch in range(3):
        out[:, ch] = np.interp(x, kc, color[:, ch])
    out[:, 3] = np.interp(x, ko, opacity)
    return out


# ---------------------------------------------------------------------------
# cameras
# ---------------------------------------------------------------------------

def look_at(pos, target, up=(0.0, 1.0, 0.0)):
    pos = np.asarray(pos, np.float64)
    d = np.asarray(target, np.float64) - pos
    return pos, d / np.linalg.norm(d), np.asarray(up, np.float64)


def orbit_position(center, radius: float, azimuth_deg: float, elevation_deg: float):
    a, e = math.radians(azimuth_deg), math.radians(elevation_deg)
    return (np.asarray(center, np.float64)
            + radius * np.array([math.sin(a) * math.cos(e), math.sin(e), math.cos(a) * math.cos(e)]))


def fibonacci_sphere(n: int) -> np.ndarray:
    i = np.arange(n, dtype=np.float64) + 0.5
    phi = np.arccos(1.0 - 2.0 * i / n)
    theta = np.pi * (1.0 + 5.0 ** 0.5) * i
    return np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], 1)


def pinhole_basis(pos, target, fovy_deg: float, width: int, height: int, up=(0.0, 1.0, 0.0)):
    """(d00, du, dv) for dir = normalize(d00 + (x+.5) du + (y+.5) dv), y down
    the image rows from the top... rows run along +dv."""
    pos, d, up = look_at(pos, target, up)
    if abs(np.dot(d, up)) > 0.999:
        up = np.array([1.0, 0.0, 0.0])
    right = np.cross(d, up)
    right /= np.linalg.norm(right)
    true_up = np.cross(right, d)
    h = 2.0 * math.tan(math.radians(fovy_deg) / 2.0)
    w = h * width / height
    du = right * (w / width)
    dv = true_up * (h / height)
    d00 = d - 0.5 * w * right - 0.5 * h * true_up
    return d00, du, dv


# ---------------------------------------------------------------------------
# scene specification shared by the ANARI-side builder and the oracle
# ---------------------------------------------------------------------------

from dataclasses import dataclass, field as _field


@dataclass
class SamplerSpec:
    """A material sampler (sampler/Image1D.cpp, Image2D.cpp, Image3D.cpp,
    TransformSampler.cpp, PrimitiveSampler.cpp): "image1D" / "image2D" /
    "image3D" over `image` ((n[, c]) / (ny, nx[, c]) / (nz, ny, nx[, c]);
    float32 x1-4, uint8 x1 / x4, uint16 x1; uint8 x4 sRGB-encoded when
    image_srgb), "transform", or "primitive" over `array` (an
    attribute-typed array read at primID + offset). Transforms are 4x4 in
    row-major (math) layout."""
    type: str
    image: np.ndarray | None = None
    image_srgb: bool = False
    array: np.ndarray | None = None
    offset: int = 0
    attribute: str = "attribute0"
    filter: str = "linear"
    wrap: tuple = ("clampToEdge", "clampToEdge", "clampToEdge")
    in_transform: np.ndarray | None = None
    in_offset: tuple = (0.0, 0.0, 0.0, 0.0)
    out_transform: np.ndarray | None = None
    out_offset: tuple = (0.0, 0.0, 0.0, 0.0)

    @property
    def image_dims(self) -> int:
        return int(self.type[5]) if self.type.startswith("image") else 0

    def texels(self) -> tuple[np.ndarray, int]:
        """The image as (texels, channels): texels reshaped to (n, c)."""
        nd = self.image_dims
        img = np.ascontiguousarray(self.image)
        c = img.shape[nd] if img.ndim > nd else 1
        return img.reshape(-1, c) if c > 1 else img.reshape(-1), c


@dataclass
class SurfaceSpec:
    type: str  # "triangle" | "quad" | "sphere" | "cylinder" | "cone" | "curve"
    vertices: np.ndarray  # (n, 3) float32
    # triangle (m, 3), quad (m, 4), cylinder / cone (m, 2), sphere / curve (m,)
    indices: np.ndarray | None = None
    normals: np.ndarray | None = None
    prim_ids: np.ndarray | None = None
    # sphere / cone / curve: per vertex ("vertex.radius"); cylinder: per
    # primitive ("primitive.radius")
    radii: np.ndarray | None = None
    radius: float = 0.01  # "radius" (sphere 0.01; cylinder / curve take 1 by default)
    caps: bool = False  # cylinder "caps"
    # geometry attributes: "vertex.<slot>" / "primitive.<slot>" -> array,
    # "<slot>" -> uniform 4-tuple; slots attribute0..3, color. Arrays:
    # float32 (n,) / (n, 2..4), uint8 (n,) / (n, 4), uint16 (n,)
    attrs: dict = _field(default_factory=dict)
    cull: bool = False
    id: int = 0xFFFFFFFF
    # value, an attribute / hit quantity name, or a SamplerSpec
    color: tuple | str | SamplerSpec = (0.8, 0.8, 0.8)
    opacity: float | str | SamplerSpec = 1.0
    alpha_mode: str = "opaque"
    cutoff: float = 0.5
    # "matte" or "physicallyBased" (color is then "baseColor"); metallic and
    # roughness: a value, an attribute / hit quantity name or a SamplerSpec
    material: str = "matte"
    metallic: float | str | SamplerSpec = 1.0
    roughness: float | str | SamplerSpec = 1.0
    ior: float = 1.5

    @property
    def num_prims(self) -> int:
        """Primitives as the device numbers them (a quad is two triangles;
        an unindexed curve has n/2 segments, Curve.cpp:88-99)."""
        n = len(self.indices) if self.indices is not None else None
        v = len(self.vertices)
        if self.type == "triangle":
            return n if n is not None else v // 3
        if self.type == "quad":
            return 2 * (n if n is not None else v // 4)
        if self.type in ("cylinder", "cone", "curve"):
            return n if n is not None else v // 2
        return n if n is not None else v


@dataclass
class InstanceSpec:
    surfaces: list  # indices into SceneSpec.surfaces (a contiguous range)
    xfm: np.ndarray = _field(default_factory=lambda: np.eye(4, dtype=np.float32))
    id: int = 0xFFFFFFFF
    zero: bool = False  # surfaces set directly on the world


@dataclass
class LightSpec:
    """A light (scene/light/*.cpp): "directional" (direction, irradiance),
    "point" / "spot" (position, intensity = `irradiance`; spot: direction,
    opening_angle, falloff_angle) or "hdri" (radiance (H, W, 3) float32,
    hdri_direction, hdri_up, scale, visible)."""
    type: str = "directional"
    direction: tuple = (0.0, 0.0, -1.0)
    color: tuple = (1.0, 1.0, 1.0)
    irradiance: float = 1.0
    position: tuple = (0.0, 0.0, 0.0)
    opening_angle: float = math.pi
    falloff_angle: float = 0.1
    radiance: np.ndarray | None = None
    hdri_direction: tuple = (1.0, 0.0, 0.0)
    hdri_up: tuple = (0.0, 0.0, 1.0)
    scale: float = 1.0
    visible: bool = True


@dataclass
class VolumeSpec:
    field: np.ndarray | None  # (nz, ny, nx) float32; None for a NanoVDB field
    origin: tuple = (0.0, 0.0, 0.0)
    spacing: tuple = (1.0, 1.0, 1.0)
    filter: str = "linear"
    color: np.ndarray | None = None  # (k, 3) float32 knots
    opacity: np.ndarray | None = None  # (k,) float32 knots
    value_range: tuple = (0.0, 1.0)
    unit_distance: float = 1.0
    id: int = 0xFFFFFFFF
    uniform_color: tuple = (1.0, 1.0, 1.0)
    uniform_opacity: float = 1.0
    # a NanoVDB grid buffer (uint8, see nanovdb.build_grid): the volume's
    # field is then a "nanovdb" spatial field and `field` is unused
    nvdb: np.ndarray | None = None


@dataclass
class CameraSpec:
    type: str = "perspective"
    position: tuple = (0.0, 0.0, 0.0)
    direction: tuple = (0.0, 0.0, 1.0)
    up: tuple = (0.0, 1.0, 0.0)
    fovy: float = math.radians(60.0)
    aspect: float = 1.0
    height: float = 1.0
    region: tuple = (0.0, 0.0, 1.0, 1.0)
    aperture: float = 0.0
    focus: float = 1.0


@dataclass
class RendererSpec:
    subtype: str = "default"
    background: tuple = (0.0, 0.0, 0.0, 1.0)
    ambient_color: tuple = (1.0, 1.0, 1.0)
    ambient_radiance: float | None = None  # None: the subtype's default
    ao_distance: float = 1e20
    cull: bool = False
    volume_sampling_rate: float = 0.125
    pixel_samples: int = 1
    ambient_samples: int = 1
    max_depth: int = 5
    max_ray_depth: int = 5  # bounce rays of the default renderer ("maxRayDepth")
    checkerboard: bool = False
    # "background" as an image: (H, W, 3|4) float32 or (H, W, 4) uint8
    # (sRGB-encoded when background_srgb)
    background_image: np.ndarray | None = None
    background_srgb: bool = False

    def resolved_ambient(self) -> float:
        if self.ambient_radiance is not None:
            return self.ambient_radiance
        return 1.0 if self.subtype in ("ao", "dpt", "diffuse_pathtracer") else 0.0


@dataclass
class SceneSpec:
    surfaces: list
    instances: list
    lights: list = _field(default_factory=list)
    volumes: list = _field(default_factory=list)  # in the zero instance
    camera: CameraSpec = _field(default_factory=CameraSpec)
    renderer: RendererSpec = _field(default_factory=RendererSpec)
    width: int = 64
    height: int = 64
    world_id: int = 0xFFFFFFFF


def background_image_type(img: np.ndarray, srgb: bool = False) -> int:
    """Element type code of a background image (RendererSpec.background_image)."""
    from . import _lib as L

    if img.dtype == np.float32 and img.shape[-1] in (3, 4):
        return L.FLOAT32_VEC3 if img.shape[-1] == 3 else L.FLOAT32_VEC4
    if img.dtype == np.uint8 and img.shape[-1] == 4:
        return L.UFIXED8_RGBA_SRGB if srgb else L.UFIXED8_VEC4
    raise ValueError("background images are (H, W, 3|4) float32 or (H, W, 4) uint8")


def sampler_image_type(sp: SamplerSpec) -> int:
    """Element type code of an image sampler's image (SamplerSpec.image)."""
    from . import _lib as L

    tex, c = sp.texels()
    if sp.image_srgb:
        if tex.dtype != np.uint8 or c != 4:
            raise ValueError("sRGB sampler images are uint8 x 4")
        return L.UFIXED8_RGBA_SRGB
    return attr_type(tex)


def attr_type(a: np.ndarray) -> int:
    """Element type code of an attribute array (see SurfaceSpec.attrs)."""
    from . import _lib as L

    comps = 1 if a.ndim == 1 else a.shape[1]
    if a.dtype == np.float32:
        return {1: L.FLOAT32, 2: L.FLOAT32_VEC2, 3: L.FLOAT32_VEC3, 4: L.FLOAT32_VEC4}[comps]
    if a.dtype == np.uint8:
        return {1: L.UFIXED8, 4: L.UFIXED8_VEC4}[comps]
    if a.dtype == np.uint16 and comps == 1:
        return L.UFIXED16
    raise ValueError(f"attribute arrays of {a.dtype} x {comps} are not supported")


def build_on_device(dev, spec: SceneSpec, channels=("color", "depth", "primitiveId",
                                                      "objectId", "instanceId"),
                    float_color: bool = False):
    """Creates the spec's ANARI objects on an anari.Device; returns
    (frame, world, keep) where keep holds every object handle. The colour
    channel is UFIXED8_RGBA_SRGB, or FLOAT32_VEC4 with `float_color`."""
    from . import _lib as L
    from .anari import DataType

    keep = []

    def arr(*a, **k):
        x = dev.new_array(*a, **k)
        keep.append(x)
        return x

    def arr3(*a, **k):
        x = dev.new_array3d(*a, **k)
        keep.append(x)
        return x

    def sampler(sp: SamplerSpec):
        smp = dev.new_sampler(sp.type)
        nd = sp.image_dims
        if nd:
            tex, _ = sp.texels()
            img = np.ascontiguousarray(sp.image)
            et = sampler_image_type(sp)
            a = (dev.new_array(tex, et) if nd == 1 else
                 dev.new_array2d(img, et) if nd == 2 else dev.new_array3d(img, et))
            keep.append(a)
            smp.set("image", a)
            smp.set("filter", sp.filter)
            if nd == 1:
                smp.set("wrapMode", sp.wrap[0])
            else:
                for k in range(nd):
                    smp.set(f"wrapMode{k + 1}", sp.wrap[k])
        elif sp.type == "primitive":
            a = np.ascontiguousarray(sp.array)
            smp.set("array", arr(a, attr_type(a)))
            smp.set("offset", int(sp.offset), L.UINT32)
        smp.set("inAttribute", sp.attribute)
        for name, mat in (("inTransform", sp.in_transform), ("outTransform", sp.out_transform)):
            if mat is not None:
                smp.set(name, np.asarray(mat, np.float32), L.FLOAT32_MAT4)
        smp.set("inOffset", tuple(map(float, sp.in_offset)), L.FLOAT32_VEC4)
        smp.set("outOffset", tuple(map(float, sp.out_offset)), L.FLOAT32_VEC4)
        smp.commit()
        keep.append(smp)
        return smp

    surfs = []
    for s in spec.surfaces:
        g = dev.new_geometry(s.type)
        g.set("vertex.position", arr(np.ascontiguousarray(s.vertices, np.float32),
                                               L.FLOAT32_VEC3))
        if s.indices is not None:
            itype = {"triangle": L.UINT32_VEC3, "quad": L.UINT32_VEC4,
                     "cylinder": L.UINT32_VEC2, "cone": L.UINT32_VEC2}.get(s.type, L.UINT32)
            g.set("primitive.index", arr(np.ascontiguousarray(s.indices, np.uint32), itype))
        if s.normals is not None:
            g.set("vertex.normal", arr(np.ascontiguousarray(s.normals, np.float32),
                                                 L.FLOAT32_VEC3))
        if s.prim_ids is not None:
            g.set("primitive.id", arr(np.ascontiguousarray(s.prim_ids, np.uint32), L.UINT32))
        if s.type in ("sphere", "cone", "curve", "cylinder"):
            if s.radii is not None:
                name = "primitive.radius" if s.type == "cylinder" else "vertex.radius"
                g.set(name, arr(np.ascontiguousarray(s.radii, np.float32), L.FLOAT32))
            if s.type != "cone":
                g.set("radius", float(s.radius))
        if s.type == "cylinder" and s.caps:
            g.set("caps", "both")
        for key, val in s.attrs.items():
            if "." in key:
                a = np.ascontiguousarray(val)
                g.set(key, arr(a, attr_type(a)))
            else:
                g.set(key, tuple(float(c) for c in val), L.FLOAT32_VEC4)
        if s.cull:
            g.set("cullBackfaces", True)
        g.commit()
        m = dev.new_material(s.material)
        cname = "baseColor" if s.material == "physicallyBased" else "color"
        if isinstance(s.color, SamplerSpec):
            m.set(cname, sampler(s.color))
        elif isinstance(s.color, str):
            m.set(cname, s.color)
        else:
            m.set(cname, tuple(float(c) for c in s.color),
                  L.FLOAT32_VEC4 if len(s.color) == 4 else L.FLOAT32_VEC3)
        if s.material == "physicallyBased":
            for name in ("metallic", "roughness"):
                val = getattr(s, name)
                if isinstance(val, SamplerSpec):
                    m.set(name, sampler(val))
                elif isinstance(val, str):
                    m.set(name, val)
                else:
                    m.set(name, float(val))
            m.set("ior", float(s.ior))
        if isinstance(s.opacity, SamplerSpec):
            m.set("opacity", sampler(s.opacity))
        else:
            m.set("opacity", s.opacity if isinstance(s.opacity, str) else float(s.opacity))
        m.set("alphaMode", s.alpha_mode)
        m.set("alphaCutoff", float(s.cutoff))
        m.commit()
        sf = dev.new_surface()
        sf.set("geometry", g).set("material", m)
        sf.set("id", int(s.id), L.UINT32)
        sf.commit()
        keep += [g, m, sf]
        surfs.append(sf)

    lights = []
    for l in spec.lights:
        lt = dev.new_light(l.type)
        lt.set("color", tuple(map(float, l.color)), L.FLOAT32_VEC3)
        if l.type == "directional":
            lt.set("direction", tuple(map(float, l.direction)), L.FLOAT32_VEC3)
            lt.set("irradiance", float(l.irradiance))
        elif l.type == "hdri":
            img = np.ascontiguousarray(l.radiance, np.float32)
            a2 = dev.new_array2d(img, L.FLOAT32_VEC3)
            keep.append(a2)
            lt.set("radiance", a2)
            lt.set("direction", tuple(map(float, l.hdri_direction)), L.FLOAT32_VEC3)
            lt.set("up", tuple(map(float, l.hdri_up)), L.FLOAT32_VEC3)
            lt.set("scale", float(l.scale))
            lt.set("visible", bool(l.visible))
        else:
            lt.set("position", tuple(map(float, l.position)), L.FLOAT32_VEC3)
            lt.set("intensity", float(l.irradiance))
            if l.type == "spot":
                lt.set("direction", tuple(map(float, l.direction)), L.FLOAT32_VEC3)
                lt.set("openingAngle", float(l.opening_angle))
                lt.set("falloffAngle", float(l.falloff_angle))
        lt.commit()
        lights.append(lt)
        keep.append(lt)

    vols = []
    for v in spec.volumes:
        if v.nvdb is not None:
            f = dev.new_spatial_field("nanovdb")
            f.set("data", arr(np.ascontiguousarray(v.nvdb, np.uint8), L.UINT8))
            f.set("filter", v.filter)
        else:
            f = dev.new_spatial_field("structuredRegular")
            fld = v.field if hasattr(v.field, "data_ptr") else np.ascontiguousarray(v.field,
                                                                                    np.float32)
            f.set("data", arr3(fld, L.FLOAT32))
            f.set("origin", tuple(map(float, v.origin)), L.FLOAT32_VEC3)
            f.set("spacing", tuple(map(float, v.spacing)), L.FLOAT32_VEC3)
            f.set("filter", v.filter)
        f.commit()
        vol = dev.new_volume("transferFunction1D")
        vol.set("value", f)
        if v.color is not None:
            vol.set("color", arr(np.ascontiguousarray(v.color, np.float32), L.FLOAT32_VEC3))
        else:
            vol.set("color", tuple(map(float, v.uniform_color)), L.FLOAT32_VEC3)
        if v.opacity is not None:
            vol.set("opacity", arr(np.ascontiguousarray(v.opacity, np.float32), L.FLOAT32))
        else:
            vol.set("opacity", float(v.uniform_opacity))
        vol.set("valueRange", tuple(map(float, v.value_range)), L.FLOAT32_BOX1)
        vol.set("unitDistance", float(v.unit_distance))
        vol.set("id", int(v.id), L.UINT32)
        vol.commit()
        keep += [f, vol]
        vols.append(vol)

    world = dev.new_world()
    insts = []
    # instances of the same surfaces share one group (one BLAS, as ANARI
    # instancing is meant to be used)
    groups = {}
    for ins in spec.instances:
        members = [surfs[i] for i in ins.surfaces]
        if ins.zero:
            if members:
                world.set("surface", arr(members))
            continue
        key = tuple(ins.surfaces)
        grp = groups.get(key)
        if grp is None:
            grp = dev.new_group()
            if members:
                grp.set("surface", arr(members))
            grp.commit()
            groups[key] = grp
        inst = dev.new_instance("transform")
        inst.set("group", grp)
        inst.set("transform", np.asarray(ins.xfm, np.float32), L.FLOAT32_MAT4)
        inst.set("id", int(ins.id), L.UINT32)
        inst.commit()
        keep += [grp, inst]
        insts.append(inst)
    if insts:
        world.set("instance", arr(insts))
    if lights:
        world.set("light", arr(lights))
    if vols:
        world.set("volume", arr(vols))
    world.set("id", int(spec.world_id), L.UINT32)
    world.commit()

    c = spec.camera
    cam = dev.new_camera(c.type)
    cam.set("position", tuple(map(float, c.position)), L.FLOAT32_VEC3)
    cam.set("direction", tuple(map(float, c.direction)), L.FLOAT32_VEC3)
    cam.set("up", tuple(map(float, c.up)), L.FLOAT32_VEC3)
    cam.set("aspect", float(c.aspect))
    cam.set("imageRegion", tuple(map(float, c.region)), L.FLOAT32_BOX2)
    if c.type == "perspective":
        cam.set("fovy", float(c.fovy))
        if c.aperture > 0:
            cam.set("apertureRadius", float(c.aperture))
            cam.set("focusDistance", float(c.focus))
    else:
        cam.set("height", float(c.height))
    cam.commit()

    r = spec.renderer
    ren = dev.new_renderer(r.subtype)
    if r.background_image is not None:
        img = np.ascontiguousarray(r.background_image)
        bga = dev.new_array2d(img, background_image_type(img, r.background_srgb))
        keep.append(bga)
        ren.set("background", bga)
    else:
        ren.set("background", tuple(map(float, r.background)), L.FLOAT32_VEC4)
    ren.set("ambientColor", tuple(map(float, r.ambient_color)), L.FLOAT32_VEC3)
    if r.ambient_radiance is not None:
        ren.set("ambientRadiance", float(r.ambient_radiance))
    ren.set("ambientOcclusionDistance", float(r.ao_distance))
    ren.set("cullTriangleBackfaces", bool(r.cull))
    ren.set("volumeSamplingRate", float(r.volume_sampling_rate))
    ren.set("pixelSamples", int(r.pixel_samples))
    ren.set("ambientSamples", int(r.ambient_samples))
    ren.set("maxDepth", int(r.max_depth))
    ren.set("maxRayDepth", int(r.max_ray_depth))
    ren.set("checkerboarding", bool(r.checkerboard))
    ren.commit()

    fr = dev.new_frame()
    fr.set("size", (spec.width, spec.height), L.UINT32_VEC2)
    fr.set("channel.color", DataType(L.FLOAT32_VEC4 if float_color else L.UFIXED8_RGBA_SRGB))
    for ch in channels:
        if ch == "depth":
            fr.set("channel.depth", DataType(L.FLOAT32))
        elif ch in ("primitiveId", "objectId", "instanceId"):
            fr.set("channel." + ch, DataType(L.UINT32))
        elif ch in ("albedo", "normal"):
            # the reference enables these for ANARI_FLOAT32 (Frame.cu:116-117)
            fr.set("channel." + ch, DataType(L.FLOAT32))
    fr.set("renderer", ren).set("camera", cam).set("world", world)
    fr.commit()
    keep += [world, cam, ren]
    return fr, world, keep


# ---------------------------------------------------------------------------
# the benchmark scenes as specs
# ---------------------------------------------------------------------------

def soup_spec(n: int = 100_000, seed: int = 0, width: int = 512, height: int = 384,
              renderer: str = "default") -> SceneSpec:
    tris = triangle_soup(n, seed)
    surf = SurfaceSpec("triangle", tris.reshape(-1, 3), id=7, color=(0.8, 0.8, 0.8))
    cam = CameraSpec(position=(0.5, 0.5, -1.5), direction=(0.0, 0.0, 1.0), up=(0.0, 1.0, 0.0),
                     fovy=math.radians(40.0), aspect=width / height)
    # light travelling away from the camera so the faces it sees are lit
    light = LightSpec(direction=(0.3, -0.4, 1.0), irradiance=1.0)
    ren = RendererSpec(subtype=renderer, ambient_samples=0, pixel_samples=1)
    return SceneSpec([surf], [InstanceSpec([0], zero=True)], [light], camera=cam, renderer=ren,
                     width=width, height=height, world_id=3)


def instanced_spec(subdiv: int = 8, n_inst: int = 64, n_spheres: int = 1_000_000, seed: int = 0,
                   width: int = 1920, height: int = 1080, spp: int = 64, ao_samples: int = 16,
                   renderer: str = "ao") -> SceneSpec:
    v, f = displaced_icosphere(subdiv, 0.05, seed)
    mesh = SurfaceSpec("triangle", v, indices=f, id=1, color=(0.7, 0.75, 0.8))
    xf = random_instances(n_inst, seed)
    c, r = random_spheres(n_spheres, seed)
    sph = SurfaceSpec("sphere", c, radii=r, id=2, color=(0.9, 0.6, 0.3))
    insts = [InstanceSpec([0], xfm=xf[i], id=100 + i) for i in range(n_inst)]
    insts.append(InstanceSpec([1], zero=True))
    cam_pos = (0.0, 6.0, -34.0)
    _, d, _ = look_at(cam_pos, (0.0, 0.0, 0.0))
    cam = CameraSpec(position=cam_pos, direction=tuple(d), fovy=math.radians(45.0),
                     aspect=width / height)
    ren = RendererSpec(subtype=renderer, pixel_samples=spp, ambient_samples=ao_samples,
                       background=(0.1, 0.1, 0.1, 1.0))
    return SceneSpec([mesh, sph], insts, [LightSpec(direction=(0.2, -1.0, 0.5))], camera=cam,
                     renderer=ren, width=width, height=height, world_id=0)


def nanovdb_volume_spec(grid: np.ndarray, width: int = 1920, height: int = 1080,
                        renderer: str = "raycast", sampling_rate: float = 1.0,
                        seed: int = 0) -> SceneSpec:
    """Volume-only scene over a NanoVDB grid buffer (nanovdb.build_grid): the
    seeded TF of volume_spec, the orbit camera framed on the grid's world
    bbox."""
    from .nanovdb import grid_info

    lo, hi = (np.asarray(b, np.float64) for b in grid_info(grid)["world_bbox"])
    color, op = tf_knots(seed)
    vol = VolumeSpec(field=None, nvdb=np.asarray(grid, np.uint8), color=color, opacity=op,
                     value_range=(0.0, 1.0), id=9)
    center = (lo + hi) / 2
    R = 1.75 * float((hi - lo).max())
    pos = orbit_position(tuple(center), R, 30.0, 20.0)
    _, d, _ = look_at(pos, tuple(center))
    cam = CameraSpec(position=tuple(pos), direction=tuple(d), fovy=math.radians(40.0),
                     aspect=width / height)
    ren = RendererSpec(subtype=renderer, volume_sampling_rate=sampling_rate,
                       background=(0.0, 0.0, 0.0, 1.0), ambient_samples=0)
    return SceneSpec([], [InstanceSpec([], zero=True)], [], [vol], camera=cam, renderer=ren,
                     width=width, height=height)


def volume_spec(n: int = 512, n_blobs: int = 64, seed: int = 0, width: int = 1920,
                height: int = 1080, field: np.ndarray | None = None, renderer: str = "raycast",
                sampling_rate: float = 1.0) -> SceneSpec:
    """Volume-only scene: 0.5-voxel steps (volumeSamplingRate 1, spacing 1)."""
    if field is None:
        field = gaussian_blobs((n, n, n), n_blobs, seed)
    nz, ny, nx = field.shape
    color, op = tf_knots(seed)
    vol = VolumeSpec(field=field, color=color, opacity=op, value_range=(0.0, 1.0), id=9)
    center = ((nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2)
    R = 1.75 * max(nx, ny, nz)
    pos = orbit_position(center, R, 30.0, 20.0)
    _, d, _ = look_at(pos, center)
    cam = CameraSpec(position=tuple(pos), direction=tuple(d), fovy=math.radians(40.0),
                     aspect=width / height)
    ren = RendererSpec(subtype=renderer, volume_sampling_rate=sampling_rate,
                       background=(0.0, 0.0, 0.0, 1.0), ambient_samples=0)
    return SceneSpec([], [InstanceSpec([], zero=True)], [], [vol], camera=cam, renderer=ren,
                     width=width, height=height)
