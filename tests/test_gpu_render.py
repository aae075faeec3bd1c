"""GPU parity: libvrtx (through the C ABI) against the CPU oracle on the same
seeded scenes, for every renderer on the hot path and the edge cases the
reference's code paths have (misses, culling, id indirection, instancing,
accumulation, volumes in front of surfaces)."""
import math

import numpy as np
import pytest

from visrtx_gb300 import scenes as S
from visrtx_gb300 import _lib as L
from tests.parity import compare, inverse_tonemap, render_gpu, render_oracle

pytestmark = pytest.mark.gpu


def soup(renderer="default", n=20_000, w=128, h=96, **kw):
    spec = S.soup_spec(n=n, width=w, height=h, renderer=renderer)
    for k, v in kw.items():
        setattr(spec.renderer, k, v)
    return spec


@pytest.mark.parametrize("renderer", ["default", "raycast", "ao", "dpt"])
def test_soup(device, renderer):
    spec = soup(renderer, ambient_samples=4 if renderer == "ao" else 0,
                pixel_samples=2 if renderer in ("ao", "dpt") else 1)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r)
    assert not device.errors()
    print(renderer, rep)


def test_soup_full_size_ids(device):
    """The 100k-triangle, 512x384 primary-ray workload at full size."""
    spec = S.soup_spec(renderer="raycast")
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r)
    print(rep)


def small_instanced(renderer="ao", spp=2, ao=4):
    spec = S.instanced_spec(subdiv=3, n_inst=8, n_spheres=3000, width=96, height=64, spp=spp,
                            ao_samples=ao, renderer=renderer)
    # spheres large enough to be seen at this resolution
    spec.surfaces[1].radii = spec.surfaces[1].radii * 40.0
    return spec


@pytest.mark.parametrize("renderer", ["ao", "default", "raycast"])
def test_instanced(device, renderer):
    spec = small_instanced(renderer)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, allow_ids=2)
    print(renderer, rep)


def test_instance_transform_array_and_ids(device):
    """An instance with a transform array and an id array: instanceId is the
    per-transform id (Instance.cpp:115-118)."""
    spec = small_instanced("raycast")
    xf = S.random_instances(4, seed=3)
    spec.instances = [S.InstanceSpec([0], xfm=xf[i], id=500 + i) for i in range(4)]
    spec.instances.append(S.InstanceSpec([1], zero=True))
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r, allow_ids=2)
    assert set(np.unique(g["instanceId"])) <= {500, 501, 502, 503, 0xFFFFFFFF, 0}


def test_primitive_id_indices_normals(device):
    """Indexed mesh with vertex normals and a primitive.id array."""
    v, f = S.icosphere(3)
    v = v.astype(np.float32)
    ids = (np.arange(len(f), dtype=np.uint32) * 7 + 11).astype(np.uint32)
    surf = S.SurfaceSpec("triangle", v, indices=f, normals=v.copy(), prim_ids=ids, id=42)
    cam = S.CameraSpec(position=(0.0, 0.0, -3.0), direction=(0.0, 0.0, 1.0), fovy=math.radians(50),
                       aspect=1.0)
    spec = S.SceneSpec([surf], [S.InstanceSpec([0], zero=True)],
                       [S.LightSpec(direction=(0.2, -0.3, 1.0))], camera=cam,
                       renderer=S.RendererSpec("default", ambient_samples=0), width=80, height=80)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r)
    hit = g["depth"] < 1e29
    assert np.all(np.isin(g["primitiveId"][hit], ids))
    assert np.all(g["objectId"][hit] == 42)


@pytest.mark.parametrize("mode", ["renderer", "geometry"])
def test_backface_culling(device, mode):
    """Triangles facing away from the camera are culled when
    cullTriangleBackfaces (renderer) or cullBackfaces (geometry) is set."""
    spec = soup("raycast", n=5000, w=64, h=48)
    if mode == "renderer":
        spec.renderer.cull = True
    else:
        spec.surfaces[0].cull = True
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r)


def test_empty_world_background(device):
    """No geometry: every pixel is background with the reference's miss ids
    (primID 0, objID/instID ~0u, depth 1e30; DirectLight_ptx.cu:389-394)."""
    spec = S.SceneSpec([], [S.InstanceSpec([], zero=True)], [], camera=S.CameraSpec(),
                       renderer=S.RendererSpec("default", background=(0.2, 0.3, 0.4, 1.0)),
                       width=32, height=16)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r)
    assert np.all(g["primitiveId"] == 0)
    assert np.all(g["objectId"] == 0xFFFFFFFF)
    assert np.all(g["depth"] == np.float32(1e30))


def test_spheres_only(device):
    c, rad = S.random_spheres(5000, seed=4)
    surf = S.SurfaceSpec("sphere", c, radii=rad * 30, id=5)
    cam = S.CameraSpec(position=(0.0, 0.0, -30.0), direction=(0.0, 0.0, 1.0),
                       fovy=math.radians(45), aspect=1.5)
    spec = S.SceneSpec([surf], [S.InstanceSpec([0], zero=True)], [S.LightSpec(direction=(0, -1, 1))],
                       camera=cam, renderer=S.RendererSpec("default", ambient_samples=0),
                       width=96, height=64)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r)


def test_accumulation_frames(device):
    """Three frames accumulate (frameID += spp; RNG offset frameID*512)."""
    spec = soup("ao", n=5000, w=48, h=32, ambient_samples=2, pixel_samples=2)
    g = render_gpu(device, spec, frames=3)
    r = render_oracle(spec, frames=3)
    compare(g, r)
    assert g["frame"].get_property("numSamples", L.INT32) == 4


@pytest.mark.parametrize("renderer", ["default", "ao"])
def test_checkerboard_frames(device, renderer):
    """Checkerboarding: four passes per frame id over every other pixel in
    x and y, with the first pass of a fresh frame splatting its colour to
    the rest of each 2x2 block (createScreenSample.h:38-46,
    gpu_util.h:424-442). Six passes cover ids 0..3 and the next frame."""
    spec = soup(renderer, n=5000, w=47, h=33, ambient_samples=2 if renderer == "ao" else 0)
    spec.renderer.checkerboard = True
    for frames in (1, 6):
        g = render_gpu(device, spec, frames=frames)
        r = render_oracle(spec, frames=frames)
        compare(g, r)
        if frames == 1:
            # the splat filled the pixels this pass did not render
            c = g["color"].reshape(33, 47)
            assert np.array_equal(c[0::2, 1::2], c[0::2, 0:46:2])


@pytest.mark.parametrize("renderer", ["default", "raycast", "ao", "dpt"])
def test_albedo_normal_channels(device, renderer):
    """channel.albedo / channel.normal: per-sample accumulations of
    accumResults' albedo (the sample colour; dpt: the background) and normal
    (directLight Ns, raycast/ao Ng, -dir in front of a volume, dir on a
    miss), mapped as accumulation / (frameID + 1) (Frame.cu:518-557)."""
    spec = soup(renderer, n=5000, w=48, h=32, ambient_samples=2 if renderer == "ao" else 0,
                pixel_samples=1 if renderer == "raycast" else 2)
    frames = 1 if renderer == "raycast" else 2
    g = render_gpu(device, spec, frames=frames, channels=True)
    r = render_oracle(spec, frames=frames, channels=True)
    compare(g, r)
    same = np.ones(g["primitiveId"].shape, bool)
    for ch in ("primitiveId", "objectId", "instanceId"):
        same &= g[ch] == r[ch]
    for ch in ("albedo", "normal"):
        assert g[ch].shape == (32, 48, 3), ch
        np.testing.assert_allclose(g[ch][same], r[ch][same], rtol=1e-4, atol=1e-5, err_msg=ch)
    assert np.abs(g["normal"]).max() > 0.1


def geometry_zoo(kind, seed=3):
    """A few hundred primitives of one of the geometry subtypes beside
    triangles and spheres, in a unit-ish cluster in front of the camera."""
    rng = np.random.default_rng(seed)
    n = 300
    if kind == "quad":
        p0 = rng.uniform(-1, 1, (n, 3))
        e1 = rng.normal(0, 0.08, (n, 3))
        e2 = rng.normal(0, 0.08, (n, 3))
        v = np.stack([p0, p0 + e1, p0 + e1 + e2, p0 + e2], 1).reshape(-1, 3).astype(np.float32)
        half = n // 2
        surfs = [S.SurfaceSpec("quad", v[:4 * half], id=31),
                 # indexed, with the quads' corners listed in another order
                 S.SurfaceSpec("quad", v[4 * half:], id=32,
                               indices=(np.arange(4 * (n - half)).reshape(-1, 4)[:, [1, 2, 3, 0]]
                                        ).astype(np.uint32))]
    elif kind in ("cylinder", "cone"):
        a = rng.uniform(-1, 1, (n, 3))
        b = a + rng.normal(0, 0.15, (n, 3))
        v = np.stack([a, b], 1).reshape(-1, 3).astype(np.float32)
        half = n // 2
        if kind == "cylinder":
            surfs = [S.SurfaceSpec("cylinder", v[:2 * half], id=41, radius=0.03, caps=True),
                     S.SurfaceSpec("cylinder", v[2 * half:], id=42,
                                   radii=rng.uniform(0.01, 0.05, n - half).astype(np.float32),
                                   caps=False)]
        else:
            r = rng.uniform(0.005, 0.06, 2 * n).astype(np.float32)
            idx = np.arange(2 * (n - half)).reshape(-1, 2)[:, ::-1].astype(np.uint32)
            surfs = [S.SurfaceSpec("cone", v[:2 * half], id=51, radii=r[:2 * half]),
                     S.SurfaceSpec("cone", v[2 * half:], id=52, radii=r[2 * half:], indices=idx)]
    else:  # curve: random-walk strands
        strands, per = 20, 16
        pts = []
        for k in range(strands):
            p = rng.uniform(-1, 1, 3)
            for i in range(per):
                pts.append(p.copy())
                p = p + rng.normal(0, 0.08, 3)
        v = np.asarray(pts, np.float32)
        rad = rng.uniform(0.01, 0.04, len(v)).astype(np.float32)
        # segments within each strand, by their first vertex
        idx = np.array([k * per + i for k in range(strands) for i in range(per - 1)], np.uint32)
        surfs = [S.SurfaceSpec("curve", v, id=61, radii=rad, indices=idx),
                 # no index: segments 0 .. n/2 - 1 from vertex i to i + 1
                 S.SurfaceSpec("curve", v[:64] + np.float32(0.3), id=62, radius=0.02)]
    cam = S.CameraSpec(position=(0.2, 0.3, -4.0), direction=(0.0, -0.05, 1.0),
                       fovy=math.radians(40), aspect=1.5)
    return S.SceneSpec(surfs, [S.InstanceSpec(list(range(len(surfs))), zero=True)],
                       [S.LightSpec(direction=(0.3, -1.0, 0.6))], camera=cam,
                       renderer=S.RendererSpec("raycast"), width=120, height=80)


@pytest.mark.parametrize("kind", ["quad", "cylinder", "cone", "curve"])
@pytest.mark.parametrize("renderer", ["raycast", "default", "ao"])
def test_geometry_subtypes(device, kind, renderer):
    """Quads (two triangles each, Quad.cpp:115-141), cylinders and cones
    (the reference's intersectors, Intersectors_ptx.cu:100-246) and round
    linear curves (this library's swept-sphere test) against the oracle:
    ids, depth, colour and the populated normals through shading."""
    spec = geometry_zoo(kind)
    spec.renderer = S.RendererSpec(renderer, ambient_samples=2 if renderer == "ao" else 0,
                                   pixel_samples=1)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    if kind == "cone":
        # The reference's cone test solves a quadratic whose coefficients
        # are products of squared dot products (k2, k1, k0 ~ |ba|^4): the
        # cancellation turns a one-ulp difference in the primary ray's
        # direction (GPU and oracle round the camera arithmetic
        # differently) into up to ~1e-4 relative in t and in the normal.
        # Both sides evaluate the test itself without contraction, so ids
        # still agree.
        rep = compare(g, r, allow_ids=3, depth_rel=3e-4, color_tol=8)
    else:
        rep = compare(g, r, allow_ids=3)
    hit = g["depth"] < 1e29
    assert hit.mean() > 0.05, "the primitives cover part of the frame"
    print(kind, renderer, rep, hit.mean())


ATTRIBUTE_CASES = {
    # subtype, material colour source, attribute key, attribute maker
    "triangle-vertex-color-f4": ("triangle", "color", "vertex.color",
                                 lambda rng, n: rng.random((n, 4)).astype(np.float32)),
    "triangle-prim-attr0-u8": ("triangle", "attribute0", "primitive.attribute0",
                               lambda rng, n: rng.integers(0, 256, (n, 4)).astype(np.uint8)),
    "triangle-uniform-attr2": ("triangle", "attribute2", "attribute2", None),
    "triangle-world-normal": ("triangle", "worldNormal", None, None),
    "quad-vertex-attr1-f3": ("quad", "attribute1", "vertex.attribute1",
                             lambda rng, n: rng.random((n, 3)).astype(np.float32)),
    "sphere-vertex-color-u8": ("sphere", "color", "vertex.color",
                               lambda rng, n: rng.integers(0, 256, (n, 4)).astype(np.uint8)),
    "cylinder-vertex-color-f2": ("cylinder", "color", "vertex.color",
                                 lambda rng, n: rng.random((n, 2)).astype(np.float32)),
    "cone-prim-attr3-f1": ("cone", "attribute3", "primitive.attribute3",
                           lambda rng, n: rng.random(n).astype(np.float32)),
    "curve-vertex-color-f4": ("curve", "color", "vertex.color",
                              lambda rng, n: rng.random((n, 4)).astype(np.float32)),
}


@pytest.mark.parametrize("case", sorted(ATTRIBUTE_CASES))
def test_material_attributes(device, case):
    """Matte colour from geometry attributes (readAttributeValue: per-vertex
    values interpolated per subtype with the hit's barycentrics / curve and
    cylinder parameter, per-primitive values, uniform values) and from hit
    quantities, against the oracle."""
    kind, src, key, make = ATTRIBUTE_CASES[case]
    rng = np.random.default_rng(11)
    if kind == "triangle":
        spec = soup("raycast", n=3000, w=96, h=72)
        surf = spec.surfaces[0]
    elif kind == "sphere":
        c, rad = S.random_spheres(3000, seed=4)
        surf = S.SurfaceSpec("sphere", c * 0.1, radii=rad * 5, id=5)
        cam = S.CameraSpec(position=(0.0, 0.0, -3.0), direction=(0.0, 0.0, 1.0),
                           fovy=math.radians(45), aspect=1.5)
        spec = S.SceneSpec([surf], [S.InstanceSpec([0], zero=True)], [], camera=cam,
                           renderer=S.RendererSpec("raycast"), width=96, height=64)
    else:
        spec = geometry_zoo(kind)
        spec.surfaces = spec.surfaces[:1]
        spec.instances = [S.InstanceSpec([0], zero=True)]
        surf = spec.surfaces[0]
    surf.color = src
    if key is not None and "." in key:
        n = (surf.num_prims // (2 if kind == "quad" else 1)) if key.startswith("primitive.") \
            else len(surf.vertices)
        surf.attrs = {key: make(rng, n)}
    elif key is not None:
        surf.attrs = {key: (0.2, 0.7, 0.4, 1.0)}
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, allow_ids=3, **({"depth_rel": 3e-4, "color_tol": 8} if kind == "cone" else {}))
    from visrtx_gb300 import anari

    hit = g["depth"] < 1e29
    c = anari.rgba8(g["color"])[..., :3][hit]
    assert hit.mean() > 0.02 and c.std() > 1.0, "the attribute varies the colour"
    print(case, rep)


def _rot(deg):
    c, s = math.cos(math.radians(deg)), math.sin(math.radians(deg))
    return np.array([[c, -s, 0, 0], [s, c, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], np.float32)


SAMPLER_CASES = {
    # name: (vertex attribute0 channels, SamplerSpec maker, colour tolerance)
    "image2D-nearest-clamp-f4": (2, lambda rng, np_: S.SamplerSpec(
        "image2D", image=rng.random((16, 16, 4)).astype(np.float32), filter="nearest"), 1),
    "image2D-linear-repeat-u8": (2, lambda rng, np_: S.SamplerSpec(
        "image2D", image=rng.integers(0, 256, (8, 12, 4)).astype(np.uint8),
        wrap=("repeat", "repeat", "clampToEdge"),
        in_transform=np.diag([3.0, 2.5, 1.0, 1.0]).astype(np.float32),
        in_offset=(-0.7, 0.3, 0.0, 0.0)), 1),
    # sRGB bytes (alpha too) linearised and truncated to 8 bits at staging
    "image2D-linear-clamp-srgb": (2, lambda rng, np_: S.SamplerSpec(
        "image2D", image=rng.integers(0, 256, (8, 12, 4)).astype(np.uint8), image_srgb=True,
        in_transform=np.diag([1.3, 1.1, 1.0, 1.0]).astype(np.float32),
        in_offset=(-0.1, -0.05, 0.0, 0.0)), 1),
    # 16-bit values truncated to 8 bits at staging
    "image1D-nearest-repeat-u16": (1, lambda rng, np_: S.SamplerSpec(
        "image1D", image=rng.integers(0, 65536, 40).astype(np.uint16), filter="nearest",
        wrap=("repeat", "clampToEdge", "clampToEdge"),
        in_transform=np.diag([2.2, 1.0, 1.0, 1.0]).astype(np.float32),
        in_offset=(-0.3, 0.0, 0.0, 0.0)), 1),
    "image1D-linear-clamp-f3": (1, lambda rng, np_: S.SamplerSpec(
        "image1D", image=rng.random((32, 3)).astype(np.float32),
        in_transform=np.diag([1.4, 1.0, 1.0, 1.0]).astype(np.float32),
        in_offset=(-0.2, 0.0, 0.0, 0.0)), 1),
    "image3D-nearest-mirror-f1": (3, lambda rng, np_: S.SamplerSpec(
        "image3D", image=rng.random((6, 7, 5)).astype(np.float32), filter="nearest",
        wrap=("mirrorRepeat",) * 3, in_transform=np.diag([2.5, 2.5, 2.5, 1.0]).astype(np.float32),
        out_transform=np.array([[1, 0, 0, 0], [0.5, 0, 0, 0], [0.25, 0, 0, 0], [0, 0, 0, 1]],
                               np.float32)), 1),
    "transform-rotate": (4, lambda rng, np_: S.SamplerSpec(
        "transform", attribute="attribute0", in_transform=_rot(30.0),
        out_transform=np.diag([0.6, 0.6, 0.6, 1.0]).astype(np.float32),
        out_offset=(0.2, 0.2, 0.2, 0.0)), 1),
    "primitive-offset-u8": (0, lambda rng, np_: S.SamplerSpec(
        "primitive", array=rng.integers(0, 256, (np_ + 5, 4)).astype(np.uint8), offset=5), 1),
}


@pytest.mark.parametrize("case", sorted(SAMPLER_CASES))
def test_material_samplers(device, case):
    """Matte colour from a sampler (evaluateSampler): the input attribute
    through inTransform / inOffset, an image1D / 2D / 3D lookup (filter and
    wrap modes as the texture hardware applies them), the primitive array at
    primID + offset, or the transformed value itself, then outTransform /
    outOffset; against the oracle's texture emulation."""
    ch, make, tol = SAMPLER_CASES[case]
    rng = np.random.default_rng(23)
    spec = soup("raycast", n=3000, w=96, h=72)
    surf = spec.surfaces[0]
    if ch:
        a = rng.random((len(surf.vertices), ch)).astype(np.float32)
        surf.attrs = {"vertex.attribute0": a if ch > 1 else a[:, 0].copy()}
    surf.color = make(rng, surf.num_prims)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, allow_ids=6, color_tol=tol)
    from visrtx_gb300 import anari

    hit = g["depth"] < 1e29
    c = anari.rgba8(g["color"])[..., :3][hit]
    assert hit.mean() > 0.02 and c.std() > 1.0, "the sampler varies the colour"
    print(case, rep)


def test_orthographic(device):
    spec = soup("raycast", n=5000, w=64, h=64)
    spec.camera = S.CameraSpec(type="orthographic", position=(0.5, 0.5, -1.0),
                               direction=(0.0, 0.0, 1.0), height=1.2, aspect=1.0)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r)


@pytest.mark.parametrize("renderer", ["default", "raycast"])
def test_depth_of_field(device, renderer):
    """Thin-lens perspective camera (apertureRadius, focusDistance;
    Perspective.cpp:40-72, cameraCreateRay.h:51-56): the lens sample uses the
    third and fourth uniforms of the pixel's first draw. The lens offset goes
    through sinf/cosf, whose last-ulp results may differ from the host's, so
    a few edge pixels may change hands."""
    spec = soup(renderer, n=5000, w=64, h=48)
    spec.camera.aperture = 0.04
    spec.camera.focus = 1.6
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r, allow_ids=4)
    # the aperture blurs: the frame differs from the pinhole frame
    spec.camera.aperture = 0.0
    assert not np.array_equal(render_gpu(device, spec)["primitiveId"], g["primitiveId"])


def test_world_bounds(device):
    spec = soup("raycast", n=1000, w=16, h=16)
    g = render_gpu(device, spec)
    b = g["world"].get_property("bounds", L.FLOAT32_BOX3)
    v = spec.surfaces[0].vertices
    np.testing.assert_allclose(b[0], v.min(0), rtol=0, atol=1e-6)
    np.testing.assert_allclose(b[1], v.max(0), rtol=0, atol=1e-6)


def small_volume(n=48, renderer="raycast", rate=1.0, seed=1, w=64, h=48):
    field = S.gaussian_blobs((n, n, n), n_blobs=6, seed=seed, sigma_scale=n / 512 * 4)
    spec = S.volume_spec(field=field, width=w, height=h, renderer=renderer, sampling_rate=rate)
    spec.volumes[0].opacity = spec.volumes[0].opacity * 4
    return spec


@pytest.mark.parametrize("rate", [1.0, 0.125])
def test_volume_parity(device, rate):
    """Scivis marcher against the oracle's fp32 restatement with emulated
    texture filtering (including both jitters and the double-applied
    opacity)."""
    spec = small_volume(rate=rate)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, color_tol=1)
    print(rep)


def test_volume_uniform_colour_with_opacity_array(device):
    """A transferFunction1D volume with an opacity array and no colour array
    takes its uniform colour for every TF entry (TransferFunction1D.cpp:
    50-54,101-150): GPU against the oracle at the colour bar."""
    spec = small_volume()
    spec.volumes[0].color = None
    spec.volumes[0].uniform_color = (0.9, 0.4, 0.1)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, color_tol=1)
    print(rep)
    c = g["color"]
    assert c.std() > 0  # the volume is visible


@pytest.mark.parametrize("renderer", ["raycast", "default"])
def test_volume_dda_march_matches_plain_march(device, renderer):
    """A volume whose TF is transparent over its low values has empty
    macrocells: its march runs the DDA over the skipping grid (empty cells
    crossed without fetches). The frames equal those of the plain
    fixed-step march ("vrtx.emptySpaceSkipping" false) bit for bit, with the
    same sample count and fewer fetches, and match the oracle."""
    spec = small_volume(n=64, renderer=renderer)
    op = np.array(spec.volumes[0].opacity, np.float32)
    op[: len(op) // 2] = 0.0
    spec.volumes[0].opacity = op
    if renderer == "default":
        spec.renderer.ambient_samples = 0
    frames = []
    for skipping in (True, False):
        fr, w, keep = S.build_on_device(device, spec)
        vols = [o for o in keep if getattr(o, "subtype", "") == "transferFunction1D"]
        assert len(vols) == 1
        vols[0].set("vrtx.emptySpaceSkipping", skipping)
        vols[0].commit()
        fr.render()
        fr.wait()
        frames.append(({ch: fr.map("channel." + ch)
                        for ch in ("color", "depth", "primitiveId", "objectId", "instanceId")},
                       fr.stats()))
    for ch in frames[0][0]:
        assert np.array_equal(frames[0][0][ch], frames[1][0][ch]), ch
    (_, st_dda), (_, st_plain) = frames
    assert st_dda["volume_samples"] == st_plain["volume_samples"]
    assert st_dda["volume_fetches"] < 0.9 * st_plain["volume_fetches"], (st_dda, st_plain)
    compare(dict(frames[0][0]), render_oracle(spec), color_tol=1)


def test_volume_fp64_rms(device):
    """Volume colour against the clean FP64 marcher (exact trilinear, FP64
    compositing): RMS <= 1e-3 over the FLOAT32_VEC4 colour channel, so no
    output quantisation enters the figure."""
    spec = small_volume()
    spec.renderer.background = (0.0, 0.0, 0.0, 1.0)
    g = render_gpu(device, spec, float_color=True)
    r = render_oracle(spec, volume_mode=1)
    cr = inverse_tonemap(r["accum"])
    cg = g["color"].astype(np.float64)
    rms = float(np.sqrt(np.mean((cg[..., :3] - cr[..., :3]) ** 2)))
    print("rms vs fp64", rms, "max", float(np.abs(cg[..., :3] - cr[..., :3]).max()))
    assert cr[..., :3].std() > 0.02  # the volume is visible
    assert rms <= 1e-3


def dpt_volume_scene(with_surface=False, spp=8):
    n = 40
    field = S.gaussian_blobs((n, n, n), n_blobs=6, seed=4, sigma_scale=n / 512 * 4)
    # the reference's delta-tracking grid reads the field near its first
    # voxels only (UniformGrid.cu); a constant corner keeps those taps exact
    # under the oracle's texture-filter emulation
    field[:4, :4, :4] = 0.35
    spec = S.volume_spec(field=field, width=64, height=48, renderer="dpt", sampling_rate=1.0)
    spec.renderer.pixel_samples = spp
    spec.renderer.background = (0.05, 0.05, 0.1, 1.0)
    if with_surface:
        tris = S.triangle_soup(1500, seed=5) * 40.0 - 2.0
        spec.surfaces = [S.SurfaceSpec("triangle", tris.reshape(-1, 3), id=21)]
        spec.instances = [S.InstanceSpec([0], zero=True)]
    return spec


@pytest.mark.parametrize("with_surface", [False, True])
def test_dpt_volume_parity(device, with_surface):
    """dpt with a volume: delta tracking over the reference's majorant grid
    (DDA cells across the field bounds, Woodcock steps scaled by the step
    size), scattering on the unit sphere, against the oracle. A path whose
    random decisions all agree gives the same pixel; logf/cosf/sinf and the
    3D filter emulation can differ by an ulp, which moves a later decision
    now and then, so most (not all) pixels must match and the image means
    must agree."""
    spec = dpt_volume_scene(with_surface)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    from visrtx_gb300 import anari

    cg = anari.rgba8(g["color"]).astype(np.int32)
    cr = anari.rgba8(r["color"]).astype(np.int32)
    same = np.all(np.abs(cg - cr) <= 1, axis=-1)
    print("dpt volume: identical pixel fraction", same.mean(),
          "mean", cg[..., :3].mean(), cr[..., :3].mean())
    assert same.mean() >= 0.999
    assert abs(cg[..., :3].mean() - cr[..., :3].mean()) <= 0.02 * max(cr[..., :3].mean(), 1.0)
    assert cr[..., :3].std() > 5.0  # the medium is visible
    # dpt writes the primary tmax as depth and ~0u ids (the raygen's
    # first-hit block never runs)
    for ch in ("depth", "primitiveId", "objectId", "instanceId"):
        assert np.array_equal(g[ch], r[ch]), ch


NVDB_TYPES = ("float", "fp4", "fp8", "fp16", "fpn")


def nvdb_volume(gtype, n=40, renderer="raycast", sparse=True, seed=1, origin=(-9, 4, 130),
                voxel=0.5, translation=(3.0, -2.0, -70.0), w=64, h=48):
    """A NanoVDB grid of the Gaussian-blob field (voxels under 0.05 left
    unset when sparse), placed off the origin, crossing internal-node
    boundaries (x < 0, z around 128)."""
    from visrtx_gb300 import nanovdb as NV

    field = S.gaussian_blobs((n, n, n), n_blobs=6, seed=seed, sigma_scale=n / 512 * 4)
    act = field > 0.05 if sparse else np.ones(field.shape, bool)
    grid = NV.build_grid(field, act, origin, voxel, translation, 0.0, gtype)
    spec = S.nanovdb_volume_spec(grid, width=w, height=h, renderer=renderer)
    spec.volumes[0].opacity = spec.volumes[0].opacity * 4
    return spec


@pytest.mark.parametrize("renderer", ["raycast", "default"])
@pytest.mark.parametrize("gtype", NVDB_TYPES)
def test_nanovdb_volume_parity(device, gtype, renderer):
    """Scivis over a "nanovdb" spatial field (NvdbRegularField.cpp; the tree
    walk and first-order sampler of gpu/sampleSpatialField.h:80-109) for
    every leaf codec the reference's marcher dispatches, against the
    oracle's restatement of the NanoVDB reader."""
    spec = nvdb_volume(gtype, renderer=renderer)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, color_tol=1)
    from visrtx_gb300 import anari

    c = anari.rgba8(g["color"])[..., :3]
    assert c.std() > 5.0, "the volume is visible"
    assert not device.errors()
    print(gtype, renderer, rep)


@pytest.mark.parametrize("gtype", NVDB_TYPES)
def test_nanovdb_golden_grids(device, gtype):
    """Grids made by NanoVDB's own builder (tests/golden/nvdb_golden.npz),
    rendered through the device, against the oracle (which reproduces
    NanoVDB's sampler bit for bit on these grids)."""
    import os

    g0 = np.load(os.path.join(os.path.dirname(__file__), "golden", "nvdb_golden.npz"))
    spec = S.nanovdb_volume_spec(g0[f"grid_{gtype}"], width=64, height=48)
    spec.volumes[0].opacity = spec.volumes[0].opacity * 4
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, color_tol=1)
    from visrtx_gb300 import anari

    assert anari.rgba8(g["color"])[..., :3].std() > 5.0
    print(gtype, rep)


@pytest.mark.parametrize("gtype", ["float", "fp4", "fpn"])
def test_nanovdb_brick_cache_matches_walk(device, gtype):
    """The brick cache (every leaf's values plus a one-voxel apron, filled by
    the tree walk) gives the same frames as walking the tree per tap, bit
    for bit ("vrtx.brickCache" false on the field)."""
    spec = nvdb_volume(gtype, renderer="default")
    a = render_gpu(device, spec)
    frame, world, keep = S.build_on_device(device, spec)
    fields = [o for o in keep if getattr(o, "subtype", "") == "nanovdb"]
    assert len(fields) == 1
    fields[0].set("vrtx.brickCache", False)
    fields[0].commit()
    frame.render()
    frame.wait()
    for ch in ("color", "depth", "primitiveId", "objectId", "instanceId"):
        assert np.array_equal(a[ch], frame.map("channel." + ch)), ch


def test_nanovdb_fp64_rms(device):
    """NanoVDB volume colour against the clean FP64 marcher: RMS <= 1e-3."""
    spec = nvdb_volume("float", sparse=False)
    g = render_gpu(device, spec, float_color=True)
    r = render_oracle(spec, volume_mode=1)
    cr = inverse_tonemap(r["accum"])
    cg = g["color"].astype(np.float64)
    rms = float(np.sqrt(np.mean((cg[..., :3] - cr[..., :3]) ** 2)))
    print("nanovdb rms vs fp64", rms)
    assert cr[..., :3].std() > 0.02
    assert rms <= 1e-3


def test_nanovdb_dpt(device):
    """dpt over a NanoVDB field: the reference's delta-tracking grid spans
    the grid's index bbox and samples it through the NanoVDB sampler at the
    (cell id +- 0.5) / cellDims positions; the grid here maps [0, 1]^3 onto
    its voxels so those taps land on data."""
    n = 40
    spec = nvdb_volume("fp16", n=n, renderer="dpt", sparse=False, origin=(0, 0, 0),
                       voxel=1.0 / n, translation=(0.0, 0.0, 0.0))
    spec.renderer.pixel_samples = 8
    spec.renderer.background = (0.05, 0.05, 0.1, 1.0)
    from oracle import oracle as O

    maj = O.dpt_majorants(spec.volumes[0])
    assert maj.max() > 0.0, "the majorant grid sees the medium"
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    from visrtx_gb300 import anari

    cg = anari.rgba8(g["color"]).astype(np.int32)
    cr = anari.rgba8(r["color"]).astype(np.int32)
    same = np.all(np.abs(cg - cr) <= 1, axis=-1)
    print("nanovdb dpt: identical pixel fraction", same.mean())
    assert same.mean() >= 0.999
    assert abs(cg[..., :3].mean() - cr[..., :3].mean()) <= 0.02 * max(cr[..., :3].mean(), 1.0)
    assert cr[..., :3].std() > 5.0


def test_nanovdb_rejects_bad_grids(device):
    """Buffers that are not a usable NanoVDB grid (wrong magic, a child
    offset pointing outside the buffer, a codec the marcher does not
    dispatch, the wrong array type) are reported and the volume is skipped;
    nothing reads outside the buffer."""
    import struct

    from visrtx_gb300 import nanovdb as NV

    good = nvdb_volume("float").volumes[0].nvdb
    bad_magic = good.copy()
    bad_magic[:8] = 0
    b = bytearray(good.tobytes())
    root = 672 + struct.unpack_from("<q", b, 672 + 24)[0]
    struct.pack_into("<q", b, root + 64 + 8, len(b) * 4)  # first tile's child far outside
    bad_child = np.frombuffer(bytes(b), np.uint8)
    b2 = bytearray(good.tobytes())
    struct.pack_into("<I", b2, 636, 6)  # Vec3f
    bad_type = np.frombuffer(bytes(b2), np.uint8)
    for buf, why in ((bad_magic, "magic"), (bad_child, "outside"), (bad_type, "grid type")):
        spec = nvdb_volume("float")
        spec.volumes[0].nvdb = buf
        device.messages.clear()
        g = render_gpu(device, spec)
        msgs = [m for _, m in device.messages]
        assert any(why in m for m in msgs), (why, msgs)
        assert np.all(g["depth"] >= 1e29), "the invalid volume is skipped"
    assert NV.grid_info(good)["type"] == 1
    device.messages.clear()


def test_volume_in_front_of_surface(device):
    """directLight with a volume and a surface: ids/depth from whichever is
    first, surface shading overwriting volume colour as the reference does."""
    spec = small_volume(n=32, renderer="default")
    tris = S.triangle_soup(2000, seed=2) * 40.0 - 4.0
    spec.surfaces = [S.SurfaceSpec("triangle", tris.reshape(-1, 3), id=77)]
    spec.instances = [S.InstanceSpec([0], zero=True)]
    spec.lights = [S.LightSpec(direction=(0.0, -1.0, 1.0))]
    spec.renderer.ambient_samples = 0
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    compare(g, r, color_tol=1, allow_ids=3)


def test_ao_wavefront_matches_megakernel(device):
    """The wavefront AO path (per-sample primary / any-hit / resolve
    kernels) and the per-pixel integrator draw the same random numbers in the
    same order: identical frames, bit for bit."""
    spec = small_instanced("ao", spp=3, ao=5)
    g1 = render_gpu(device, spec)
    spec2 = small_instanced("ao", spp=3, ao=5)
    from visrtx_gb300 import scenes as S2

    fr, w, keep = S2.build_on_device(device, spec2)
    fr.set("vrtx.megakernel", True)
    fr.commit()
    fr.render()
    fr.wait()
    for ch in ("color", "depth", "primitiveId", "objectId", "instanceId"):
        a = g1[ch]
        b = fr.map("channel." + ch)
        assert np.array_equal(a, b), ch
    assert g1["frame"].kernel_launches() > fr.kernel_launches()


def _frames_equal_forced_megakernel(device, spec, frames=1, channels=False):
    """Renders spec twice, the second time with "vrtx.megakernel" (the
    per-pixel integrator kernel); returns both frames' channel maps after
    asserting they are equal bit for bit."""
    from visrtx_gb300 import scenes as S2

    chans = ("color", "depth", "primitiveId", "objectId", "instanceId")
    if channels:
        chans += ("albedo", "normal")
    outs = []
    for mega in (False, True):
        fr, w, keep = S2.build_on_device(device, spec, channels=chans)
        if mega:
            fr.set("vrtx.megakernel", True)
            fr.commit()
        for _ in range(frames):
            fr.render()
        fr.wait()
        outs.append(({ch: fr.map("channel." + ch) for ch in chans}, fr.kernel_launches()))
    for ch in chans:
        assert np.array_equal(outs[0][0][ch], outs[1][0][ch]), ch
    return outs


@pytest.mark.parametrize("case", ["soup-1spp", "lights-ao3-spp3", "hdri-hidden-checkerboard"])
def test_default_wavefront_matches_megakernel(device, case):
    """The wavefront "default" renderer (primary kernel queuing AO and
    shadow rays, the any-hit queue kernel, resolve) draws every random
    number where the per-pixel kernel does and sums the lights in the same
    order: identical frames, bit for bit, over directional, point, spot and
    HDRI lights, AO samples, several samples per pixel and checkerboarding."""
    if case == "soup-1spp":
        spec = S.soup_spec(n=20_000, width=128, height=96, renderer="default")
        frames = 1
    else:
        spec = soup("default", n=4000, w=96, h=72)
        spec.lights = [S.LightSpec(direction=(0.3, -0.4, 1.0), irradiance=1.5),
                       S.LightSpec("point", position=(0.5, 1.2, -0.6), irradiance=1.5),
                       S.LightSpec("spot", position=(0.4, 0.6, -1.2), direction=(0.1, -0.1, 1.0),
                                   opening_angle=0.45, falloff_angle=0.1, irradiance=2.0)]
        spec.renderer.ambient_samples = 3
        spec.renderer.ambient_radiance = 0.4
        spec.renderer.pixel_samples = 3
        frames = 2
        if case.startswith("hdri"):
            spec.lights.append(S.LightSpec("hdri", radiance=hdri_image(seed=5), visible=False))
            spec.renderer.checkerboard = True
            spec.renderer.pixel_samples = 1
            frames = 5
    outs = _frames_equal_forced_megakernel(device, spec, frames=frames)
    assert outs[0][1] > outs[1][1]  # the wavefront ran (more launches)
    hit = outs[0][0]["depth"] < 1e29
    assert hit.any()
    assert not device.errors()


@pytest.mark.parametrize("case", ["soup", "instanced", "checkerboard"])
def test_raycast_wavefront_matches_megakernel(device, case):
    """The one-kernel "raycast" (opaque surfaces, no volumes) equals the
    per-pixel kernel bit for bit."""
    if case == "instanced":
        spec = small_instanced("raycast")
    else:
        spec = soup("raycast", n=8000, w=100, h=70)
        spec.renderer.checkerboard = case == "checkerboard"
    outs = _frames_equal_forced_megakernel(device, spec, frames=4 if case == "checkerboard" else 1)
    assert (outs[0][0]["depth"] < 1e29).any()
    assert not device.errors()


# --- lights and the physically based material -------------------------------

def hdri_image(w=32, h=16, seed=3):
    """A seeded environment: a sky gradient plus two bright lobes."""
    rng = np.random.default_rng(seed)
    v, u = np.meshgrid((np.arange(h) + 0.5) / h, (np.arange(w) + 0.5) / w, indexing="ij")
    img = np.stack([0.2 + 0.3 * (1 - v), 0.3 + 0.2 * (1 - v), 0.5 + 0.4 * (1 - v)], -1)
    for _ in range(2):
        cu, cv = rng.uniform(0.1, 0.9, 2)
        lobe = np.exp(-(((u - cu) * 8) ** 2 + ((v - cv) * 8) ** 2))
        img += lobe[..., None] * rng.uniform(2.0, 6.0, 3)
    return img.astype(np.float32)


LIGHT_SETS = {
    "directional": lambda: [S.LightSpec(direction=(0.3, -0.4, 1.0), irradiance=1.5)],
    "point": lambda: [S.LightSpec("point", position=(0.5, 1.2, -0.6), irradiance=1.5)],
    "spot": lambda: [S.LightSpec("spot", position=(0.4, 0.6, -1.2), direction=(0.1, -0.1, 1.0),
                                 opening_angle=0.45, falloff_angle=0.1, irradiance=2.0)],
    "hdri": lambda: [S.LightSpec("hdri", radiance=hdri_image(), hdri_direction=(1.0, 0.2, 0.0),
                                 hdri_up=(0.0, 1.0, 0.0), scale=0.8)],
    "hdri-hidden+point": lambda: [
        S.LightSpec("hdri", radiance=hdri_image(seed=5), visible=False),
        S.LightSpec("point", position=(0.5, 0.5, -1.0), irradiance=1.0)],
}


def lit_scene(material, lights, renderer="default", n=2500, w=96, h=72):
    spec = soup(renderer, n=n, w=w, h=h)
    surf = spec.surfaces[0]
    surf.material = material
    surf.color = (0.75, 0.6, 0.45)
    if material == "physicallyBased":
        surf.metallic = 0.6
        surf.roughness = 0.55
        surf.ior = 1.45
    spec.lights = LIGHT_SETS[lights]()
    spec.renderer.background = (0.15, 0.2, 0.3, 1.0)
    spec.renderer.max_ray_depth = 3
    return spec


@pytest.mark.parametrize("lights", sorted(LIGHT_SETS))
@pytest.mark.parametrize("material", ["matte", "physicallyBased"])
def test_lights_and_materials(device, material, lights):
    """The default renderer with every light type (sampleLight.h:60-173:
    directional, point and spot without distance falloff, the HDRI light's
    CDF sampling) on matte and physically based surfaces
    (PhysicallyBasedShader_ptx.cu: Fresnel-Schlick, GGX, Smith; the cone
    next-ray with up to maxRayDepth bounces shaded by the HDRI or the
    background), and a visible HDRI as the background, against the oracle."""
    spec = lit_scene(material, lights)
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, allow_ids=3, color_tol=1)
    from visrtx_gb300 import anari

    c = anari.rgba8(g["color"])[..., :3]
    hit = g["depth"] < 1e29
    assert c[hit].std() > 2.0, "the lights shade the surfaces"
    assert not device.errors()
    print(material, lights, rep)


@pytest.mark.parametrize("renderer", ["raycast", "ao", "dpt"])
def test_hdri_background(device, renderer):
    """A visible HDRI light is every renderer's background (getBackground,
    gpu_util.h:298-307): the miss pixels show the environment."""
    spec = lit_scene("matte", "hdri", renderer=renderer)
    spec.renderer.ambient_samples = 2 if renderer == "ao" else 0
    spec.renderer.pixel_samples = 2 if renderer == "dpt" else 1
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    from visrtx_gb300 import anari

    if renderer == "dpt":
        cg = anari.rgba8(g["color"]).astype(np.int32)
        cr = anari.rgba8(r["color"]).astype(np.int32)
        same = np.all(np.abs(cg - cr) <= 1, axis=-1)
        assert same.mean() >= 0.999, same.mean()
    else:
        compare(g, r, allow_ids=3, color_tol=1)
    miss = g["depth"] >= 1e29
    bg = anari.rgba8(g["color"])[..., :3][miss].astype(np.float64)
    assert miss.any() and bg.std() > 2.0, "the environment varies across the background"


@pytest.mark.parametrize("case", ["float3-raycast", "srgb8-default-pbr", "float4-ao"])
def test_background_image(device, case):
    """The renderer's "background" given as an image (Renderer.cpp:152-175):
    RGBA8-staged (utility/CudaImageTexture.cpp), read with linear filtering
    at each sample's screen position; the default renderer's bounce rays
    read it at the pixel position (DirectLight_ptx.cu:196-216)."""
    fmt, renderer = case.split("-")[:2]
    rng = np.random.default_rng(9)
    yy, xx = np.meshgrid(np.linspace(0, 1, 12), np.linspace(0, 1, 20), indexing="ij")
    base = np.stack([xx, yy, 0.5 * (xx + yy)], -1)
    if fmt == "float3":
        img = (base * 0.9).astype(np.float32)
    elif fmt == "float4":
        img = np.concatenate([base, np.ones_like(xx)[..., None]], -1).astype(np.float32)
    else:
        img = np.concatenate([base * 255, rng.integers(200, 256, xx.shape)[..., None]],
                             -1).astype(np.uint8)
    spec = lit_scene("physicallyBased" if case.endswith("pbr") else "matte", "directional",
                     renderer=renderer)
    spec.renderer.background_image = img
    spec.renderer.background_srgb = fmt == "srgb8"
    spec.renderer.ambient_samples = 2 if renderer == "ao" else 0
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, allow_ids=3, color_tol=1)
    from visrtx_gb300 import anari

    miss = g["depth"] >= 1e29
    bg = anari.rgba8(g["color"])[..., :3][miss].astype(np.float64)
    assert miss.any() and bg.std() > 5.0, "the image varies across the background"
    print(case, rep)


@pytest.mark.parametrize("renderer", ["default", "raycast"])
def test_pbr_parameters_from_attributes_and_samplers(device, renderer):
    """physicallyBased parameters from every source: baseColor from a vertex
    colour, metallic from a per-primitive attribute, roughness through a
    transform sampler of attribute1 (getMaterialParameter,
    evalMaterialParameters.h:336-374)."""
    rng = np.random.default_rng(17)
    spec = lit_scene("physicallyBased", "point", renderer=renderer)
    surf = spec.surfaces[0]
    nv = len(surf.vertices)
    surf.attrs = {
        "vertex.color": rng.random((nv, 4)).astype(np.float32),
        "primitive.attribute0": rng.random(surf.num_prims).astype(np.float32),
        "vertex.attribute1": rng.random((nv, 2)).astype(np.float32),
    }
    surf.color = "color"
    surf.metallic = "attribute0"
    surf.roughness = S.SamplerSpec("transform", attribute="attribute1",
                                   in_transform=np.diag([0.5, 1.0, 1.0, 1.0]).astype(np.float32),
                                   in_offset=(0.3, 0.0, 0.0, 0.0))
    g = render_gpu(device, spec)
    r = render_oracle(spec)
    rep = compare(g, r, allow_ids=3, color_tol=1)
    from visrtx_gb300 import anari

    hit = g["depth"] < 1e29
    assert anari.rgba8(g["color"])[..., :3][hit].std() > 5.0
    print(renderer, rep)


def test_objects_from_many_threads(device):
    """Objects created, set and committed from eight host threads at once
    (the reference's TestMultiThreadedObjectCreation): every handle is valid
    and the frame built from them renders as a single-threaded build does."""
    import threading

    from visrtx_gb300 import anari

    spec = soup("raycast", n=2000, w=48, h=32)
    base = render_gpu(device, spec)
    made, errors = [], []

    def work(k):
        try:
            for i in range(25):
                g = device.new_geometry("sphere")
                a = device.new_array(np.random.default_rng(k * 100 + i).random((8, 3))
                                     .astype(np.float32), L.FLOAT32_VEC3)
                g.set("vertex.position", a)
                g.commit()
                m = device.new_material("matte")
                m.commit()
                sf = device.new_surface()
                sf.set("geometry", g).set("material", m)
                sf.commit()
                made.append((g, a, m, sf))
        except Exception as e:  # noqa: BLE001
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    assert len(made) == 200 and all(o.handle.value for quad in made for o in quad)
    again = render_gpu(device, spec)
    for ch in ("color", "depth", "primitiveId"):
        assert np.array_equal(base[ch], again[ch]), ch
    for quad in made:
        for o in quad:
            o.release()
    assert not device.errors()
    del anari
