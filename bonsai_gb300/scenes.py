"""Seeded synthetic workloads of the path-tracing hot path.

No public benchmark or dataset is involved: every scene here is generated from a stated seed so
the device path and the CPU oracle receive bit-identical float32 inputs.

* ``cornell()``      - the Cornell box (256x256, 16 spp, max depth 5)
* ``ray_soup()``     - 2M random triangles + 16M random rays (closest-hit / any-hit microbenchmark)
* ``production()``   - 1920x1080 scene: 64 fBm-displaced level-5 icospheres (1.31M triangles),
                       2000 lognormal spheres, ground quad, 4 quad area lights, 64 spp, depth 8

Scene records use numpy structured dtypes whose layout equals the C structs of bonsai_gpu.h.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

MATERIAL_DT = np.dtype([("type", "<u4"), ("kd", "<f4", 3), ("ks", "<f4", 3), ("roughness", "<f4"),
                        ("remap_roughness", "<u4"), ("eta", "<f4", 3), ("k", "<f4", 3),
                        ("ior", "<f4"), ("sigma", "<f4"), ("kd_texture", "<u4"), ("ks_texture", "<u4")])
LIGHT_DT = np.dtype([("intensity", "<f4", 3), ("two_sided", "<u4")])
SPHERE_DT = np.dtype([("center", "<f4", 3), ("radius", "<f4"), ("material_id", "<u4"),
                      ("light_id", "<i4")])
QUADRIC_DT = np.dtype([("kind", "<u4"), ("reverse_orientation", "<u4"), ("object_to_world", "<f4", 12),
                       ("world_to_object", "<f4", 12), ("radius", "<f4"), ("inner_radius", "<f4"),
                       ("z_min", "<f4"), ("z_max", "<f4"), ("height", "<f4"), ("phi_max_deg", "<f4"),
                       ("material_id", "<u4"), ("light_id", "<i4")])
RAY_DT = np.dtype([("org", "<f4", 3), ("tmax", "<f4"), ("dir", "<f4", 3), ("pad", "<f4")])
HIT_DT = np.dtype([("prim", "<i4"), ("t", "<f4")])

MATTE, PLASTIC, CONDUCTOR, DIELECTRIC = 0, 1, 2, 3
CYLINDER, DISK, CONE = 0, 1, 2

# Conductor constants (copper, RGB): one fixed triple used identically on CPU and GPU.
COPPER_ETA = (0.200438, 0.924033, 1.10221)
COPPER_K = (3.91295, 2.45285, 2.14219)


def material(kind: int, kd=(0, 0, 0), ks=(0, 0, 0), roughness=0.0, remap=False,
             eta=COPPER_ETA, k=COPPER_K, ior=1.5, sigma=0.0, kd_texture=0, ks_texture=0) -> np.ndarray:
    """A bg_material record; kd_texture / ks_texture are texture indices + 1 (0 = the constant)."""
    m = np.zeros((), MATERIAL_DT)
    m["type"] = kind
    m["kd"] = kd
    m["ks"] = ks
    m["roughness"] = roughness
    m["remap_roughness"] = int(remap)
    m["eta"] = eta
    m["k"] = k
    m["ior"] = ior
    m["sigma"] = sigma
    m["kd_texture"] = kd_texture
    m["ks_texture"] = ks_texture
    return m


def texture_struct(t: "Texture"):
    """(bg_texture, keep-alive array) for a Texture."""
    from ._abi import bg_texture
    c = bg_texture()
    c.kind, c.wrap, c.mapping = t.kind, t.wrap, t.mapping
    keep = None
    if t.kind == 0:
        keep = np.ascontiguousarray(t.rgb, np.float32)
        c.height, c.width = keep.shape[0], keep.shape[1]
        c.rgb = keep.ctypes.data
    c.uv_scale[:] = t.uv_scale
    c.uv_delta[:] = t.uv_delta
    c.world_to_texture[:] = np.asarray(t.world_to_texture, np.float32).reshape(12)
    c.vs[:] = t.vs
    c.vt[:] = t.vt
    c.ds, c.dt = t.ds, t.dt
    return c, keep


@dataclass
class StratifiedSampler:
    """StratifiedSamplerOptions (src/samplers/stratified.rs:32-37); spp = x * y."""
    x_pixel_samples: int
    y_pixel_samples: int
    sampled_dimensions: int
    jitter_samples: bool = True

    @property
    def spp(self) -> int:
        return self.x_pixel_samples * self.y_pixel_samples


def set_sampler(o, sampler: "StratifiedSampler | None"):
    """Fills a bg_render_opts' sampler fields (None: the independent counter-RNG sampler)."""
    if sampler is None:
        o.sampler = 0
        return
    o.sampler = 1
    o.x_pixel_samples, o.y_pixel_samples = sampler.x_pixel_samples, sampler.y_pixel_samples
    o.sampled_dimensions, o.jitter_samples = sampler.sampled_dimensions, int(bool(sampler.jitter_samples))


@dataclass
class EnvMap:
    """bg_infinite_light: an environment map (rgb of shape (h, w, 3), power-of-two sizes, row 0 at
    theta = 0) scaled by `intensity`, oriented by a 3x4 light_to_world (src/lights/infinite.rs)."""
    rgb: np.ndarray
    intensity: tuple = (1.0, 1.0, 1.0)
    light_to_world: np.ndarray = field(default_factory=lambda: np.eye(3, 4, dtype=np.float32))


def env_struct(e: EnvMap):
    """(bg_infinite_light, keep-alive array) for an EnvMap."""
    from ._abi import bg_infinite_light
    c = bg_infinite_light()
    keep = np.ascontiguousarray(e.rgb, np.float32)
    c.height, c.width = keep.shape[0], keep.shape[1]
    c.rgb = keep.ctypes.data
    c.intensity[:] = e.intensity
    c.light_to_world[:] = np.asarray(e.light_to_world, np.float32).reshape(12)
    return c, keep


def triangle_runs(sd: "SceneData"):
    """Consecutive triangle ranges [a, b) sharing (has normals, flags): one mesh call each."""
    n = sd.ntri
    has_n = np.zeros(n, bool)
    if sd.tri_normals is not None:
        has_n[:] = True if sd.tri_normal_mask is None else np.asarray(sd.tri_normal_mask, bool)
    fl = np.zeros(n, np.uint32) if sd.tri_flags is None else np.asarray(sd.tri_flags, np.uint32)
    runs, a = [], 0
    for i in range(1, n + 1):
        if i == n or has_n[i] != has_n[a] or fl[i] != fl[a]:
            runs.append((a, i, bool(has_n[a]), int(fl[a])))
            a = i
    return runs


@dataclass
class Texture:
    """bg_texture: an image (rgb of shape (h, w, 3), power-of-two sizes) or a uv texture, with its
    mapping (src/base/texture.rs)."""
    kind: int = 0                     # 0 image, 1 uv
    rgb: np.ndarray | None = None     # (h, w, 3) float32, row 0 at the top
    wrap: int = 0                     # 0 repeat, 1 black, 2 clamp
    mapping: int = 0                  # 0 uv, 1 spherical, 2 cylindrical, 3 planar
    uv_scale: tuple = (1.0, 1.0)
    uv_delta: tuple = (0.0, 0.0)
    world_to_texture: np.ndarray = field(default_factory=lambda: np.eye(3, 4, dtype=np.float32))
    vs: tuple = (1.0, 0.0, 0.0)
    vt: tuple = (0.0, 1.0, 0.0)
    ds: float = 0.0
    dt: float = 0.0


def rotation(axis, deg: float) -> np.ndarray:
    """4x4 rotation about `axis` by `deg` degrees (Transform::rotate, src/base/transform.rs:100-116)."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    t = np.radians(deg)
    c, s_ = np.cos(t), np.sin(t)
    x, y, z = a
    m = np.eye(4)
    m[:3, :3] = [[x * x + (1 - x * x) * c, x * y * (1 - c) - z * s_, x * z * (1 - c) + y * s_],
                 [x * y * (1 - c) + z * s_, y * y + (1 - y * y) * c, y * z * (1 - c) - x * s_],
                 [x * z * (1 - c) - y * s_, y * z * (1 - c) + x * s_, z * z + (1 - z * z) * c]]
    return m


def translation(t) -> np.ndarray:
    m = np.eye(4)
    m[:3, 3] = t
    return m


def quadric(kind: int, object_to_world: np.ndarray, material_id: int, radius: float = 1.0,
            inner_radius: float = 0.0, z_min: float = -1.0, z_max: float = 1.0, height: float = 1.0,
            phi_max_deg: float = 360.0, reverse: bool = False) -> np.ndarray:
    q = np.zeros((), QUADRIC_DT)
    q["kind"] = kind
    q["reverse_orientation"] = int(reverse)
    m = np.asarray(object_to_world, np.float64)
    q["object_to_world"] = m[:3, :4].astype(np.float32).ravel()
    q["world_to_object"] = np.linalg.inv(m)[:3, :4].astype(np.float32).ravel()
    q["radius"], q["inner_radius"], q["z_min"], q["z_max"] = radius, inner_radius, z_min, z_max
    q["height"], q["phi_max_deg"], q["material_id"], q["light_id"] = height, phi_max_deg, material_id, -1
    return q


@dataclass
class Camera:
    position: tuple
    look_at: tuple
    up: tuple
    fov_deg: float
    width: int
    height: int
    near_plane: float = 0.01
    far_plane: float = 1000.0
    lens_radius: float = 0.0        # thin lens (0: pinhole)
    focal_distance: float = 1e6


@dataclass
class SceneData:
    """Flat scene: triangle soup (n, 9) + spheres + materials + emission records."""
    tri: np.ndarray                      # (ntri, 9) float32, world space p0 p1 p2
    tri_mat: np.ndarray                  # (ntri,) uint32
    tri_light: np.ndarray                # (ntri,) int32, emission record or -1
    spheres: np.ndarray                  # (nsph,) SPHERE_DT
    materials: np.ndarray                # (nmat,) MATERIAL_DT
    lights: np.ndarray                   # (nlights,) LIGHT_DT
    camera: Camera | None = None
    quadrics: np.ndarray = field(default_factory=lambda: np.zeros(0, QUADRIC_DT))
    # triangle mesh attributes: (ntri, 9) vertex normals with a (ntri,) mask of the triangles that
    # have them (None = all), (ntri, 6) uvs, (ntri,) BG_TRI_* flags; None = absent
    tri_normals: np.ndarray | None = None
    tri_normal_mask: np.ndarray | None = None
    tri_uvs: np.ndarray | None = None
    tri_flags: np.ndarray | None = None
    textures: list = field(default_factory=list)
    env: EnvMap | None = None            # the infinite area light, last in the light list
    spp: int = 16
    max_depth: int = 5
    rr_threshold: float = 1.0
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def ntri(self) -> int:
        return int(self.tri.shape[0])

    @property
    def nsph(self) -> int:
        return int(self.spheres.shape[0])


def _quad(a, b, c, d, normal):
    """Two triangles (a,b,c), (a,c,d) wound so (p1-p0)x(p2-p0) points along `normal`."""
    a, b, c, d = (np.asarray(v, np.float32) for v in (a, b, c, d))
    n = np.cross(b - a, c - a)
    if np.dot(n, np.asarray(normal, np.float32)) < 0:
        b, d = d, b
    return np.stack([np.concatenate([a, b, c]), np.concatenate([a, c, d])]).astype(np.float32)


def cornell(width: int = 256, height: int = 256, spp: int = 16, max_depth: int = 5) -> SceneData:
    """Cornell box in [-1,1]^3: 5 diffuse walls (10 triangles, inward normals), a 0.5x0.5 ceiling
    light at y=0.999 (2 triangles, emission (17,12,4)), a diffuse and a Trowbridge-Reitz
    conductor sphere (r=0.3), pinhole camera at (0,0,3.5) looking at the origin, fov 40.

    The light is two-sided: the reference's DiffuseAreaLight::sample_point evaluates emission
    toward +wi (src/lights/diffuse.rs:67), so a one-sided light facing the room returns black
    light samples there and the reference image would be dark apart from the light itself.
    """
    grey, red, green = (0.725, 0.725, 0.725), (0.63, 0.065, 0.05), (0.14, 0.45, 0.091)
    mats = [material(MATTE, kd=grey), material(MATTE, kd=red), material(MATTE, kd=green),
            material(CONDUCTOR, roughness=0.1), material(MATTE, kd=(0, 0, 0))]
    tris, tmat = [], []

    def add(q, m):
        tris.append(q)
        tmat.extend([m] * len(q))
    add(_quad((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), (0, 1, 0)), 0)   # floor
    add(_quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), (0, -1, 0)), 0)      # ceiling
    add(_quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (0, 0, 1)), 0)   # back
    add(_quad((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), (1, 0, 0)), 1)   # left (red)
    add(_quad((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1), (-1, 0, 0)), 2)      # right (green)
    nwall = sum(len(t) for t in tris)
    add(_quad((-0.25, 0.999, -0.25), (0.25, 0.999, -0.25), (0.25, 0.999, 0.25), (-0.25, 0.999, 0.25),
              (0, -1, 0)), 4)
    tri = np.concatenate(tris).astype(np.float32)
    tri_light = np.full(len(tri), -1, np.int32)
    tri_light[nwall:] = 0
    sph = np.zeros(2, SPHERE_DT)
    sph[0] = ((-0.4, -0.7, -0.3), 0.3, 0, -1)
    sph[1] = ((0.4, -0.7, 0.3), 0.3, 3, -1)
    lights = np.zeros(1, LIGHT_DT)
    lights[0] = ((17.0, 12.0, 4.0), 1)
    cam = Camera((0.0, 0.0, 3.5), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, width, height)
    return SceneData(tri, np.asarray(tmat, np.uint32), tri_light, sph, np.stack(mats), lights, cam,
                     spp=spp, max_depth=max_depth, rr_threshold=1.0, name="cornell")


def quadric_box(width: int = 64, height: int = 64, spp: int = 8, max_depth: int = 5) -> SceneData:
    """The Cornell box with a cylinder, a disk and a cone (rotated and partial) in place of the
    spheres: exercises the quadric shapes (src/shapes/{cylinder,disk,cone}.rs)."""
    sd = cornell(width, height, spp, max_depth)
    mats = list(sd.materials) + [material(MATTE, kd=(0.3, 0.6, 0.8)), material(PLASTIC, kd=(0.6, 0.3, 0.2),
                                                                              ks=(0.4, 0.4, 0.4), roughness=0.2)]
    m_cyl, m_pl = len(mats) - 2, len(mats) - 1
    q = [quadric(CYLINDER, translation((-0.45, -0.5, -0.2)) @ rotation((1, 0, 0), -90), m_cyl, radius=0.25,
                 z_min=-0.5, z_max=0.3, phi_max_deg=300.0),
         quadric(DISK, translation((0.4, -0.6, 0.2)) @ rotation((1, 0, 0), -70), m_pl, radius=0.3, inner_radius=0.1,
                 height=0.0, phi_max_deg=360.0),
         quadric(CONE, translation((0.1, -1.0, -0.5)) @ rotation((1, 0, 0), -90), 3, radius=0.3, height=0.8,
                 phi_max_deg=330.0)]
    sd.materials = np.stack(mats)
    sd.quadrics = np.stack(q)
    sd.spheres = np.zeros(0, SPHERE_DT)
    sd.name = "quadric_box"
    return sd


def shape_lights(width: int = 64, height: int = 64, spp: int = 8, max_depth: int = 5,
                 triangle_light: bool = True) -> SceneData:
    """The Cornell box lit by DiffuseAreaLights on a sphere (r 0.12, two-sided), a full disk facing
    down from the ceiling, a partial annulus (inner radius, 270 degrees) and a cylinder (one-sided,
    outward), with or without the box's own triangle light."""
    sd = cornell(width, height, spp, max_depth)
    lights = list(sd.lights)
    for inten, two in (((6.0, 5.0, 4.0), 1), ((3.0, 4.0, 6.0), 0), ((5.0, 2.0, 2.0), 0), ((2.0, 5.0, 3.0), 0)):
        l = np.zeros((), LIGHT_DT)
        l["intensity"], l["two_sided"] = inten, two
        lights.append(l)
    mats = list(sd.materials) + [material(MATTE, kd=(0.0, 0.0, 0.0))]
    m_black = len(mats) - 1
    sph = list(sd.spheres) + [np.zeros((), SPHERE_DT)]
    sph[-1]["center"], sph[-1]["radius"], sph[-1]["material_id"], sph[-1]["light_id"] = (0.0, 0.55, -0.2), 0.12, m_black, 1
    q = [quadric(DISK, translation((0.45, 0.985, 0.25)) @ rotation((1, 0, 0), 90), m_black, radius=0.2, height=0.0),
         quadric(DISK, translation((-0.45, 0.985, 0.3)) @ rotation((1, 0, 0), 90), m_black, radius=0.2,
                 inner_radius=0.08, height=0.0, phi_max_deg=270.0),
         quadric(CYLINDER, translation((-0.55, 0.3, -0.4)), m_black, radius=0.06, z_min=-0.2, z_max=0.2)]
    q[0]["light_id"], q[1]["light_id"], q[2]["light_id"] = 2, 3, 4
    tri, tm, tl = sd.tri, sd.tri_mat, sd.tri_light
    if not triangle_light:
        keep = tl < 0
        tri, tm, tl = tri[keep], tm[keep], tl[keep]
    out = SceneData(tri.copy(), tm.copy(), tl.copy(), np.stack(sph), np.stack(mats), np.stack(lights), sd.camera,
                    quadrics=np.stack(q), spp=spp, max_depth=max_depth, rr_threshold=1.0,
                    name="shape_lights" + ("" if triangle_light else "_only"))
    return out


def checker_image(n: int = 64, tiles: int = 8, seed: int = 0) -> np.ndarray:
    """(n, n, 3) float32 test image: a two-colour checkerboard with per-texel noise in blue."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:n, 0:n]
    c = ((x * tiles // n + y * tiles // n) % 2).astype(np.float32)
    img = np.empty((n, n, 3), np.float32)
    img[..., 0] = 0.15 + 0.7 * c
    img[..., 1] = 0.2 + 0.5 * (1.0 - c)
    img[..., 2] = (0.2 + 0.4 * rng.random((n, n))).astype(np.float32)
    return img


def textured_room(width: int = 64, height: int = 64, spp: int = 16, max_depth: int = 5) -> SceneData:
    """The Cornell box with every texture and mesh-attribute path of the reference in use:
    back wall: image texture (64^2, repeat) through UVMapping2D with per-vertex uvs, scaled so the
    MIPMap filters between levels; floor: UVTexture through PlanarMapping2D on an Oren-Nayar matte
    (sigma 25); left wall: plastic whose ks is an image through CylindricalMapping2D (black wrap);
    diffuse sphere: image through SphericalMapping2D (clamp); a smooth-shaded icosphere (vertex
    normals, Oren-Nayar sigma 40); ceiling triangles marked as mirrored by their transform; a
    one-sided ceiling light of two triangles wound upward, one turned toward the room by
    reverse_orientation and one by its vertex normals."""
    sd = cornell(width, height, spp, max_depth)
    nwall = 10
    mats = list(sd.materials)  # 0 grey, 1 red, 2 green, 3 conductor, 4 light (black)
    m_back = len(mats); mats.append(material(MATTE, kd_texture=1))
    m_floor = len(mats); mats.append(material(MATTE, kd=(0.7, 0.7, 0.7), kd_texture=2, sigma=25.0))
    m_sph = len(mats); mats.append(material(MATTE, kd_texture=3))
    m_left = len(mats); mats.append(material(PLASTIC, kd=(0.35, 0.1, 0.08), ks_texture=4, roughness=0.3))
    m_ico = len(mats); mats.append(material(MATTE, kd=(0.6, 0.6, 0.5), sigma=40.0))
    tex = [Texture(kind=0, rgb=checker_image(64, 8, 1), wrap=0, mapping=0, uv_scale=(6.0, 6.0), uv_delta=(0.1, 0.0)),
           Texture(kind=1, mapping=3, vs=(1.5, 0.0, 0.0), vt=(0.0, 0.0, 1.5), ds=0.25, dt=0.5),
           Texture(kind=0, rgb=checker_image(32, 4, 2), wrap=2, mapping=1,
                   world_to_texture=translation((0.4, 0.7, 0.3))[:3].astype(np.float32)),
           Texture(kind=0, rgb=checker_image(16, 2, 3), wrap=1, mapping=2,
                   world_to_texture=(rotation((1, 0, 0), 90) @ translation((1.0, 0.0, 0.0)))[:3].astype(np.float32))]
    tri = sd.tri[:nwall].copy()
    tmat = sd.tri_mat[:nwall].copy()
    tmat[0:2] = m_floor
    tmat[4:6] = m_back
    tmat[6:8] = m_left
    uvs = np.tile(np.array([0, 0, 1, 0, 1, 1], np.float32), (nwall, 1))
    for t in (4, 5):  # back wall: uv = position x, y mapped to [0, 1]
        p = tri[t].reshape(3, 3)
        uvs[t] = np.stack([(p[:, 0] + 1) / 2, (p[:, 1] + 1) / 2], axis=1).reshape(6)
    flags = np.zeros(nwall, np.uint8)
    flags[2:4] = 2  # ceiling: transform swaps handedness
    # smooth icosphere (level 2) with vertex normals
    v, f = icosphere(2)
    c, r = np.array([0.35, -0.55, -0.35]), 0.3
    ico = (c + r * v[f]).reshape(-1, 9).astype(np.float32)
    ico_n = v[f].reshape(-1, 9).astype(np.float32)
    nico = len(ico)
    # one-sided light: two triangles with upward winding
    a, b, cc, d = (-0.25, 0.999, -0.25), (0.25, 0.999, -0.25), (0.25, 0.999, 0.25), (-0.25, 0.999, 0.25)
    lq = _quad(a, b, cc, d, (0, 1, 0))
    ln = np.tile(np.array([0.1, -1.0, 0.05], np.float32), 3)
    all_tri = np.concatenate([tri, ico, lq]).astype(np.float32)
    n = len(all_tri)
    normals = np.zeros((n, 9), np.float32)
    normals[nwall:nwall + nico] = ico_n
    normals[n - 1] = ln
    mask = np.zeros(n, bool)
    mask[nwall:nwall + nico] = True
    mask[n - 1] = True
    all_uv = np.tile(np.array([0, 0, 1, 0, 1, 1], np.float32), (n, 1))
    all_uv[:nwall] = uvs
    all_flags = np.zeros(n, np.uint8)
    all_flags[:nwall] = flags
    all_flags[n - 2] = 1  # reverse_orientation
    tmat_all = np.concatenate([tmat, np.full(nico, m_ico, np.uint32), np.full(2, 4, np.uint32)]).astype(np.uint32)
    tl = np.full(n, -1, np.int32)
    tl[n - 2:] = 0
    lights = sd.lights.copy()
    lights[0]["two_sided"] = 0
    sph = sd.spheres.copy()
    sph[0]["material_id"] = m_sph
    return SceneData(all_tri, tmat_all, tl, sph, np.stack(mats), lights, sd.camera, spp=spp, max_depth=max_depth,
                     rr_threshold=1.0, name="textured_room", tri_normals=normals, tri_normal_mask=mask,
                     tri_uvs=all_uv, tri_flags=all_flags, textures=tex)


def environment_image(w: int = 64, h: int = 32, seed: int = 0, sun=(0.25, 0.3), sun_radius: float = 0.12,
                      sun_radiance: float = 40.0) -> np.ndarray:
    """(h, w, 3) float32 synthetic environment map over (phi, theta) = (2 pi (x + .5) / w,
    pi (y + .5) / h): a blue sky above the horizon (theta < pi / 2), a brown ground below, a small
    bright sun at (theta, phi) = pi * sun[0], 2 pi * sun[1], and seeded per-texel noise."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    theta = np.pi * (y + 0.5) / h
    phi = 2 * np.pi * (x + 0.5) / w
    up = np.cos(theta)[..., None]
    sky = np.array([0.25, 0.45, 0.9], np.float32) * (0.4 + 0.6 * np.clip(up, 0, 1)) + 0.15
    ground = np.array([0.3, 0.24, 0.18], np.float32) * (0.6 + 0.4 * np.clip(-up, 0, 1))
    img = np.where(up > 0, sky, ground)
    ts, ps = np.pi * sun[0], 2 * np.pi * sun[1]
    cosang = np.sin(theta) * np.sin(ts) * np.cos(phi - ps) + np.cos(theta) * np.cos(ts)
    sun_mask = np.arccos(np.clip(cosang, -1, 1)) < sun_radius
    img = img + sun_mask[..., None] * (sun_radiance * np.array([1.0, 0.9, 0.7], np.float32))
    img = img * (0.9 + 0.2 * rng.random((h, w, 1)))
    return img.astype(np.float32)


def env_sphere(width: int = 64, height: int = 64, spp: int = 16, max_depth: int = 5, env_w: int = 64,
               env_h: int = 32, seed: int = 0, extra: bool = False) -> SceneData:
    """The reference's example scene (src/main.rs): a unit sphere at the origin, matte with a
    UVTexture through the default UVMapping2D, lit only by an InfiniteAreaLight of identity
    transform; camera at (5, 0, 0) looking at the origin, up (0, 0, 1), fov 45.  The environment map
    is synthetic (environment_image).  extra = True adds a glass and a plastic sphere and a small
    one-sided emitting quad, so the light list mixes area lights with the infinite light."""
    mats = [material(MATTE, kd_texture=1, sigma=0.0)]
    tex = [Texture(kind=1, mapping=0)]
    spheres = [((0.0, 0.0, 0.0), 1.0, 0)]
    tri = np.zeros((0, 9), np.float32)
    tri_light = np.zeros(0, np.int32)
    lights = np.zeros(0, LIGHT_DT)
    if extra:
        mats.append(material(DIELECTRIC, ior=1.5))
        mats.append(material(PLASTIC, kd=(0.1, 0.3, 0.6), ks=(0.4, 0.4, 0.4), roughness=0.2))
        mats.append(material(MATTE, kd=(0.0, 0.0, 0.0)))
        spheres += [((1.2, 1.6, 0.3), 0.5, 1), ((0.8, -1.5, -0.6), 0.45, 2)]
        tri = _quad((1.5, -0.4, 1.6), (1.5, 0.4, 1.6), (1.5, 0.4, 2.2), (1.5, -0.4, 2.2), (-1, 0, 0))
        tri_light = np.zeros(2, np.int32)
        lights = np.zeros(1, LIGHT_DT)
        lights[0]["intensity"] = (6.0, 5.0, 4.0)
        lights[0]["two_sided"] = 0
    sph = np.zeros(len(spheres), SPHERE_DT)
    for i, (c, r, m) in enumerate(spheres):
        sph[i]["center"], sph[i]["radius"], sph[i]["material_id"], sph[i]["light_id"] = c, r, m, -1
    tri_mat = np.full(len(tri), len(mats) - 1, np.uint32)
    cam = Camera((5.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 45.0, width, height)
    env = EnvMap(environment_image(env_w, env_h, seed))
    return SceneData(tri.astype(np.float32), tri_mat, tri_light, sph, np.stack(mats), lights, cam, spp=spp,
                     max_depth=max_depth, rr_threshold=1.0, name="env_sphere" + ("_extra" if extra else ""),
                     textures=tex, env=env)


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)


def random_triangles(n: int, seed: int = 1) -> np.ndarray:
    """n equilateral triangles: centroids U[0,1]^3, edge U[0.002,0.02], uniform random rotation."""
    rng = np.random.default_rng(seed)
    cen = rng.random((n, 3))
    edge = rng.uniform(0.002, 0.02, n)
    rot = _random_rotations(rng, n)
    ang = np.array([0.0, 2 * np.pi / 3, 4 * np.pi / 3])
    local = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)], -1)  # (3,3) unit circumradius
    circ = edge / np.sqrt(3.0)
    verts = cen[:, None, :] + circ[:, None, None] * np.einsum("nij,vj->nvi", rot, local)
    return verts.reshape(n, 9).astype(np.float32)


def random_rays(n: int, seed: int = 2) -> np.ndarray:
    """n rays: origins uniform on the unit cube surface (face uniform), directions uniform on S^2."""
    rng = np.random.default_rng(seed)
    face = rng.integers(0, 6, n)
    uv = rng.random((n, 2))
    org = np.empty((n, 3))
    axis = face // 2
    side = (face % 2).astype(np.float64)
    for a in range(3):
        m = axis == a
        o = np.empty((m.sum(), 3))
        others = [i for i in range(3) if i != a]
        o[:, a] = side[m]
        o[:, others[0]] = uv[m, 0]
        o[:, others[1]] = uv[m, 1]
        org[m] = o
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    r = np.sqrt(np.maximum(0.0, 1 - z * z))
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], -1)
    rays = np.zeros(n, RAY_DT)
    rays["org"] = org.astype(np.float32)
    rays["dir"] = d.astype(np.float32)
    rays["tmax"] = np.float32(np.inf)
    return rays


def ray_soup(ntri: int = 2_097_152, nrays: int = 16_777_216):
    """Ray/BVH microbenchmark: triangle soup (seed 1) + ray set (seed 2).  All triangles diffuse."""
    tri = random_triangles(ntri, seed=1)
    sd = SceneData(tri, np.zeros(ntri, np.uint32), np.full(ntri, -1, np.int32),
                   np.zeros(0, SPHERE_DT), np.stack([material(MATTE, kd=(0.5, 0.5, 0.5))]),
                   np.zeros(0, LIGHT_DT), name=f"ray_soup_{ntri}")
    return sd, random_rays(nrays, seed=2)


# ---------------------------------------------------------------- icospheres + fBm
def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (vertices (V,3) float64, faces (F,3) int).  Level 5 has 20480 faces."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.asarray(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = f
    for _ in range(level):
        cache: dict = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.asarray(verts), np.asarray(faces, np.int64)


def _value_noise(p: np.ndarray, perm: np.ndarray, vals: np.ndarray) -> np.ndarray:
    """3D value noise in [-1,1]: hashed lattice values, smoothstep trilinear interpolation."""
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    w = pf * pf * (3 - 2 * pf)
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                h = perm[(perm[(perm[(pi[:, 0] + dx) & 255] + pi[:, 1] + dy) & 255] + pi[:, 2] + dz) & 255]
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out = out + wx * wy * wz * vals[h]
    return out


def fbm(p: np.ndarray, seed: int, octaves: int = 5, base_freq: float = 2.0) -> np.ndarray:
    """Fractal Brownian motion of value noise, normalised to [-1,1]."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    vals = rng.uniform(-1, 1, 256)
    total, amp, norm = 0.0, 1.0, 0.0
    for o in range(octaves):
        total = total + amp * _value_noise(p * (base_freq * 2 ** o) + 17.31 * o, perm, vals)
        norm += amp
        amp *= 0.5
    return total / norm


def production(width: int = 1920, height: int = 1080, spp: int = 64, max_depth: int = 8,
               n_ico: int = 64, ico_level: int = 5, n_spheres: int = 2000, seed: int = 3) -> SceneData:
    """1080p production-style scene (defaults are the full size).

    64 level-5 icospheres (20480 triangles each, 1.31M total), radially displaced by seeded fBm
    (amplitude 0.1 r, 5 octaves) on an 8x8 jittered grid; 2000 analytic spheres with lognormal radii
    (mu=-3, sigma=0.5); a ground quad (2 triangles); 4 one-sided quad area lights facing down.
    Materials per object (seed 3): 50% diffuse (albedo U[0.1,0.9]), 30% Trowbridge-Reitz conductor
    (roughness U[0.05,0.5], copper eta/k), 20% dielectric (IOR 1.5).
    """
    rng = np.random.default_rng(seed)
    uv, uf = icosphere(ico_level)
    mats = [material(MATTE, kd=(0.5, 0.5, 0.5)), material(MATTE, kd=(0, 0, 0))]  # ground, light

    def random_material():
        r = rng.random()
        if r < 0.5:
            return material(MATTE, kd=tuple(rng.uniform(0.1, 0.9, 3)))
        if r < 0.8:
            return material(CONDUCTOR, roughness=float(rng.uniform(0.05, 0.5)))
        return material(DIELECTRIC, ior=1.5)

    tris, tmat = [], []
    g = int(np.ceil(np.sqrt(n_ico)))
    cells = np.linspace(-9, 9, g)
    for i in range(n_ico):
        gx, gz = cells[i % g], cells[(i // g) % g]
        r = rng.uniform(0.6, 1.2)
        c = np.array([gx + rng.uniform(-0.6, 0.6), r * 1.1, gz + rng.uniform(-0.6, 0.6)])
        d = 1.0 + 0.1 * fbm(uv * 1.5, seed=seed * 1000 + i)
        v = c + (uv * (r * d)[:, None])
        tris.append(v[uf].reshape(-1, 9))
        mats.append(random_material())
        tmat.append(np.full(len(uf), len(mats) - 1, np.uint32))
    ground = _quad((-12, 0, -12), (12, 0, -12), (12, 0, 12), (-12, 0, 12), (0, 1, 0))
    tris.append(ground)
    tmat.append(np.zeros(2, np.uint32))
    nonlight = sum(len(t) for t in tris)
    for lx in (-4.0, 4.0):
        for lz in (-4.0, 4.0):
            tris.append(_quad((lx - 1, 6, lz - 1), (lx + 1, 6, lz - 1), (lx + 1, 6, lz + 1),
                              (lx - 1, 6, lz + 1), (0, -1, 0)))
            tmat.append(np.ones(2, np.uint32))
    tri = np.concatenate(tris).astype(np.float32)
    tri_mat = np.concatenate(tmat).astype(np.uint32)
    tri_light = np.full(len(tri), -1, np.int32)
    tri_light[nonlight:] = 0
    radii = np.exp(rng.normal(-3.0, 0.5, n_spheres))
    sph = np.zeros(n_spheres, SPHERE_DT)
    sph["center"][:, 0] = rng.uniform(-10, 10, n_spheres)
    sph["center"][:, 2] = rng.uniform(-10, 10, n_spheres)
    sph["center"][:, 1] = radii + rng.uniform(0, 2.5, n_spheres)
    sph["radius"] = radii
    for i in range(n_spheres):
        mats.append(random_material())
        sph["material_id"][i] = len(mats) - 1
    sph["light_id"] = -1
    lights = np.zeros(1, LIGHT_DT)
    lights[0] = ((12.0, 12.0, 12.0), 0)
    cam = Camera((0.0, 8.0, 14.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, width, height)
    return SceneData(tri, tri_mat, tri_light, sph, np.stack(mats), lights, cam, spp=spp,
                     max_depth=max_depth, rr_threshold=1.0, name="production",
                     meta={"n_ico": n_ico, "ico_level": ico_level, "n_spheres": n_spheres})


def slit_room(width: int = 1280, height: int = 720, spp: int = 64, max_depth: int = 10, n_ico: int = 10,
              ico_level: int = 5, n_spheres: int = 200, light_intensity: float = 60.0, seed: int = 4) -> SceneData:
    """Indirect-dominated scene for learned path guiding (defaults are the full size).

    A closed 10 x 4 x 10 room (x, z in [-5, 5], y in [0, 4]), diffuse 0.7, with a 0.2-wide vertical
    slit (z in [-0.1, 0.1], full height) in the x = +5 wall; a closed room with a slit needs 14
    triangles (the slit wall is two quads).  The only light is a one-sided 3 x 3 quad outside the
    slit at x = 6, facing the room.  Inside: `n_ico` fBm-displaced icospheres (level 5: 20480
    triangles each, 204,800 in total) and `n_spheres` spheres with lognormal radii; materials per
    object (seed 4) 50% matte, 25% plastic, 25% Trowbridge-Reitz conductor.
    """
    rng = np.random.default_rng(seed)
    mats = [material(MATTE, kd=(0.7, 0.7, 0.7)), material(MATTE, kd=(0, 0, 0))]  # walls, light

    def random_material():
        r = rng.random()
        if r < 0.5:
            return material(MATTE, kd=tuple(rng.uniform(0.2, 0.9, 3)))
        if r < 0.75:
            return material(PLASTIC, kd=tuple(rng.uniform(0.2, 0.8, 3)), ks=(0.3, 0.3, 0.3),
                            roughness=float(rng.uniform(0.05, 0.4)))
        return material(CONDUCTOR, roughness=float(rng.uniform(0.05, 0.5)))

    X, Y, Z, S = 5.0, 4.0, 5.0, 0.1
    walls = [
        _quad((-X, 0, -Z), (X, 0, -Z), (X, 0, Z), (-X, 0, Z), (0, 1, 0)),        # floor
        _quad((-X, Y, -Z), (X, Y, -Z), (X, Y, Z), (-X, Y, Z), (0, -1, 0)),       # ceiling
        _quad((-X, 0, -Z), (-X, Y, -Z), (-X, Y, Z), (-X, 0, Z), (1, 0, 0)),      # x = -5
        _quad((-X, 0, -Z), (X, 0, -Z), (X, Y, -Z), (-X, Y, -Z), (0, 0, 1)),      # z = -5
        _quad((-X, 0, Z), (X, 0, Z), (X, Y, Z), (-X, Y, Z), (0, 0, -1)),         # z = +5
        _quad((X, 0, -Z), (X, Y, -Z), (X, Y, -S), (X, 0, -S), (-1, 0, 0)),       # x = +5, z < -0.1
        _quad((X, 0, S), (X, Y, S), (X, Y, Z), (X, 0, Z), (-1, 0, 0)),           # x = +5, z > 0.1
    ]
    tris = [np.concatenate(walls)]
    tmat = [np.zeros(14, np.uint32)]
    uv, uf = icosphere(ico_level)
    for i in range(n_ico):
        r = rng.uniform(0.35, 0.75)
        c = np.array([rng.uniform(-4.0, 3.5), r * 1.05, rng.uniform(-4.0, 4.0)])
        d = 1.0 + 0.1 * fbm(uv * 1.5, seed=seed * 1000 + i)
        tris.append((c + uv * (r * d)[:, None])[uf].reshape(-1, 9))
        mats.append(random_material())
        tmat.append(np.full(len(uf), len(mats) - 1, np.uint32))
    nonlight = sum(len(t) for t in tris)
    tris.append(_quad((X + 1, 0.5, -1.5), (X + 1, 3.5, -1.5), (X + 1, 3.5, 1.5), (X + 1, 0.5, 1.5), (-1, 0, 0)))
    tmat.append(np.ones(2, np.uint32))
    tri = np.concatenate(tris).astype(np.float32)
    tri_mat = np.concatenate(tmat).astype(np.uint32)
    tri_light = np.full(len(tri), -1, np.int32)
    tri_light[nonlight:] = 0
    radii = np.clip(np.exp(rng.normal(-2.0, 0.5, n_spheres)), 0.03, 0.6)
    sph = np.zeros(n_spheres, SPHERE_DT)
    sph["center"][:, 0] = rng.uniform(-4.5, 4.3, n_spheres)
    sph["center"][:, 2] = rng.uniform(-4.5, 4.5, n_spheres)
    sph["center"][:, 1] = radii + rng.uniform(0.0, 2.5, n_spheres)
    sph["radius"] = radii
    for i in range(n_spheres):
        mats.append(random_material())
        sph["material_id"][i] = len(mats) - 1
    sph["light_id"] = -1
    lights = np.zeros(1, LIGHT_DT)
    lights[0] = ((light_intensity, light_intensity * 0.92, light_intensity * 0.8), 0)
    cam = Camera((-4.6, 2.2, 4.2), (1.0, 1.0, -1.5), (0.0, 1.0, 0.0), 65.0, width, height)
    return SceneData(tri, tri_mat, tri_light, sph, np.stack(mats), lights, cam, spp=spp,
                     max_depth=max_depth, rr_threshold=1.0, name="slit_room",
                     meta={"n_ico": n_ico, "ico_level": ico_level, "n_spheres": n_spheres})


def uneven_batch(n: int = 256, seed: int = 5, max_tris: int = 500_000, min_tris: int = 1_000) -> list[SceneData]:
    """Seeded batch of scenes of uneven size (the multi-scene batch workload).

    Per scene: triangle count log-uniform in [min_tris, max_tris], about 70% from fBm-displaced
    icospheres (level 2..5) and the rest random triangles; resolution from {128^2, 256^2, 512^2,
    640x360}; spp uniform in 4..64; max depth uniform in 4..10; materials 50% diffuse / 30%
    conductor / 20% dielectric; ground quad and 4 quad area lights as in the production scene.
    """
    rng = np.random.default_rng(seed)
    res = [(128, 128), (256, 256), (512, 512), (640, 360)]
    out = []
    for k in range(n):
        target = int(np.exp(rng.uniform(np.log(min_tris), np.log(max_tris))))
        level = 2 if target < 20_000 else (3 if target < 80_000 else (4 if target < 300_000 else 5))
        uv, uf = icosphere(level)
        n_ico = max(1, int(round(0.7 * target / len(uf))))
        mats = [material(MATTE, kd=(0.5, 0.5, 0.5)), material(MATTE, kd=(0, 0, 0))]

        def random_material():
            r = rng.random()
            if r < 0.5:
                return material(MATTE, kd=tuple(rng.uniform(0.1, 0.9, 3)))
            if r < 0.8:
                return material(CONDUCTOR, roughness=float(rng.uniform(0.05, 0.5)))
            return material(DIELECTRIC, ior=1.5)
        tris, tmat = [], []
        g = int(np.ceil(np.sqrt(n_ico)))
        span = 2.0 * g
        for i in range(n_ico):
            r = rng.uniform(0.5, 0.9)
            c = np.array([(i % g - (g - 1) / 2) * 2.0, r * 1.05, (i // g - (g - 1) / 2) * 2.0])
            d = 1.0 + 0.1 * fbm(uv * 1.5, seed=seed * 100000 + k * 100 + i)
            tris.append((c + uv * (r * d)[:, None])[uf].reshape(-1, 9))
            mats.append(random_material())
            tmat.append(np.full(len(uf), len(mats) - 1, np.uint32))
        nrand = max(0, target - n_ico * len(uf))
        if nrand:
            rt = random_triangles(nrand, seed=seed * 7919 + k).reshape(-1, 3, 3)
            rt = (rt - 0.5) * np.array([span, 2.0, span], np.float32) + np.array([0.0, 1.2, 0.0], np.float32)
            tris.append(rt.reshape(-1, 9))
            mats.append(random_material())
            tmat.append(np.full(nrand, len(mats) - 1, np.uint32))
        e = span / 2 + 2
        tris.append(_quad((-e, 0, -e), (e, 0, -e), (e, 0, e), (-e, 0, e), (0, 1, 0)))
        tmat.append(np.zeros(2, np.uint32))
        nonlight = sum(len(t) for t in tris)
        for lx in (-0.5 * e, 0.5 * e):
            for lz in (-0.5 * e, 0.5 * e):
                tris.append(_quad((lx - 1, 6, lz - 1), (lx + 1, 6, lz - 1), (lx + 1, 6, lz + 1), (lx - 1, 6, lz + 1),
                                  (0, -1, 0)))
                tmat.append(np.ones(2, np.uint32))
        tri = np.concatenate(tris).astype(np.float32)
        tri_mat = np.concatenate(tmat).astype(np.uint32)
        tri_light = np.full(len(tri), -1, np.int32)
        tri_light[nonlight:] = 0
        lights = np.zeros(1, LIGHT_DT)
        lights[0] = ((12.0, 12.0, 12.0), 0)
        w, h = res[int(rng.integers(0, len(res)))]
        spp = int(rng.integers(4, 65))
        depth = int(rng.integers(4, 11))
        cam = Camera((0.0, 0.35 * span + 3.0, 0.7 * span + 4.0), (0.0, 0.5, 0.0), (0.0, 1.0, 0.0), 50.0, w, h)
        out.append(SceneData(tri, tri_mat, tri_light, np.zeros(0, SPHERE_DT), np.stack(mats), lights, cam, spp=spp,
                             max_depth=depth, rr_threshold=1.0, name=f"batch{k}", meta={"target_tris": target}))
    return out
