"""Known answers for the oracle's InfiniteAreaLight (src/lights/infinite.rs) and Distribution2D
(src/base/sampling.rs), no GPU.  A convex matte sphere of albedo rho under an environment of
uniform radiance 1 reflects exactly rho (the furnace); under a non-uniform map its direct lighting is
rho / pi times the cosine-weighted integral of the map, computed here by quadrature.  PBRT mode meets
both; REF_COMPAT mode carries the reference's Distribution2D defects (a conditional keeps the whole
tail of the function, so sampled u shrinks; pdf() truncates its point to cell (0, 0)) and is biased."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import scenes as S

ALBEDO = 0.5


def _grey_sphere(env_rgb, w=32, h=32):
    sd = S.env_sphere(w, h, spp=16, max_depth=1)
    sd.env.rgb = env_rgb
    sd.materials = np.stack([S.material(S.MATTE, kd=(ALBEDO, ALBEDO, ALBEDO))])
    sd.textures = []
    return sd


def _sphere_normals(sd):
    """Pixels whose whole footprint (its four corner rays) hits the unit sphere, with the normal
    where the pixel-centre camera ray hits it."""
    cam = sd.camera

    def hit(fx, fy):
        r = O.camera_ray(cam, fx, fy)
        o, d = r[:3].astype(np.float64), r[3:].astype(np.float64)
        b = np.dot(o, d)
        disc = b * b - (np.dot(o, o) - 1.0)
        return None if disc <= 0.0 else o + (-b - np.sqrt(disc)) * d

    out = {}
    for y in range(cam.height):
        for x in range(cam.width):
            if all(hit(x + dx, y + dy) is not None for dx in (0, 1) for dy in (0, 1)):
                out[(y, x)] = hit(x + 0.5, y + 0.5)
    return out


def _bilinear_repeat(img, s, t):
    """MIPMap::triangle at level 0 with repeat wrapping (src/base/mipmap.rs:156-173), vectorised."""
    h, w, _ = img.shape
    fs, ft = s * w - 0.5, t * h - 0.5
    x0, y0 = np.floor(fs).astype(np.int64), np.floor(ft).astype(np.int64)
    ds, dt = (fs - x0)[..., None], (ft - y0)[..., None]
    x1, y1 = (x0 + 1) % w, (y0 + 1) % h
    x0, y0 = x0 % w, y0 % h
    return ((1 - ds) * (1 - dt) * img[y0, x0] + (1 - ds) * dt * img[y1, x0] + ds * (1 - dt) * img[y0, x1] +
            ds * dt * img[y1, x1])


def _irradiance(img, n, nt=512, nphi=1024):
    """Integral of the map's radiance times max(0, cos) over the sphere of directions (midpoint rule)."""
    theta = (np.arange(nt) + 0.5) * np.pi / nt
    phi = (np.arange(nphi) + 0.5) * 2 * np.pi / nphi
    T, P = np.meshgrid(theta, phi, indexing="ij")
    w = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1)
    L = _bilinear_repeat(img.astype(np.float64), P / (2 * np.pi), T / np.pi)
    cos = np.clip(w @ n, 0, None)
    dA = (np.pi / nt) * (2 * np.pi / nphi) * np.sin(T)
    return (L * (cos * dA)[..., None]).sum(axis=(0, 1))


def test_uniform_environment_furnace():
    sd = _grey_sphere(np.ones((16, 32, 3), np.float32))
    o = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=512, threads=4)
    rgb, n = o["rgb"], 512
    var = o["sumsq"] / n - (o["sum"] / n) ** 2
    px = _sphere_normals(sd)
    vals = np.array([rgb[y, x, 0] for (y, x) in px])
    se = np.sqrt(np.mean([var[y, x, 0] for (y, x) in px]) / n / len(px))
    assert abs(vals.mean() - ALBEDO) < 4 * se + 1e-4
    # pixels that miss the sphere see the map: radiance 1 (bilinear weights summing to one)
    np.testing.assert_allclose(rgb[0, 0], 1.0, atol=1e-5)
    np.testing.assert_allclose(rgb[-1, -1], 1.0, atol=1e-5)


def test_environment_direct_lighting_matches_quadrature():
    """A smooth sky / ground map with a broad bright lobe: each pixel's mean within 5 standard
    errors of rho / pi times the irradiance (pixel footprints are small against the map's scale)."""
    img = S.environment_image(64, 32, seed=3, sun=(0.3, 0.05), sun_radius=0.6, sun_radiance=3.0)
    img = np.ascontiguousarray(img.mean(axis=2, keepdims=True).repeat(3, axis=2) * [1.0, 0.8, 0.6], np.float32)
    sd = _grey_sphere(img)
    spp = 256
    o = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=spp, threads=4)
    var = o["sumsq"] / spp - (o["sum"] / spp) ** 2
    px = _sphere_normals(sd)
    keys = sorted(px)[:: max(1, len(px) // 24)]
    z = []
    for (y, x) in keys:
        expect = ALBEDO / np.pi * _irradiance(img, px[(y, x)], 256, 512)
        got = o["rgb"][y, x]
        se = np.sqrt(var[y, x] / spp) + 1e-3 * expect
        z.append(np.abs(got - expect) / se)
    z = np.array(z)
    assert z.max() < 5.0, z.max()


def test_ref_compat_distribution_defects_bias_the_estimate():
    """REF_COMPAT's light half samples directions whose pdf it misreports: the furnace is off."""
    sd = _grey_sphere(np.ones((16, 32, 3), np.float32))
    rgb = O.OracleScene(sd).render(A.BG_MODE_REF_COMPAT, spp=128, threads=4)["rgb"]
    px = _sphere_normals(sd)
    vals = np.array([rgb[y, x, 0] for (y, x) in px])
    assert abs(vals.mean() - ALBEDO) > 0.05
    np.testing.assert_allclose(rgb[0, 0], 1.0, atol=1e-5)  # escaping camera rays still see the map


def test_light_list_order_and_single_infinite_light():
    sd = S.env_sphere(8, 8, extra=True)
    sc = O.OracleScene(sd)
    assert O.lib().orc_num_lights(sc.h) == 3  # two emitting triangles, then the infinite light
    el, keep = S.env_struct(sd.env)
    assert O.lib().orc_scene_add_infinite_light(sc.h, C.byref(el)) == -1


@pytest.mark.parametrize("mode", [A.BG_MODE_PBRT, A.BG_MODE_REF_COMPAT])
@pytest.mark.parametrize("integrator,strategy", [(A.BG_INTEGRATOR_PATH, 0), (A.BG_INTEGRATOR_WHITTED, 0),
                                                 (A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL),
                                                 (A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ONE)])
def test_every_integrator_sees_the_environment(mode, integrator, strategy):
    """Background pixels show the map itself; the lit sphere is finite and not black."""
    sd = S.env_sphere(24, 24, spp=4, extra=True)
    o = O.OracleScene(sd).render(mode, spp=4, integrator=integrator, light_strategy=strategy, threads=4)
    rgb = o["rgb"]
    assert np.isfinite(rgb).all()
    assert rgb[12, 12].sum() > 0.0
    assert rgb[0, 0].sum() > 0.0 and rgb[-1, 0].sum() > 0.0
