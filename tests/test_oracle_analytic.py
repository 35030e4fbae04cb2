"""Analytic known answers for the CPU oracle (it has no reference outputs to be checked against).

* White furnace: a closed box of albedo rho whose walls all emit L_e = 1 has L = L_e / (1 - rho)
  everywhere; the PBRT estimator (MIS next-event estimation + BSDF sampling + roulette) must give it.
* A glass sphere inside an emitting black box transmits or reflects everything: L = 1.
* BSDF sample / pdf / eval consistency: E[f cos / pdf] over sampled directions equals the
  quadrature of f cos over the hemisphere (PBRT mode); in REF_COMPAT mode the Trowbridge-Reitz
  pdf uses G1 = lambda (src/base/microfacet.rs:17-19), which breaks the identity.
"""
import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import scenes as S


def _closed_box(rho, emit=1.0, two_sided=1):
    quads = [((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), (0, 1, 0)),
             ((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), (0, -1, 0)),
             ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (0, 0, 1)),
             ((-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1), (0, 0, -1)),
             ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), (1, 0, 0)),
             ((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1), (-1, 0, 0))]
    tri = np.concatenate([S._quad(*q) for q in quads])
    mats = [S.material(S.MATTE, kd=(rho, rho, rho)), S.material(S.DIELECTRIC, ior=1.5)]
    lights = np.zeros(1, S.LIGHT_DT)
    lights[0] = ((emit, emit, emit), two_sided)
    cam = S.Camera((0.0, 0.0, 0.6), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), 60.0, 12, 12)
    return S.SceneData(tri, np.zeros(len(tri), np.uint32), np.zeros(len(tri), np.int32), np.zeros(0, S.SPHERE_DT),
                       np.stack(mats), lights, cam, spp=128, max_depth=60, rr_threshold=1.0)


@pytest.mark.parametrize("rho", [0.0, 0.5, 0.8])
def test_white_furnace(rho):
    sd = _closed_box(rho)
    r = O.OracleScene(sd).render(A.BG_MODE_PBRT, seed=11)
    n = 12 * 12 * sd.spp
    x = r["sum"].sum(axis=2) / 3.0  # per pixel sum of samples (channel mean)
    mean = x.sum() / n
    var = (r["sumsq"].sum(axis=2) / 3.0).sum() / n - mean ** 2
    se = np.sqrt(max(var, 0.0) / n)
    expected = 1.0 / (1.0 - rho)
    assert abs(mean - expected) <= 4 * se + 1e-9, (mean, expected, se)


def test_glass_sphere_in_emitting_box():
    sd = _closed_box(0.0)
    sph = np.zeros(1, S.SPHERE_DT)
    sph[0] = ((0.0, 0.0, -0.2), 0.4, 1, -1)
    sd.spheres = sph
    r = O.OracleScene(sd).render(A.BG_MODE_PBRT, seed=3)
    mean = r["sum"].sum() / (3 * 12 * 12 * sd.spp)
    # paths trapped by total internal reflection past max_depth lose a little energy
    assert 0.98 <= mean <= 1.0 + 1e-3


def _hemisphere_quadrature(mat, wo, mode, n=256):
    # midpoint rule in (cos theta, phi): dw = d(cos theta) d(phi)
    ct = (np.arange(n) + 0.5) / n
    ph = (np.arange(2 * n) + 0.5) * np.pi / n
    tot = 0.0
    for c in ct[::4]:
        s = np.sqrt(1 - c * c)
        for p in ph[::4]:
            wi = (s * np.cos(p), s * np.sin(p), c)
            f = O.bsdf_eval(mat, wo, wi, mode)[:3]
            tot += f.mean() * c
    return tot * (1.0 / (n / 4)) * (np.pi / (n / 4))


def _sampled_estimate(mat, wo, mode, n=4000, seed=0):
    rng = np.random.default_rng(seed)
    acc = 0.0
    for _ in range(n):
        out = O.bsdf_sample(mat, wo, float(rng.random()), float(rng.random()), mode)
        f, pdf, wi = out[:3], out[3], out[4:7]
        if pdf > 0:
            acc += f.mean() * abs(wi[2]) / pdf
    return acc / n


@pytest.mark.parametrize("kind", ["matte", "conductor", "plastic", "oren_nayar"])
def test_bsdf_sampling_matches_quadrature_pbrt(kind):
    mat = {"matte": S.material(S.MATTE, kd=(0.6, 0.5, 0.4)),
           "conductor": S.material(S.CONDUCTOR, roughness=0.3),
           "plastic": S.material(S.PLASTIC, kd=(0.5, 0.5, 0.5), ks=(0.3, 0.3, 0.3), roughness=0.3),
           "oren_nayar": S.material(S.MATTE, kd=(0.6, 0.5, 0.4), sigma=25.0)}[kind]
    wo = np.array([0.3, 0.2, 0.0])
    wo[2] = np.sqrt(1 - 0.13)
    q = _hemisphere_quadrature(mat, wo, A.BG_MODE_PBRT)
    e = _sampled_estimate(mat, wo, A.BG_MODE_PBRT)
    assert abs(e - q) <= 0.05 * q, (e, q)


def test_ref_compat_microfacet_pdf_is_inconsistent():
    # F4: G1 = lambda makes the reference's pdf disagree with its own sampling
    mat = S.material(S.CONDUCTOR, roughness=0.3)
    wo = np.array([0.6, 0.0, 0.8])
    q = _hemisphere_quadrature(mat, wo, A.BG_MODE_REF_COMPAT)
    e = _sampled_estimate(mat, wo, A.BG_MODE_REF_COMPAT)
    assert abs(e - q) > 0.2 * q


def test_lambertian_closed_form():
    mat = S.material(S.MATTE, kd=(0.6, 0.5, 0.4))
    out = O.bsdf_eval(mat, (0.0, 0.0, 1.0), (0.6, 0.0, 0.8), A.BG_MODE_PBRT)
    np.testing.assert_allclose(out[:3], np.array([0.6, 0.5, 0.4]) / np.pi, rtol=1e-6)
    np.testing.assert_allclose(out[3], 0.8 / np.pi, rtol=1e-6)


def test_oren_nayar_closed_form():
    """The Oren-Nayar qualitative model (Oren & Nayar 1994, as in PBRT-v3):
    f = R/pi (A + B max(0, cos(phi_i - phi_o)) sin(alpha) tan(beta)), A = 1 - s^2 / (2 (s^2 + 0.33)),
    B = 0.45 s^2 / (s^2 + 0.09), s = sigma in radians, alpha / beta the larger / smaller of the angles."""
    sigma = 30.0
    mat = S.material(S.MATTE, kd=(0.6, 0.5, 0.4), sigma=sigma)
    s2 = np.radians(sigma) ** 2
    a, b = 1 - s2 / (2 * (s2 + 0.33)), 0.45 * s2 / (s2 + 0.09)
    for wo, wi in [((0.3, 0.1, 0.0), (-0.5, 0.2, 0.0)), ((0.0, 0.6, 0.0), (0.1, 0.45, 0.0))]:
        wo, wi = np.array(wo), np.array(wi)
        wo[2], wi[2] = np.sqrt(1 - wo @ wo), np.sqrt(1 - wi @ wi)
        ti, to = np.arccos(wi[2]), np.arccos(wo[2])
        dphi = np.arctan2(wi[1], wi[0]) - np.arctan2(wo[1], wo[0])
        want = np.array([0.6, 0.5, 0.4]) / np.pi * (a + b * max(0.0, np.cos(dphi)) * np.sin(max(ti, to))
                                                     * np.tan(min(ti, to)))
        out = O.bsdf_eval(mat, wo, wi, A.BG_MODE_PBRT)
        np.testing.assert_allclose(out[:3], want, rtol=2e-5)
        np.testing.assert_allclose(out[3], wi[2] / np.pi, rtol=1e-5)


def test_oren_nayar_sigma_zero_is_lambertian():
    wo, wi = (0.3, 0.1, np.sqrt(0.9)), (-0.5, 0.2, np.sqrt(0.71))
    a = O.bsdf_eval(S.material(S.MATTE, kd=(0.6, 0.5, 0.4), sigma=0.0), wo, wi, A.BG_MODE_PBRT)
    b = O.bsdf_eval(S.material(S.MATTE, kd=(0.6, 0.5, 0.4)), wo, wi, A.BG_MODE_PBRT)
    np.testing.assert_array_equal(a, b)


def test_thin_lens_rays_meet_on_the_plane_of_focus():
    """PerspectiveCamera with a lens (perspective.rs:127-139): the rays of one film point through
    different lens points cross the plane at focal_distance along the view axis in one point, and
    their origins lie on the lens disk of radius lens_radius."""
    cam = S.Camera((0.0, 1.0, 6.0), (0.0, 0.5, 0.0), (0.0, 1.0, 0.0), 40.0, 64, 48, lens_radius=0.25,
                   focal_distance=4.0)
    pos = np.array(cam.position, np.float64)
    fwd = np.array(cam.look_at, np.float64) - pos
    fwd /= np.linalg.norm(fwd)
    rng = np.random.default_rng(3)
    for fx, fy in ((10.5, 7.25), (32.0, 24.0), (60.0, 40.0)):
        pts = []
        for lu in rng.random((12, 2)):
            r = O.camera_ray(cam, fx, fy, 0.0, lens=tuple(lu)).astype(np.float64)
            o, d = r[:3], r[3:]
            assert np.linalg.norm(o - pos) <= 0.25 * (1 + 1e-5) + 1e-5
            assert abs(np.dot(o - pos, fwd)) < 1e-4  # the lens plane is perpendicular to the view axis
            t = (4.0 - np.dot(o - pos, fwd)) / np.dot(d, fwd)
            pts.append(o + t * d)
        pts = np.array(pts)
        assert np.abs(pts - pts.mean(axis=0)).max() < 2e-4
        # the pinhole ray of the film point passes through the same focus point
        pin = S.Camera(cam.position, cam.look_at, cam.up, 40.0, 64, 48)
        r = O.camera_ray(pin, fx, fy).astype(np.float64)
        t = (4.0 - np.dot(r[:3] - pos, fwd)) / np.dot(r[3:], fwd)
        assert np.abs(r[:3] + t * r[3:] - pts.mean(axis=0)).max() < 1e-3


def _floor_scene(w, h, cam, sphere=None, disk=None, albedo=0.5, inner=0.0, cylinder=None):
    """A matte floor (y = 0, 20 x 20) lit only by one shape light of unit radiance: `sphere` =
    (center, radius), `disk` = (center, radius) facing down."""
    tri = S._quad((-10, 0, -10), (10, 0, -10), (10, 0, 10), (-10, 0, 10), (0, 1, 0))
    mats = np.stack([S.material(S.MATTE, kd=(albedo,) * 3), S.material(S.MATTE)])
    lights = np.zeros(1, S.LIGHT_DT)
    lights[0]["intensity"], lights[0]["two_sided"] = (1.0, 1.0, 1.0), 0
    sph = np.zeros(0, S.SPHERE_DT)
    quads = np.zeros(0, S.QUADRIC_DT)
    if sphere is not None:
        sph = np.zeros(1, S.SPHERE_DT)
        sph[0]["center"], sph[0]["radius"], sph[0]["material_id"], sph[0]["light_id"] = sphere[0], sphere[1], 1, 0
    if disk is not None:
        q = S.quadric(S.DISK, S.translation(disk[0]) @ S.rotation((1, 0, 0), 90), 1, radius=disk[1], height=0.0,
                      inner_radius=inner)
        q["light_id"] = 0
        quads = np.stack([q])
    if cylinder is not None:  # (center, radius, half length): axis along world z
        q = S.quadric(S.CYLINDER, S.translation(cylinder[0]), 1, radius=cylinder[1], z_min=-cylinder[2],
                      z_max=cylinder[2])
        q["light_id"] = 0
        quads = np.stack([q])
    return S.SceneData(tri.astype(np.float32), np.zeros(2, np.uint32), np.full(2, -1, np.int32), sph, mats, lights,
                       cam, quadrics=quads, spp=16, max_depth=1, rr_threshold=1.0)


def test_sphere_light_direct_lighting_known_answer():
    """Irradiance from a sphere of radiance L fully above the horizon: pi L (r / d)^2 cos(theta);
    a matte floor of albedo rho shows rho L (r / d)^2 cos(theta) (PBRT, direct lighting only)."""
    c, r = np.array([1.2, 1.0, 0.0]), 0.4
    cam = S.Camera((0.0, 2.0, 0.01), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 30.0, 33, 33)
    sd = _floor_scene(33, 33, cam, sphere=(tuple(c), r))
    spp = 1024
    o = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=spp, rows=(12, 21, 4), threads=4)
    var = o["sumsq"] / spp - (o["sum"] / spp) ** 2
    for y in (12, 16, 20):
        for x in (12, 16, 20):
            ray = O.camera_ray(cam, x + 0.5, y + 0.5).astype(np.float64)
            t = -ray[1] / ray[4]
            p = ray[:3] + t * ray[3:]
            d = c - p
            dist2 = d @ d
            expect = 0.5 * (r * r / dist2) * (d[1] / np.sqrt(dist2))
            se = np.sqrt(var[y, x, 0] / spp) + 2e-3 * expect
            assert abs(o["rgb"][y, x, 0] - expect) < 5 * se, (x, y, o["rgb"][y, x, 0], expect)


def test_disk_light_on_axis_known_answer():
    """A disk of radius R and radiance L at height h facing down: irradiance on its axis
    pi L R^2 / (h^2 + R^2); both the PBRT annulus sampling and the intersection pdf are exercised."""
    h, R = 1.5, 0.6
    cam = S.Camera((0.0, 0.8, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 10.0, 33, 33)
    sd = _floor_scene(33, 33, cam, disk=((0.0, h, 0.0), R))
    spp = 4096
    o = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=spp, rows=(16, 17, 1), threads=4)
    expect = 0.5 * R * R / (h * h + R * R)
    v = o["rgb"][16, 16, 0]
    se = np.sqrt(max(o["sumsq"][16, 16, 0] / spp - (o["sum"][16, 16, 0] / spp) ** 2, 0) / spp)
    assert abs(v - expect) < 5 * se + 1e-3 * expect, (v, expect)


def test_ref_compat_shape_light_defects_change_the_estimate():
    """REF_COMPAT: the sphere's sample normal of length r (F21) and its cone pdf against area
    sampling (F20) move the estimate away from the PBRT value."""
    c, r = (1.2, 1.0, 0.0), 0.4
    cam = S.Camera((0.0, 2.0, 0.01), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 30.0, 17, 17)
    sd = _floor_scene(17, 17, cam, sphere=(c, r))
    pb = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_PBRT, spp=256, threads=4)["rgb"].mean()
    rf = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_REF_COMPAT, spp=256, threads=4)["rgb"].mean()
    assert abs(rf - pb) > 0.1 * pb, (rf, pb)


def test_annulus_light_on_axis_known_answer_and_ref_defect():
    """An annulus (radii Ri < R) at height h facing down: irradiance on its axis
    pi L (R^2 / (h^2 + R^2) - Ri^2 / (h^2 + Ri^2)).  PBRT draws the annulus and meets it; REF_COMPAT
    draws the whole disk (F22), and samples in the hole find no surface behind them."""
    h, R, Ri = 1.5, 0.6, 0.35
    cam = S.Camera((0.0, 0.8, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 10.0, 33, 33)
    sd = _floor_scene(33, 33, cam, disk=((0.0, h, 0.0), R), inner=Ri)
    spp = 4096
    expect = 0.5 * (R * R / (h * h + R * R) - Ri * Ri / (h * h + Ri * Ri))
    o = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=spp, rows=(16, 17, 1), threads=4)
    v = o["rgb"][16, 16, 0]
    se = np.sqrt(max(o["sumsq"][16, 16, 0] / spp - (o["sum"][16, 16, 0] / spp) ** 2, 0) / spp)
    assert abs(v - expect) < 5 * se + 1e-3 * expect, (v, expect)
    rf = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_REF_COMPAT, spp=spp, rows=(16, 17, 1), threads=4)
    assert abs(rf["rgb"][16, 16, 0] - expect) > 0.05 * expect


def test_cylinder_light_direct_lighting_matches_quadrature():
    """A one-sided (outward) tube light of unit radiance above a matte floor: the floor shows
    rho / pi * integral of cos_p cos_l / d^2 over the tube's surface facing the point (the tube is
    convex, so that part is unoccluded), integrated here with a midpoint rule (PBRT)."""
    c, rad, half = np.array([0.0, 0.8, 0.0]), 0.25, 0.6
    cam = S.Camera((0.3, 0.3, 0.0), (0.3, 0.0, 0.0), (0.0, 0.0, -1.0), 10.0, 33, 33)
    sd = _floor_scene(33, 33, cam, cylinder=(tuple(c), rad, half))
    spp = 4096
    o = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=spp, rows=(16, 17, 1), threads=4)
    ray = O.camera_ray(cam, 16.5, 16.5).astype(np.float64)
    p = ray[:3] + (-ray[1] / ray[4]) * ray[3:]
    nz, nphi = 400, 800
    z = -half + (np.arange(nz) + 0.5) * (2 * half / nz)
    phi = (np.arange(nphi) + 0.5) * (2 * np.pi / nphi)
    Z, PH = np.meshgrid(z, phi, indexing="ij")
    nrm = np.stack([np.cos(PH), np.sin(PH), np.zeros_like(PH)], -1)
    x = c + rad * nrm + np.stack([np.zeros_like(Z), np.zeros_like(Z), Z], -1)
    d = p - x
    dist2 = np.sum(d * d, -1)
    dn = d / np.sqrt(dist2)[..., None]
    cos_l = np.sum(nrm * dn, -1)
    cos_p = -dn[..., 1]  # the floor's normal is +y; d points from the tube to p
    dA = rad * (2 * np.pi / nphi) * (2 * half / nz)
    E = np.sum(np.where((cos_l > 0) & (cos_p > 0), cos_l * cos_p / dist2, 0.0) * dA)
    expect = 0.5 / np.pi * E
    v = o["rgb"][16, 16, 0]
    se = np.sqrt(max(o["sumsq"][16, 16, 0] / spp - (o["sum"][16, 16, 0] / spp) ** 2, 0) / spp)
    assert abs(v - expect) < 5 * se + 2e-3 * expect, (v, expect, se)
