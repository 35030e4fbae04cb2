"""The CPU oracle against its committed golden fixtures (tests/golden/make_golden.py) and the
published Philox4x32-10 known-answer vectors (Random123, Salmon et al. SC'11)."""
import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import scenes as S

from .conftest import ROOT

GOLD = ROOT / "tests" / "golden"
RTOL = 1e-6  # transcendental functions come from the platform libm


def test_philox_known_answers():
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kat:
        assert [int(x) for x in O.philox(ctr, key)] == list(want)


def test_rng_golden():
    g = np.load(GOLD / "oracle_rng.npz")
    got = np.array([O.rng_uniform(int(s), int(p), int(n), int(d)) for s, p, n, d in g["rng_index"]], np.float32)
    assert np.array_equal(got, g["rng_value"])
    assert ((got >= 0) & (got < 1)).all()


@pytest.mark.parametrize("fixed", [0, 1])
def test_trace_golden(fixed):
    g = np.load(GOLD / "oracle_trace.npz")
    sd, rays = S.ray_soup(3000, 4000)
    sc = O.OracleScene(sd, fixed_bvh=bool(fixed))
    h, cnt = sc.trace(rays, count=True, threads=1)
    assert sc.bvh_nodes == int(g[f"nodes_{fixed}"])
    assert np.array_equal(h["prim"], g[f"prim_{fixed}"])
    np.testing.assert_allclose(h["t"], g[f"t_{fixed}"], rtol=0)
    assert np.array_equal(sc.trace(rays, any_hit=True, threads=1), g[f"occ_{fixed}"])
    assert np.array_equal(cnt, g[f"counters_{fixed}"])


def test_faithful_bvh_is_a_chain():
    # F7: the bucket index is 0 or 15, so every split peels off the max-centroid primitives
    g = np.load(GOLD / "oracle_trace.npz")
    assert int(g["counters_0"][0]) > 10 * int(g["counters_1"][0])  # node visits explode


def test_render_golden():
    g = np.load(GOLD / "oracle_render.npz")
    sd = S.cornell(16, 16, spp=4)
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=False).render(mode, seed=7, threads=1)
        np.testing.assert_allclose(r["sum"], g[f"cornell_sum_{mode}"], rtol=RTOL, atol=1e-9)
        np.testing.assert_allclose(r["rgb"], g[f"cornell_rgb_{mode}"], rtol=RTOL, atol=1e-7)
    sd = S.production(24, 16, spp=2, n_ico=2, ico_level=2, n_spheres=20)
    r = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_PBRT, seed=1, threads=1)
    np.testing.assert_allclose(r["sum"], g["production_sum"], rtol=RTOL, atol=1e-9)


def test_quadric_render_golden():
    g = np.load(GOLD / "oracle_quadric.npz")
    sd = S.quadric_box(16, 16, spp=4)
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=False).render(mode, seed=9, threads=1)
        np.testing.assert_allclose(r["sum"], g[f"sum_{mode}"], rtol=RTOL, atol=1e-9)


def test_texture_and_integrator_golden():
    g = np.load(GOLD / "oracle_texture.npz")
    sd = S.textured_room(16, 16, spp=4)
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=True).render(mode, seed=3, threads=1)
        np.testing.assert_allclose(r["sum"], g[f"textured_sum_{mode}"], rtol=RTOL, atol=1e-9)
    mats = list(sd.materials) + [S.material(S.DIELECTRIC, ior=1.5)]
    sd.materials = np.stack(mats)
    sd.spheres = sd.spheres.copy()
    sd.spheres[1]["material_id"] = len(mats) - 1
    for name, kind, strategy in (("whitted", A.BG_INTEGRATOR_WHITTED, 0),
                                 ("direct_all", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL),
                                 ("direct_one", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ONE)):
        r = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_PBRT, seed=5, threads=1, integrator=kind,
                                                     light_strategy=strategy)
        np.testing.assert_allclose(r["sum"], g[f"{name}_sum"], rtol=RTOL, atol=1e-9)


def test_lights_and_samplers_golden():
    """The infinite light (rotated, with area lights besides), the stratified sampler, area lights on
    spheres, disks and cylinders and a thin-lens camera, both modes, against the committed fixture
    (the same renders as tests/golden/make_golden.py's lights_case)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(GOLD / "oracle_lights.npz")
    got = mg.lights_case()
    assert sorted(got) == sorted(g.files)
    for k in g.files:
        np.testing.assert_allclose(got[k], g[k], rtol=RTOL, atol=1e-9, err_msg=k)
