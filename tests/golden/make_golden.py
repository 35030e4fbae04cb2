"""Generates the committed golden fixtures of the CPU oracle (tests/golden/*.npz).

The reference has no golden vectors of its own, so these fixtures pin the oracle's behaviour
against regressions: small seeded ray-set traces (closest hit + any hit, reference-layout BVH
with and without the bucket bug) and small renders in both estimator modes.
Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle as O  # noqa: E402
from bonsai_gb300 import _abi as A  # noqa: E402
from bonsai_gb300 import scenes as S  # noqa: E402


def trace_case():
    sd, rays = S.ray_soup(3000, 4000)
    out = {}
    for fixed in (0, 1):
        sc = O.OracleScene(sd, fixed_bvh=bool(fixed))
        h, cnt = sc.trace(rays, count=True, threads=1)
        occ = sc.trace(rays, any_hit=True, threads=1)
        out[f"prim_{fixed}"] = h["prim"]
        out[f"t_{fixed}"] = h["t"]
        out[f"occ_{fixed}"] = occ
        out[f"counters_{fixed}"] = cnt
        out[f"nodes_{fixed}"] = np.array(sc.bvh_nodes)
    return out


def render_case():
    out = {}
    sd = S.cornell(16, 16, spp=4)
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=False).render(mode, seed=7, threads=1)
        out[f"cornell_sum_{mode}"] = r["sum"]
        out[f"cornell_rgb_{mode}"] = r["rgb"]
    sd = S.production(24, 16, spp=2, n_ico=2, ico_level=2, n_spheres=20)
    r = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_PBRT, seed=1, threads=1)
    out["production_sum"] = r["sum"]
    return out


def quadric_case():
    sd = S.quadric_box(16, 16, spp=4)
    out = {}
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=False).render(mode, seed=9, threads=1)
        out[f"sum_{mode}"] = r["sum"]
    return out


def texture_case():
    """The textured room (image / uv textures, the four mappings, MIPMap filtering, Oren-Nayar,
    vertex normals, orientation flags), both estimator modes, and the Whitted / direct-lighting
    integrators on the same room with its conductor sphere turned to glass."""
    out = {}
    sd = S.textured_room(16, 16, spp=4)
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=True).render(mode, seed=3, threads=1)
        out[f"textured_sum_{mode}"] = r["sum"]
    mats = list(sd.materials) + [S.material(S.DIELECTRIC, ior=1.5)]
    sd.materials = np.stack(mats)
    sd.spheres = sd.spheres.copy()
    sd.spheres[1]["material_id"] = len(mats) - 1
    for name, kind, strategy in (("whitted", A.BG_INTEGRATOR_WHITTED, 0),
                                 ("direct_all", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL),
                                 ("direct_one", A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ONE)):
        r = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_PBRT, seed=5, threads=1, integrator=kind,
                                                     light_strategy=strategy)
        out[f"{name}_sum"] = r["sum"]
    return out


def lights_case():
    """The lights and samplers beyond the box's triangle light: the reference's example scene with its
    infinite light (two area lights besides), rotated; area lights on spheres, disks and cylinders;
    the stratified sampler; a thin-lens camera; both estimator modes."""
    out = {}
    sd = S.env_sphere(16, 16, spp=4, max_depth=4, extra=True, env_w=16, env_h=8)
    sd.env.light_to_world = (S.rotation((0, 0, 1), 40.0) @ S.rotation((1, 0, 0), 20.0))[:3].astype(np.float32)
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=True).render(mode, seed=11, threads=1)
        out[f"env_sum_{mode}"] = r["sum"]
        r = O.OracleScene(sd, fixed_bvh=True).render(mode, seed=11, threads=1, sampler=S.StratifiedSampler(2, 2, 4))
        out[f"env_strat_sum_{mode}"] = r["sum"]
    sd = S.shape_lights(16, 16, spp=4, max_depth=4)
    sd.camera.lens_radius, sd.camera.focal_distance = 0.1, 3.0
    for mode in (A.BG_MODE_REF_COMPAT, A.BG_MODE_PBRT):
        r = O.OracleScene(sd, fixed_bvh=True).render(mode, seed=13, threads=1)
        out[f"shapes_sum_{mode}"] = r["sum"]
    return out


def rng_case():
    idx = np.array([(0, 0, 0, 0), (1, 2, 3, 4), (12345, 999, 7, 41), (2**32 - 1, 2**31, 65535, 1023)], np.uint64)
    vals = np.array([O.rng_uniform(int(s), int(p), int(n), int(d)) for s, p, n, d in idx], np.float32)
    return {"rng_index": idx, "rng_value": vals}


CASES = {"oracle_trace.npz": trace_case, "oracle_render.npz": render_case, "oracle_rng.npz": rng_case,
         "oracle_quadric.npz": quadric_case, "oracle_texture.npz": texture_case, "oracle_lights.npz": lights_case}

if __name__ == "__main__":
    # writes the fixtures named on the command line (all of them without arguments)
    names = sys.argv[1:] or list(CASES)
    for name in names:
        np.savez_compressed(HERE / name, **CASES[name]())
    print("wrote", names)
