"""OBJ meshes through bg_scene_add_obj render exactly like the same triangles added directly, and
bg_film_write_exr stores the resolved film that bg_render returns."""
import ctypes as C

import numpy as np
import pytest

from bonsai_gb300 import _abi as A
from bonsai_gb300 import gpu as G
from bonsai_gb300 import io as bio
from bonsai_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _obj_text(tri):
    lines = []
    for t in tri.reshape(-1, 3, 3):
        for v in t:
            lines.append("v %r %r %r" % tuple(float(x) for x in v))
    for i in range(len(tri)):
        lines.append("f %d %d %d" % (3 * i + 1, 3 * i + 2, 3 * i + 3))
    return "\n".join(lines) + "\n"


def test_obj_scene_renders_like_direct_triangles(gpu_ctx, tmp_path):
    sd = S.cornell(48, 48, spp=4, max_depth=4)
    nonlight = sd.tri_light < 0
    mesh = sd.tri[nonlight]
    p = tmp_path / "walls.obj"
    p.write_text(_obj_text(mesh))
    xf = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)
    np.testing.assert_array_equal(bio.read_obj(p, xf), mesh)

    # scene A: the OBJ file for the walls (one material per call, so one call per material)
    lib, ctx = gpu_ctx.lib, gpu_ctx
    h = C.c_void_p()
    ctx.check(lib.bg_scene_create(ctx.h, C.byref(h)))
    try:
        for m in sd.materials:
            mm = A.bg_material.from_buffer_copy(np.ascontiguousarray(m).tobytes())
            ctx.check(lib.bg_scene_add_material(h, C.byref(mm), None))
        for l in sd.lights:
            ll = A.bg_area_light.from_buffer_copy(np.ascontiguousarray(l).tobytes())
            ctx.check(lib.bg_scene_add_area_light(h, C.byref(ll), None))
        mats = sd.tri_mat[nonlight]
        order = []
        for mid in np.unique(mats):
            sel = np.nonzero(mats == mid)[0]
            q = tmp_path / f"m{mid}.obj"
            q.write_text(_obj_text(mesh[sel]))
            n = C.c_size_t()
            ctx.check(lib.bg_scene_add_obj(h, str(q).encode(), xf.ctypes.data, int(mid), -1, C.byref(n)))
            assert n.value == len(sel)
            order.extend(sel.tolist())
        lt = np.ascontiguousarray(sd.tri[~nonlight])
        lm = np.ascontiguousarray(sd.tri_mat[~nonlight])
        ll = np.ascontiguousarray(sd.tri_light[~nonlight])
        ctx.check(lib.bg_scene_add_triangles(h, lt.ctypes.data, len(lt), lm.ctypes.data, ll.ctypes.data))
        if sd.nsph:
            sp = np.ascontiguousarray(sd.spheres)
            ctx.check(lib.bg_scene_add_spheres(h, sp.ctypes.data, sd.nsph))
        st = A.bg_build_stats()
        ctx.check(lib.bg_scene_commit(h, A.BG_BVH_WIDE, C.byref(st)))
        cam = G.camera_struct(sd.camera)
        o = A.bg_render_opts()
        o.spp, o.max_depth, o.rr_threshold, o.mode, o.seed = 16, 4, 1.0, A.BG_MODE_PBRT, 3
        rgb_a = np.zeros((48, 48, 3), np.float32)
        rs = A.bg_render_stats()
        ctx.check(lib.bg_render(ctx.h, h, C.byref(cam), C.byref(o), rgb_a.ctypes.data, C.byref(rs)))
        exr = tmp_path / "film.exr"
        ctx.check(lib.bg_film_write_exr(ctx.h, str(exr).encode()))
        np.testing.assert_array_equal(bio.read_exr(exr), rgb_a)
    finally:
        lib.bg_scene_destroy(h)

    # scene B: the same triangles in the same order, added directly
    sd2 = S.SceneData(np.concatenate([mesh[order], sd.tri[~nonlight]]),
                      np.concatenate([sd.tri_mat[nonlight][order], sd.tri_mat[~nonlight]]),
                      np.concatenate([np.full(len(order), -1, np.int32), sd.tri_light[~nonlight]]),
                      sd.spheres, sd.materials, sd.lights, sd.camera, spp=16, max_depth=4, rr_threshold=1.0)
    sc = G.Scene(gpu_ctx, sd2, A.BG_BVH_WIDE)
    try:
        rgb_b = G.PathIntegrator(sd.camera, 16, 4, mode=A.BG_MODE_PBRT, seed=3).render(sc).rgb
    finally:
        sc.close()
    np.testing.assert_array_equal(rgb_a, rgb_b)
