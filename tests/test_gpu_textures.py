"""Textures, MIPMap filtering, ray differentials, Oren-Nayar and triangle-mesh attributes (vertex
normals, uvs, orientation flags): the device renders of a scene that uses all of them against the
CPU oracle (same random numbers, same bar as tests/test_gpu_render.py), in both estimator modes and
through both the wavefront (8-wide BVH) and the megakernel (reference-layout BVH)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import gpu as G
from bonsai_gb300 import io as bio
from bonsai_gb300 import scenes as S

from .parity import compare_renders

pytestmark = pytest.mark.gpu

Z3_FRAC = 0.01


def _pair(ctx, sd, mode, bvh, spp, seed=0):
    orc = O.OracleScene(sd, fixed_bvh=True)
    o = orc.render(mode, spp=spp, seed=seed)
    sc = G.Scene(ctx, sd, bvh)
    try:
        r = G.PathIntegrator(sd.camera, spp, sd.max_depth, sd.rr_threshold, mode=mode, seed=seed).render(sc)
    finally:
        sc.close()
    s1, s2, n = G.PathIntegrator.moments(ctx, sd.camera.width, sd.camera.height)
    assert (n == spp).all()
    return r, o, compare_renders(s1, s2, n, o["sum"], o["sumsq"], np.full(n.shape, spp))


@pytest.mark.parametrize("bvh", [A.BG_BVH_WIDE, A.BG_BVH_REFERENCE_FIXED])
def test_textured_room_pbrt(gpu_ctx, bvh):
    sd = S.textured_room(48, 48, spp=16)
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_MODE_PBRT, bvh, 16)
    print(cmp)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9
    np.testing.assert_allclose(r.rgb.mean(), o["rgb"].mean(), rtol=2e-3)


def test_textured_room_ref_compat(gpu_ctx):
    sd = S.textured_room(48, 48, spp=16)
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_MODE_REF_COMPAT, A.BG_BVH_REFERENCE_FIXED, 16)
    print(cmp)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9


def test_textures_and_attributes_change_the_image(gpu_ctx):
    """Guards against a silently ignored feature: the textured room differs from the same room with
    the texture references, vertex normals and flags removed, in the regions they cover."""
    sd = S.textured_room(48, 48, spp=8)
    plain = S.textured_room(48, 48, spp=8)
    plain.textures = []
    plain.materials = plain.materials.copy()
    plain.materials["kd_texture"] = 0
    plain.materials["ks_texture"] = 0
    plain.materials["sigma"] = 0.0
    plain.tri_normals = plain.tri_normal_mask = plain.tri_flags = None
    out = []
    for d in (sd, plain):
        sc = G.Scene(gpu_ctx, d, A.BG_BVH_WIDE)
        try:
            out.append(G.PathIntegrator(d.camera, 8, d.max_depth, 1.0, mode=A.BG_MODE_PBRT).render(sc).rgb)
        finally:
            sc.close()
    a, b = out
    back = (slice(8, 20), slice(16, 32))  # back wall, above the spheres
    assert np.abs(a[back] - b[back]).mean() > 0.05


def _mesh_obj(tmp_path):
    """A smooth-shaded, uv-mapped grid bump (vertex normals and texture coordinates per face vertex)."""
    n = 6
    xs = np.linspace(-0.6, 0.6, n + 1)
    lines, faces = [], []
    for j in range(n + 1):
        for i in range(n + 1):
            x, z = xs[i], xs[j]
            y = 0.15 * np.cos(2.5 * x) * np.cos(2.5 * z)
            lines.append(f"v {x:.6f} {y:.6f} {z:.6f}")
            lines.append(f"vt {i / n:.6f} {j / n:.6f}")
            nx, nz = 0.375 * np.sin(2.5 * x) * np.cos(2.5 * z), 0.375 * np.cos(2.5 * x) * np.sin(2.5 * z)
            lines.append(f"vn {nx:.6f} 1 {nz:.6f}")
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i + 1
            b, c, d = a + 1, a + n + 2, a + n + 1
            for t in ((a, d, c), (a, c, b)):
                faces.append("f " + " ".join(f"{k}/{k}/{k}" for k in t))
    p = tmp_path / "bump.obj"
    p.write_text("\n".join(lines + faces) + "\n")
    return p


@pytest.mark.parametrize("mirror", [False, True])
def test_obj_mesh_attributes_render_like_oracle(gpu_ctx, tmp_path, mirror):
    path = _mesh_obj(tmp_path)
    xf = np.array([[1, 0, 0, 0], [0, 1, 0, -0.85], [0, 0, 1, 0]], np.float32)
    if mirror:
        xf[0, 0] = -1.0  # swaps handedness
    tri, nrm, uv, flags = bio.read_obj_mesh(path, xf)
    assert nrm is not None and uv is not None and bool(flags & A.BG_TRI_SWAPS_HANDEDNESS) == mirror
    base = S.textured_room(40, 40, spp=16)
    nb = base.ntri
    sd = S.SceneData(np.concatenate([base.tri, tri]), np.concatenate([base.tri_mat, np.full(len(tri), 5, np.uint32)]),
                     np.concatenate([base.tri_light, np.full(len(tri), -1, np.int32)]), base.spheres[:0],
                     base.materials, base.lights, base.camera, spp=16, max_depth=4, rr_threshold=1.0,
                     tri_normals=np.concatenate([base.tri_normals, nrm]),
                     tri_normal_mask=np.concatenate([base.tri_normal_mask, np.ones(len(tri), bool)]),
                     tri_uvs=np.concatenate([base.tri_uvs, uv]),
                     tri_flags=np.concatenate([base.tri_flags, np.full(len(tri), flags, np.uint8)]),
                     textures=base.textures)
    # the library's own OBJ path gives the same scene as the attributes added directly
    lib, ctx = gpu_ctx.lib, gpu_ctx
    h = C.c_void_p()
    ctx.check(lib.bg_scene_create(ctx.h, C.byref(h)))
    try:
        for t in base.textures:
            tt, keep = S.texture_struct(t)
            ctx.check(lib.bg_scene_add_texture(h, C.byref(tt), None))
        for m in base.materials:
            mm = A.bg_material.from_buffer_copy(np.ascontiguousarray(m).tobytes())
            ctx.check(lib.bg_scene_add_material(h, C.byref(mm), None))
        for l in base.lights:
            ll = A.bg_area_light.from_buffer_copy(np.ascontiguousarray(l).tobytes())
            ctx.check(lib.bg_scene_add_area_light(h, C.byref(ll), None))
        bt = np.ascontiguousarray(base.tri, np.float32)
        bm = np.ascontiguousarray(base.tri_mat, np.uint32)
        bl = np.ascontiguousarray(base.tri_light, np.int32)
        bn = np.ascontiguousarray(base.tri_normals, np.float32)
        bu = np.ascontiguousarray(base.tri_uvs, np.float32)
        for a, b, has_n, fl in S.triangle_runs(base):
            ctx.check(lib.bg_scene_add_triangle_mesh(h, bt[a:].ctypes.data, b - a, bm[a:].ctypes.data,
                                                     bl[a:].ctypes.data, bn[a:].ctypes.data if has_n else None,
                                                     bu[a:].ctypes.data, fl))
        n = C.c_size_t()
        ctx.check(lib.bg_scene_add_obj(h, str(path).encode(), xf.ctypes.data, 5, -1, C.byref(n)))
        assert n.value == len(tri)
        st = A.bg_build_stats()
        ctx.check(lib.bg_scene_commit(h, A.BG_BVH_WIDE, C.byref(st)))
        cam = G.camera_struct(sd.camera)
        o = A.bg_render_opts()
        o.spp, o.max_depth, o.rr_threshold, o.mode, o.seed = 16, 4, 1.0, A.BG_MODE_PBRT, 0
        rgb_obj = np.zeros((40, 40, 3), np.float32)
        rs = A.bg_render_stats()
        ctx.check(lib.bg_render(ctx.h, h, C.byref(cam), C.byref(o), rgb_obj.ctypes.data, C.byref(rs)))
    finally:
        lib.bg_scene_destroy(h)
    r, orc, cmp = _pair(gpu_ctx, sd, A.BG_MODE_PBRT, A.BG_BVH_WIDE, 16)
    print(cmp)
    np.testing.assert_array_equal(rgb_obj, r.rgb)
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9
    assert nb < sd.ntri


def test_emitter_with_straddling_vertex_normals_is_refused(gpu_ctx):
    sd = S.cornell(8, 8)
    n = sd.ntri
    normals = np.zeros((n, 9), np.float32)
    normals[n - 1] = [0, 1, 0, 0, -1, 0, 0, -1, 0]  # light triangle: one vertex normal up, two down
    mask = np.zeros(n, bool)
    mask[n - 1] = True
    sd.tri_normals, sd.tri_normal_mask = normals, mask
    with pytest.raises(RuntimeError, match="both sides"):
        G.Scene(gpu_ctx, sd, A.BG_BVH_WIDE)


def test_texture_arguments(gpu_ctx):
    lib, ctx = gpu_ctx.lib, gpu_ctx
    h = C.c_void_p()
    ctx.check(lib.bg_scene_create(ctx.h, C.byref(h)))
    try:
        t, keep = S.texture_struct(S.Texture(kind=0, rgb=np.zeros((32, 48, 3), np.float32)))
        assert lib.bg_scene_add_texture(h, C.byref(t), None) == A.BG_ERR_UNSUPPORTED  # not a power of two
        t.kind = 7
        assert lib.bg_scene_add_texture(h, C.byref(t), None) == A.BG_ERR_INVALID
        t, keep = S.texture_struct(S.Texture(kind=0, rgb=np.ones((8, 16, 3), np.float32)))
        tid = C.c_uint32()
        ctx.check(lib.bg_scene_add_texture(h, C.byref(t), C.byref(tid)))
        assert tid.value == 0
        m = A.bg_material.from_buffer_copy(np.ascontiguousarray(S.material(S.MATTE, kd_texture=3)).tobytes())
        ctx.check(lib.bg_scene_add_material(h, C.byref(m), None))
        tri = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
        mat = np.zeros(1, np.uint32)
        ctx.check(lib.bg_scene_add_triangles(h, tri.ctypes.data, 1, mat.ctypes.data, None))
        assert lib.bg_scene_commit(h, A.BG_BVH_WIDE, None) == A.BG_ERR_INVALID  # texture 2 does not exist
        assert b"unknown texture" in lib.bg_last_error(ctx.h)
    finally:
        lib.bg_scene_destroy(h)


@pytest.mark.parametrize("shape", [(1, 1), (2, 64), (64, 2), (8, 8)])
@pytest.mark.parametrize("wrap", [A.BG_WRAP_REPEAT, A.BG_WRAP_BLACK, A.BG_WRAP_CLAMP])
def test_texture_shapes_and_wrap_modes(gpu_ctx, shape, wrap):
    """Degenerate pyramids (a 1 x 1 image has a single level; 2 x 64 and 64 x 2 reach 1 texel in one
    axis long before the other) under every wrap mode, on the back wall through a UV mapping that
    runs past [0, 1], against the oracle."""
    h, w = shape
    rng = np.random.default_rng(h * 100 + w)
    img = rng.random((h, w, 3)).astype(np.float32)
    sd = S.cornell(32, 32, spp=8, max_depth=3)
    mats = list(sd.materials) + [S.material(S.MATTE, kd_texture=1)]
    sd.materials = np.stack(mats)
    sd.tri_mat = sd.tri_mat.copy()
    sd.tri_mat[4:6] = len(mats) - 1
    sd.tri_uvs = np.tile(np.array([0, 0, 1, 0, 1, 1], np.float32), (sd.ntri, 1))
    sd.textures = [S.Texture(kind=0, rgb=img, wrap=wrap, mapping=A.BG_MAPPING_UV, uv_scale=(2.5, 1.5),
                             uv_delta=(-0.7, 0.3))]
    r, o, cmp = _pair(gpu_ctx, sd, A.BG_MODE_PBRT, A.BG_BVH_WIDE, 8)
    assert r.stats.error_word == 0
    assert cmp["frac_z3"] <= Z3_FRAC
    assert cmp["frac_close"] >= 0.9
