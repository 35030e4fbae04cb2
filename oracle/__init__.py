"""CPU oracle for the path-tracing hot path - TEST INFRASTRUCTURE ONLY.

A C++ restatement of kazijawad/bonsai's PathIntegrator path (see oracle.cpp) behind ctypes.
Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may use it, as the test oracle.
Parity unpinned: the reference ships no tests or golden vectors and cannot be built here (no Rust
toolchain), so this restatement is pinned only by analytic known answers and by its own fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from bonsai_gb300 import scenes as S
from bonsai_gb300._abi import bg_camera, bg_render_opts

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.orc_scene_create.restype = P
        L.orc_scene_create.argtypes = [P, C.c_int64, P, P, P, C.c_int64, P, C.c_int32, P, C.c_int32, C.c_int32,
                                       P, C.c_int64]
        L.orc_scene_destroy.argtypes = [P]
        L.orc_scene_set_tri_attrs.argtypes = [P, P, P, P, P]
        L.orc_scene_add_texture.restype = C.c_int32
        L.orc_scene_add_texture.argtypes = [P, P]
        L.orc_strat_sample.restype = C.c_int32
        L.orc_strat_sample.argtypes = [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, P]
        L.orc_scene_add_infinite_light.restype = C.c_int32
        L.orc_scene_add_infinite_light.argtypes = [P, P]
        L.orc_bvh_nodes.restype = C.c_int64
        L.orc_bvh_nodes.argtypes = [P]
        L.orc_num_lights.restype = C.c_int64
        L.orc_num_lights.argtypes = [P]
        L.orc_trace.argtypes = [P, P, C.c_int64, C.c_int32, P, P, P, C.c_int32]
        L.orc_render.restype = C.c_int
        L.orc_render.argtypes = [P, C.POINTER(bg_camera), C.POINTER(bg_render_opts), C.c_int32, C.c_int32,
                                 C.c_int32, C.c_int32, C.c_int32, P, P, P, P]
        L.orc_bsdf_sample.argtypes = [P, P, C.c_float, C.c_float, C.c_int32, P]
        L.orc_bsdf_eval.argtypes = [P, P, P, C.c_int32, P]
        L.orc_rng_uniform.restype = C.c_float
        L.orc_rng_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_camera_ray.argtypes = [C.POINTER(bg_camera), C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, P]
        L.orc_philox.argtypes = [P, P, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def camera_struct(cam: S.Camera) -> bg_camera:
    c = bg_camera()
    c.position[:] = cam.position
    c.look_at[:] = cam.look_at
    c.up[:] = cam.up
    c.fov_deg = cam.fov_deg
    c.near_plane = cam.near_plane
    c.far_plane = cam.far_plane
    c.lens_radius = cam.lens_radius
    c.focal_distance = cam.focal_distance
    c.width = cam.width
    c.height = cam.height
    return c


class OracleScene:
    """Scene + reference-layout BVH (faithful or bucket-fixed build)."""

    def __init__(self, sd: S.SceneData, fixed_bvh: bool = True):
        self.sd = sd
        self._keep = [np.ascontiguousarray(sd.tri, np.float32), np.ascontiguousarray(sd.tri_mat, np.uint32),
                      np.ascontiguousarray(sd.tri_light, np.int32), np.ascontiguousarray(sd.spheres),
                      np.ascontiguousarray(sd.materials), np.ascontiguousarray(sd.lights),
                      np.ascontiguousarray(sd.quadrics)]
        t, tm, tl, sp, ma, li, qu = self._keep
        self.h = lib().orc_scene_create(_ptr(t), sd.ntri, _ptr(tm), _ptr(tl), _ptr(sp) if len(sp) else None,
                                        sd.nsph, _ptr(ma), len(ma), _ptr(li) if len(li) else None, len(li),
                                        int(fixed_bvh), _ptr(qu) if len(qu) else None, len(qu))
        if sd.tri_normals is not None or sd.tri_uvs is not None or sd.tri_flags is not None:
            nrm = None if sd.tri_normals is None else np.ascontiguousarray(sd.tri_normals, np.float32)
            mask = None if sd.tri_normal_mask is None else np.ascontiguousarray(sd.tri_normal_mask, np.uint8)
            uvs = None if sd.tri_uvs is None else np.ascontiguousarray(sd.tri_uvs, np.float32)
            fl = None if sd.tri_flags is None else np.ascontiguousarray(sd.tri_flags, np.uint8)
            self._keep += [nrm, mask, uvs, fl]
            lib().orc_scene_set_tri_attrs(self.h, _ptr(nrm), _ptr(mask), _ptr(uvs), _ptr(fl))
        for tex in sd.textures:
            tt, keep = S.texture_struct(tex)
            lib().orc_scene_add_texture(self.h, C.byref(tt))
        if sd.env is not None:
            el, keep = S.env_struct(sd.env)
            if lib().orc_scene_add_infinite_light(self.h, C.byref(el)) != 0:
                raise ValueError("a scene holds at most one infinite light")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_destroy(self.h)
            self.h = None

    @property
    def bvh_nodes(self) -> int:
        return lib().orc_bvh_nodes(self.h)

    def trace(self, rays: np.ndarray, any_hit: bool = False, threads: int = 0, count: bool = False):
        rays = np.ascontiguousarray(rays)
        n = len(rays)
        cnt = np.zeros(2, np.int64) if count else None
        if any_hit:
            occ = np.zeros(n, np.uint8)
            lib().orc_trace(self.h, _ptr(rays), n, 1, None, _ptr(occ), _ptr(cnt), threads)
            return (occ, cnt) if count else occ
        hits = np.zeros(n, S.HIT_DT)
        lib().orc_trace(self.h, _ptr(rays), n, 0, _ptr(hits), None, _ptr(cnt), threads)
        return (hits, cnt) if count else hits

    def render(self, mode: int, spp: int | None = None, seed: int = 0, first_sample: int = 0,
               rows: tuple[int, int, int] | None = None, threads: int = 0, count_traversal: bool = False,
               camera: S.Camera | None = None, max_depth: int | None = None, integrator: int = 0,
               light_strategy: int = 0, sampler: S.StratifiedSampler | None = None):
        """Returns dict(rgb, sum, sumsq, counters).  rows = (y0, y1, ystep) restricts the rendered rows."""
        sd = self.sd
        cam = camera or sd.camera
        c = camera_struct(cam)
        o = bg_render_opts()
        o.spp = spp if spp is not None else sd.spp
        o.max_depth = max_depth if max_depth is not None else sd.max_depth
        o.rr_threshold = sd.rr_threshold
        o.mode = mode
        o.seed = seed
        o.first_sample = first_sample
        o.flags = 0
        o.integrator, o.light_strategy = integrator, light_strategy
        S.set_sampler(o, sampler)
        W, H = cam.width, cam.height
        rgb = np.zeros((H, W, 3), np.float32)
        s1 = np.zeros((H, W, 3), np.float64)
        s2 = np.zeros((H, W, 3), np.float64)
        cnt = np.zeros(7, np.int64)
        y0, y1, ys = rows if rows else (0, H, 1)
        if lib().orc_render(self.h, C.byref(c), C.byref(o), y0, y1, ys, threads, int(count_traversal),
                            _ptr(rgb), _ptr(s1), _ptr(s2), _ptr(cnt)) != 0:
            raise ValueError("the stratified sampler needs spp == x_pixel_samples * y_pixel_samples")
        return {"rgb": rgb, "sum": s1, "sumsq": s2, "counters": cnt, "spp": o.spp}


def bsdf_sample(mat: np.ndarray, wo, u0: float, u1: float, mode: int) -> np.ndarray:
    m = np.ascontiguousarray(mat)
    w = np.asarray(wo, np.float32)
    out = np.zeros(8, np.float32)
    lib().orc_bsdf_sample(_ptr(m), _ptr(w), u0, u1, mode, _ptr(out))
    return out


def bsdf_eval(mat: np.ndarray, wo, wi, mode: int) -> np.ndarray:
    m = np.ascontiguousarray(mat)
    a = np.asarray(wo, np.float32)
    b = np.asarray(wi, np.float32)
    out = np.zeros(4, np.float32)
    lib().orc_bsdf_eval(_ptr(m), _ptr(a), _ptr(b), mode, _ptr(out))
    return out


def rng_uniform(seed: int, pixel: int, sample: int, dim: int) -> float:
    return lib().orc_rng_uniform(seed, pixel, sample, dim)


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox(_ptr(c), _ptr(k), _ptr(out))
    return out


def camera_ray(cam: S.Camera, fx: float, fy: float, tu: float = 0.0, lens=(0.5, 0.5)) -> np.ndarray:
    """(origin, direction) of PerspectiveCamera::generate_ray; `lens` is the lens sample (thin lens)."""
    c = camera_struct(cam)
    out = np.zeros(6, np.float32)
    lib().orc_camera_ray(C.byref(c), fx, fy, tu, lens[0], lens[1], _ptr(out))
    return out


def threads_available() -> int:
    return os.cpu_count() or 1


def strat_sample(sampler: S.StratifiedSampler, mode: int, pixel: int, sample: int, k: int, is2d: bool,
                 seed: int = 0) -> np.ndarray:
    """The stratified sampler's value of stratified dimension k for (pixel, sample): (2,) floats."""
    o = bg_render_opts()
    o.spp, o.mode, o.seed = sampler.spp, mode, seed
    S.set_sampler(o, sampler)
    out = np.zeros(2, np.float32)
    if lib().orc_strat_sample(C.byref(o), pixel, sample, k, int(is2d), _ptr(out)) != 0:
        raise ValueError("not a stratified sampler")
    return out
