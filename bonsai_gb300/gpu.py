"""Python handle on libbonsai_gpu.so (ctypes over include/bonsai_gpu.h).

Mirrors the reference's integrator surface: a ``Scene`` is built once from shapes, materials and
area lights (BVH::new + Scene::new, src/accelerators/bvh.rs:53-89, src/base/scene.rs:16-33) and a
``PathIntegrator(camera, max_depth, rr_threshold)`` renders it (src/integrators/path.rs:27-39,
SamplerIntegrator::render, src/base/integrator.rs:35-133).  Every call goes through the C ABI;
errors raise ``BonsaiError`` with the library's message.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from . import scenes as S


class BonsaiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{status} ({A.load().bg_status_string(status).decode()}): {msg}")
        self.status = status


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Context:
    """One CUDA device + stream (bg_ctx)."""

    def __init__(self, device: int = 0, max_queue_paths: int = 0, memory_cap_bytes: int = 0):
        self.lib = A.load()
        o = A.bg_device_opts()
        o.device = device
        o.max_queue_paths = max_queue_paths
        o.memory_cap_bytes = memory_cap_bytes
        h = C.c_void_p()
        st = self.lib.bg_create(C.byref(o), C.byref(h))
        if st != A.BG_OK:
            raise BonsaiError(st, "bg_create failed")
        self.h = h
        self._scenes: weakref.WeakSet = weakref.WeakSet()
        self._guides: weakref.WeakSet = weakref.WeakSet()

    def check(self, st: int):
        if st != A.BG_OK:
            raise BonsaiError(st, self.lib.bg_last_error(self.h).decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            for sc in list(getattr(self, "_scenes", [])):
                sc.close()
            for g in list(getattr(self, "_guides", [])):
                g.close()
            self.lib.bg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def flush_l2(self):
        self.check(self.lib.bg_flush_l2(self.h))

    def synchronize(self):
        self.check(self.lib.bg_synchronize(self.h))

    # raw device buffers (for device-resident timing)
    def alloc(self, nbytes: int) -> C.c_void_p:
        p = C.c_void_p()
        self.check(self.lib.bg_device_alloc(self.h, nbytes, C.byref(p)))
        return p

    def free(self, p: C.c_void_p):
        self.check(self.lib.bg_device_free(self.h, p))

    def h2d(self, dst: C.c_void_p, src: np.ndarray):
        self.check(self.lib.bg_memcpy_h2d(self.h, dst, _ptr(src), src.nbytes))

    def d2h(self, dst: np.ndarray, src: C.c_void_p):
        self.check(self.lib.bg_memcpy_d2h(self.h, _ptr(dst), src, dst.nbytes))


class Scene:
    """Device scene (bg_scene) built from a ``scenes.SceneData``."""

    def __init__(self, ctx: Context, sd: S.SceneData, bvh: int = A.BG_BVH_WIDE):
        self.ctx, self.sd, self.layout = ctx, sd, bvh
        lib = ctx.lib
        h = C.c_void_p()
        ctx.check(lib.bg_scene_create(ctx.h, C.byref(h)))
        self.h = h
        ctx._scenes.add(self)
        try:
            for m in sd.materials:
                mm = A.bg_material.from_buffer_copy(np.ascontiguousarray(m).tobytes())
                ctx.check(lib.bg_scene_add_material(h, C.byref(mm), None))
            for l in sd.lights:
                ll = A.bg_area_light.from_buffer_copy(np.ascontiguousarray(l).tobytes())
                ctx.check(lib.bg_scene_add_area_light(h, C.byref(ll), None))
            for t in sd.textures:
                tt, keep = S.texture_struct(t)
                ctx.check(lib.bg_scene_add_texture(h, C.byref(tt), None))
            if sd.env is not None:
                el, keep = S.env_struct(sd.env)
                ctx.check(lib.bg_scene_add_infinite_light(h, C.byref(el)))
            tri = np.ascontiguousarray(sd.tri, np.float32)
            tm = np.ascontiguousarray(sd.tri_mat, np.uint32)
            tl = np.ascontiguousarray(sd.tri_light, np.int32)
            if sd.tri_normals is None and sd.tri_uvs is None and sd.tri_flags is None:
                ctx.check(lib.bg_scene_add_triangles(h, _ptr(tri), sd.ntri, _ptr(tm), _ptr(tl)))
            else:
                nrm = None if sd.tri_normals is None else np.ascontiguousarray(sd.tri_normals, np.float32)
                uvs = None if sd.tri_uvs is None else np.ascontiguousarray(sd.tri_uvs, np.float32)
                for a, b, has_n, fl in S.triangle_runs(sd):
                    ctx.check(lib.bg_scene_add_triangle_mesh(
                        h, tri[a:].ctypes.data, b - a, tm[a:].ctypes.data, tl[a:].ctypes.data,
                        nrm[a:].ctypes.data if has_n else None, uvs[a:].ctypes.data if uvs is not None else None, fl))
            if sd.nsph:
                sp = np.ascontiguousarray(sd.spheres)
                ctx.check(lib.bg_scene_add_spheres(h, _ptr(sp), sd.nsph))
            if len(sd.quadrics):
                qu = np.ascontiguousarray(sd.quadrics)
                ctx.check(lib.bg_scene_add_quadrics(h, _ptr(qu), len(qu)))
            st = A.bg_build_stats()
            ctx.check(lib.bg_scene_commit(h, bvh, C.byref(st)))
        except BaseException:
            self.close()  # a failed build releases what it had allocated
            raise
        self.build_ms, self.nodes, self.bvh = st.build_ms, st.nodes, bvh

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.bg_scene_destroy(self.h)  # safe after bg_destroy: the scene is orphaned
            self.h = None

    def __del__(self):
        self.close()

    def trace(self, rays: np.ndarray, any_hit: bool = False) -> np.ndarray:
        rays = np.ascontiguousarray(rays)
        if any_hit:
            occ = np.zeros(len(rays), np.uint8)
            self.ctx.check(self.ctx.lib.bg_trace_any(self.ctx.h, self.h, _ptr(rays), len(rays), _ptr(occ)))
            return occ
        hits = np.zeros(len(rays), S.HIT_DT)
        self.ctx.check(self.ctx.lib.bg_trace_closest(self.ctx.h, self.h, _ptr(rays), len(rays), _ptr(hits)))
        return hits

    def trace_device(self, d_rays, n: int, d_out, any_hit: bool = False) -> float:
        ms = C.c_float()
        fn = self.ctx.lib.bg_trace_any_device if any_hit else self.ctx.lib.bg_trace_closest_device
        self.ctx.check(fn(self.ctx.h, self.h, d_rays, n, d_out, C.byref(ms)))
        return ms.value


def camera_struct(cam: S.Camera) -> A.bg_camera:
    c = A.bg_camera()
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


@dataclass
class RenderResult:
    rgb: np.ndarray
    stats: A.bg_render_stats


class PathIntegrator:
    """PathIntegrator::new(camera, sampler, max_depth, rr_threshold) rendering on the GPU."""

    integrator = A.BG_INTEGRATOR_PATH
    light_strategy = 0

    def __init__(self, camera: S.Camera, spp: int, max_depth: int, rr_threshold: float = 1.0,
                 mode: int = A.BG_MODE_PBRT, seed: int = 0, sampler: S.StratifiedSampler | None = None):
        self.camera, self.spp, self.max_depth = camera, spp, max_depth
        self.rr_threshold, self.mode, self.seed = rr_threshold, mode, seed
        self.sampler = sampler

    def render(self, scene: Scene, first_sample: int = 0, accumulate: bool = False, readback: bool = True,
               spp: int | None = None, graph: bool = False, stage_timing: bool = False) -> RenderResult:
        ctx = scene.ctx
        c = camera_struct(self.camera)
        o = A.bg_render_opts()
        o.spp = self.spp if spp is None else spp
        o.max_depth = self.max_depth
        o.rr_threshold = self.rr_threshold
        o.mode = self.mode
        o.seed = self.seed
        o.first_sample = first_sample
        o.integrator, o.light_strategy = self.integrator, self.light_strategy
        S.set_sampler(o, self.sampler)
        o.flags = ((A.BG_RENDER_ACCUMULATE if accumulate else 0) | (0 if readback else A.BG_RENDER_NO_READBACK) |
                   (A.BG_RENDER_GRAPH if graph else 0) | (A.BG_RENDER_STAGE_TIMING if stage_timing else 0))
        rgb = np.zeros((self.camera.height, self.camera.width, 3), np.float32) if readback else None
        st = A.bg_render_stats()
        ctx.check(ctx.lib.bg_render(ctx.h, scene.h, C.byref(c), C.byref(o), _ptr(rgb), C.byref(st)))
        return RenderResult(rgb, st)

    def render_guided(self, scene: Scene, guide: "Guide", first_sample: int = 0, accumulate: bool = False,
                      readback: bool = True, spp: int | None = None) -> "GuidedResult":
        """Progressive guided render (bg_render_guided): spp passes of 1 spp, online training."""
        ctx = scene.ctx
        c = camera_struct(self.camera)
        o = A.bg_render_opts()
        o.spp = self.spp if spp is None else spp
        o.max_depth = self.max_depth
        o.rr_threshold = self.rr_threshold
        o.mode = self.mode
        o.seed = self.seed
        o.first_sample = first_sample
        S.set_sampler(o, self.sampler)
        o.flags = (A.BG_RENDER_ACCUMULATE if accumulate else 0) | (0 if readback else A.BG_RENDER_NO_READBACK)
        rgb = np.zeros((self.camera.height, self.camera.width, 3), np.float32) if readback else None
        st = A.bg_render_stats()
        gs = A.bg_guide_stats()
        ctx.check(ctx.lib.bg_render_guided(ctx.h, scene.h, guide.h, C.byref(c), C.byref(o), _ptr(rgb), C.byref(st),
                                           C.byref(gs)))
        return GuidedResult(rgb, st, gs)

    @staticmethod
    def moments(ctx: Context, width: int, height: int):
        s1 = np.zeros((height, width, 3), np.float64)
        s2 = np.zeros((height, width, 3), np.float64)
        n = np.zeros((height, width), np.uint32)
        ctx.check(ctx.lib.bg_film_moments(ctx.h, _ptr(s1), _ptr(s2), _ptr(n)))
        return s1, s2, n


class WhittedIntegrator(PathIntegrator):
    """WhittedIntegrator::new(camera, sampler, max_depth) (src/integrators/whitted.rs:128-136)."""

    integrator = A.BG_INTEGRATOR_WHITTED

    def __init__(self, camera: S.Camera, spp: int, max_depth: int, mode: int = A.BG_MODE_PBRT, seed: int = 0,
                 sampler: S.StratifiedSampler | None = None):
        super().__init__(camera, spp, max_depth, 1.0, mode, seed, sampler)


class DirectLightingIntegrator(PathIntegrator):
    """DirectLightingIntegrator::new(camera, sampler, scene, max_depth, strategy)
    (src/integrators/direct.rs:27-53); strategy = A.BG_LIGHT_UNIFORM_ALL or A.BG_LIGHT_UNIFORM_ONE."""

    integrator = A.BG_INTEGRATOR_DIRECT

    def __init__(self, camera: S.Camera, spp: int, max_depth: int, strategy: int = A.BG_LIGHT_UNIFORM_ALL,
                 mode: int = A.BG_MODE_PBRT, seed: int = 0, sampler: S.StratifiedSampler | None = None):
        super().__init__(camera, spp, max_depth, 1.0, mode, seed, sampler)
        self.light_strategy = strategy


@dataclass
class GuidedResult:
    rgb: np.ndarray
    stats: A.bg_render_stats
    guide: A.bg_guide_stats


class Guide:
    """Guiding network (bg_guide): 78 -> 4 x 64 -> 2 x 41 MLP, two heads of an 8-lobe vMF mixture and
    a selection logit each (continuation head first, then the next-event head)."""

    def __init__(self, ctx: Context, learning_rate: float = 1e-3, batch_size: int = 16384,
                 samples_per_pass: int = 1 << 18, warmup_passes: int = 4, alpha: float = 0.5, seed: int = 0,
                 no_fallback: bool = False, no_train: bool = False, pass_paths: int = 1 << 22, epochs: int = 1,
                 flags: int = 0):
        self.ctx = ctx
        o = A.bg_guide_opts()
        o.learning_rate, o.beta1, o.beta2, o.eps, o.alpha = learning_rate, 0.9, 0.999, 1e-8, alpha
        o.batch_size, o.samples_per_pass, o.warmup_passes = batch_size, samples_per_pass, warmup_passes
        o.flags = (A.BG_GUIDE_NO_FALLBACK if no_fallback else 0) | (A.BG_GUIDE_NO_TRAIN if no_train else 0) | flags
        o.seed = seed
        o.pass_paths, o.epochs = pass_paths, epochs
        self.opts = o
        h = C.c_void_p()
        ctx.check(ctx.lib.bg_guide_create(ctx.h, C.byref(o), C.byref(h)))
        self.h = h
        ctx._guides.add(self)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.bg_guide_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def params(self) -> np.ndarray:
        p = np.zeros(A.BG_GUIDE_PARAMS, np.float32)
        self.ctx.check(self.ctx.lib.bg_guide_get_params(self.h, _ptr(p)))
        return p

    @params.setter
    def params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == A.BG_GUIDE_PARAMS
        self.ctx.check(self.ctx.lib.bg_guide_set_params(self.h, _ptr(p)))

    def set_wait_limit(self, cycles: int):
        """Limit of the network kernels' tensor-core waits in SM cycles (0 = the default, ~1 s)."""
        self.ctx.check(self.ctx.lib.bg_guide_set_wait_limit(self.h, cycles))

    def forward(self, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, A.BG_GUIDE_QUERY_FLOATS)
        out = np.zeros((len(q), A.BG_GUIDE_OUTPUTS), np.float32)
        self.ctx.check(self.ctx.lib.bg_guide_forward(self.h, _ptr(q), len(q), _ptr(out)))
        return out

    def gradient(self, samples: np.ndarray) -> tuple[np.ndarray, float]:
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, A.BG_GUIDE_SAMPLE_FLOATS)
        g = np.zeros(A.BG_GUIDE_PARAMS, np.float32)
        loss = C.c_float()
        self.ctx.check(self.ctx.lib.bg_guide_gradient(self.h, _ptr(s), len(s), _ptr(g), C.byref(loss)))
        return g, loss.value

    def train(self, samples: np.ndarray) -> float:
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, A.BG_GUIDE_SAMPLE_FLOATS)
        loss = C.c_float()
        self.ctx.check(self.ctx.lib.bg_guide_train(self.h, _ptr(s), len(s), C.byref(loss)))
        return loss.value

    def pool(self) -> np.ndarray:
        """Training samples gathered by the last guided render pass (n x 16 floats)."""
        out = np.zeros((self.opts.samples_per_pass, A.BG_GUIDE_SAMPLE_FLOATS), np.float32)
        n = C.c_size_t()
        self.ctx.check(self.ctx.lib.bg_guide_pool(self.h, _ptr(out), len(out), C.byref(n)))
        return out[: n.value]

    def time(self, samples: np.ndarray, queries: np.ndarray, reps: int = 20) -> tuple[float, float]:
        """(ms per training step on one batch, ms per inference pass over the queries), device-timed."""
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, A.BG_GUIDE_SAMPLE_FLOATS)
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, A.BG_GUIDE_QUERY_FLOATS)
        t, i = C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.bg_guide_time(self.h, _ptr(s), len(s), _ptr(q), len(q), reps, C.byref(t), C.byref(i)))
        return t.value, i.value

    def mixture_eval(self, raw: np.ndarray, u: np.ndarray, w: np.ndarray, p_bsdf: np.ndarray) -> np.ndarray:
        """Device evaluation of one head's mixture: raw (n, 41) outputs of a head."""
        raw = np.ascontiguousarray(raw, np.float32).reshape(-1, A.BG_GUIDE_OUTPUTS // 2)
        n = len(raw)
        u = np.ascontiguousarray(u, np.float32).reshape(n, 3)
        w = np.ascontiguousarray(w, np.float32).reshape(n, 3)
        pb = np.ascontiguousarray(p_bsdf, np.float32).reshape(n)
        out = np.zeros((n, 48), np.float32)
        self.ctx.check(self.ctx.lib.bg_guide_mixture_eval(self.h, _ptr(raw), _ptr(u), _ptr(w), _ptr(pb), n, _ptr(out)))
        return out


@dataclass
class BatchJob:
    scene: "Scene"
    camera: S.Camera
    spp: int
    max_depth: int
    rr_threshold: float = 1.0
    seed: int = 0
    first_sample: int = 0
    sampler: S.StratifiedSampler | None = None


def render_batch(ctx: Context, jobs: list, readback: bool = True):
    """Renders every job in one batch (bg_render_batch): paths of all scenes share the wavefront.
    Returns (list of images or None, bg_render_stats)."""
    items = (A.bg_batch_item * len(jobs))()
    outs = []
    for it, j in zip(items, jobs):
        it.scene = j.scene.h
        it.camera = camera_struct(j.camera)
        it.opts.spp, it.opts.max_depth, it.opts.rr_threshold = j.spp, j.max_depth, j.rr_threshold
        it.opts.mode, it.opts.seed, it.opts.first_sample, it.opts.flags = A.BG_MODE_PBRT, j.seed, j.first_sample, 0
        S.set_sampler(it.opts, j.sampler)
        img = np.zeros((j.camera.height, j.camera.width, 3), np.float32) if readback else None
        it.rgb_out = img.ctypes.data if img is not None else None
        outs.append(img)
    st = A.bg_render_stats()
    ctx.check(ctx.lib.bg_render_batch(ctx.h, items, len(jobs), C.byref(st)))
    return outs, st
