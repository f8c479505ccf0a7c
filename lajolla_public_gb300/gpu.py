"""Python binding of liblj_gpu.so (include/lj_gpu.h) -- the GPU hot path.

This is the host-side mirror of the reference's render interface:
  GpuScene(scene)              ~ Scene::Scene (src/scene.cpp:4-53): upload +
                                 device BVH build
  GpuScene.render(...)         ~ Image3 render(const Scene&) (src/render.cpp:155-170)
  GpuScene.trace_closest(...)  ~ rtcIntersect1 per ray (src/intersection.cpp:32)
  GpuScene.trace_any(...)      ~ rtcOccluded1 per ray (src/intersection.cpp:83)
Errors raise LjError (the reference throws fl_exception, src/flexception.h).

There is no CPU fallback: if the CUDA library is missing or no GB300-class
device is present, construction raises.
"""
import ctypes as C
import os
import weakref

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblj_gpu.so")

_lib = None


class LjError(RuntimeError):
    def __init__(self, code, msg, status=None):
        super().__init__("lj_gpu error %d: %s" % (code, msg))
        self.code = code
        self.status = status


def lib():
    """Load liblj_gpu.so (building it first if needed).  Raises if it cannot."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _build
            _build.build()
        L = C.CDLL(LIB_PATH)
        vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
        L.lj_gpu_init.argtypes = [C.c_int, C.POINTER(vp)]
        L.lj_gpu_shutdown.argtypes = [vp]
        L.lj_gpu_last_error.argtypes = [vp]
        L.lj_gpu_last_error.restype = C.c_char_p
        L.lj_gpu_abi_version.argtypes = []
        L.lj_gpu_abi_version.restype = C.c_int
        if L.lj_gpu_abi_version() != abi.LJ_GPU_ABI_VERSION:
            raise LjError(abi.LJ_ERR_UNSUPPORTED, "liblj_gpu.so has ABI version %d, the bindings expect %d"
                          % (L.lj_gpu_abi_version(), abi.LJ_GPU_ABI_VERSION))
        L.lj_gpu_scene_create.argtypes = [vp, C.POINTER(abi.lj_scene_desc), C.POINTER(vp)]
        L.lj_gpu_scene_validate.argtypes = [C.POINTER(abi.lj_scene_desc), C.c_char_p, C.c_int]
        L.lj_gpu_scene_create_many.argtypes = [vp, i32, C.POINTER(C.POINTER(abi.lj_scene_desc)), C.POINTER(vp)]
        L.lj_gpu_scene_destroy.argtypes = [vp]
        L.lj_gpu_scene_update_mesh.argtypes = [vp, i32, vp, vp, i32, i32]
        L.lj_gpu_scene_info.argtypes = [vp, C.POINTER(abi.lj_scene_info)]
        L.lj_gpu_render.argtypes = [vp, C.POINTER(abi.lj_render_params), vp, C.POINTER(abi.lj_stats)]
        L.lj_gpu_render_device.argtypes = [vp, C.POINTER(abi.lj_render_params), vp, vp,
                                           C.POINTER(abi.lj_stats)]
        L.lj_gpu_trace_closest.argtypes = [vp, vp, vp, i64, vp]
        L.lj_gpu_trace_any.argtypes = [vp, vp, vp, i64, vp]
        L.lj_gpu_prim_to_shape.argtypes = [vp, i32, C.POINTER(i32), C.POINTER(i32)]
        L.lj_gpu_morton_sort.argtypes = [vp, vp, i64, vp, vp, vp]
        L.lj_gpu_morton_sort_noalloc.argtypes = [vp, i64, vp, vp, vp]
        L.lj_gpu_trace_counters.argtypes = [vp, vp, i64, i32, C.POINTER(i64), C.POINTER(i64)]
        L.lj_gpu_bsdf_param_count.argtypes = [i32]
        L.lj_gpu_bsdf_batch.argtypes = [vp, C.POINTER(abi.lj_bsdf_batch), i64, vp]
        L.lj_gpu_light_sample_batch.argtypes = [vp, vp, vp, vp, vp, vp, vp, i64, vp]
        L.lj_gpu_phase_batch.argtypes = [vp, i32, C.c_float, vp, vp, vp, vp, vp, vp, i64, vp]
        L.lj_gpu_light_emission_batch.argtypes = [vp, vp, vp, vp, vp, vp, i64, vp]
        L.lj_gpu_camera_ray_batch.argtypes = [vp, vp, vp, vp, i64, vp]
        L.lj_gpu_medium_batch.argtypes = [vp, i32, vp, vp, vp, vp, vp, i64, vp]
        L.lj_gpu_server_start.argtypes = [vp, C.POINTER(abi.lj_server_options), C.POINTER(vp)]
        L.lj_gpu_server_submit.argtypes = [vp, vp, C.POINTER(abi.lj_job_desc), C.POINTER(i64)]
        L.lj_gpu_server_poll.argtypes = [vp, i64, C.POINTER(abi.lj_job_status)]
        L.lj_gpu_server_wait.argtypes = [vp, i64, C.c_double, vp, C.POINTER(abi.lj_job_status)]
        L.lj_gpu_server_cancel.argtypes = [vp, i64]
        L.lj_gpu_server_stats.argtypes = [vp, C.POINTER(abi.lj_server_stats)]
        L.lj_gpu_server_last_error.argtypes = [vp]
        L.lj_gpu_server_last_error.restype = C.c_char_p
        L.lj_gpu_server_stop.argtypes = [vp]
        L.lj_gpu_bvh_leaf_prims.argtypes = [vp, vp, i64, C.POINTER(i64)]
        L.lj_gpu_render_job_device.argtypes = [vp, C.POINTER(abi.lj_job_desc), vp, vp, C.POINTER(abi.lj_stats)]
        L.lj_gpu_server_autotune.argtypes = [vp, C.POINTER(vp), C.POINTER(abi.lj_job_desc), C.POINTER(i32), i32,
                                             C.c_char_p, C.POINTER(abi.lj_server_options)]
        _lib = L
    return _lib


def validate_scene(scene):
    """Checks a scenes.Scene's description the way lj_gpu_scene_create does,
    without a device; raises LjError with the reason if it is invalid."""
    desc, keep = scene.desc()
    buf = C.create_string_buffer(512)
    rc = lib().lj_gpu_scene_validate(C.byref(desc), buf, len(buf))
    if rc != abi.LJ_OK:
        raise LjError(rc, buf.value.decode())


def _ptr(t):
    """Device pointer of a torch tensor (or None)."""
    return None if t is None else C.c_void_p(t.data_ptr())


class Context:
    def __init__(self, device=0):
        self.h = C.c_void_p()
        rc = lib().lj_gpu_init(device, C.byref(self.h))
        if rc != abi.LJ_OK:
            raise LjError(rc, "lj_gpu_init failed (no CUDA device of compute capability >= 10.0?)")
        self.device = device
        self._scenes = weakref.WeakSet()
        self._servers = weakref.WeakSet()

    def check(self, rc):
        if rc != abi.LJ_OK:
            raise LjError(rc, lib().lj_gpu_last_error(self.h).decode())

    def close(self):
        """Destroys the context and every scene still open on it."""
        if self.h:
            for s in list(self._servers):
                s.stop()
            for s in list(self._scenes):
                s.close()
            lib().lj_gpu_shutdown(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stateless batch kernels (torch CUDA tensors in, torch tensors out) --
    def morton_sort(self, tri_vertices, stream=None):
        import torch
        n = tri_vertices.shape[0]
        codes = torch.empty(n, dtype=torch.int32, device=tri_vertices.device)
        order = torch.empty(n, dtype=torch.int32, device=tri_vertices.device)
        self.check(lib().lj_gpu_morton_sort(self.h, _ptr(tri_vertices), n, _ptr(codes), _ptr(order),
                                            stream))
        return codes, order

    def bsdf(self, material_type, op, params, dir_in, dir_out=None, rnd=None, to_view=False, stream=None):
        import torch
        n = dir_in.shape[0]
        dev = dir_in.device
        b = abi.lj_bsdf_batch()
        b.material_type, b.op, b.transport_to_view = material_type, op, 1 if to_view else 0
        out = {}
        b.d_params, b.d_dir_in = params.data_ptr(), dir_in.data_ptr()
        if dir_out is not None:
            b.d_dir_out = dir_out.data_ptr()
        if rnd is not None:
            b.d_rnd = rnd.data_ptr()
        if op == abi.LJ_BSDF_OP_EVAL:
            out["value"] = torch.empty((n, 3), dtype=torch.float32, device=dev)
            b.d_out_value = out["value"].data_ptr()
        elif op == abi.LJ_BSDF_OP_PDF:
            out["pdf"] = torch.empty(n, dtype=torch.float32, device=dev)
            b.d_out_pdf = out["pdf"].data_ptr()
        else:
            out["dir"] = torch.empty((n, 3), dtype=torch.float32, device=dev)
            out["eta"] = torch.empty(n, dtype=torch.float32, device=dev)
            out["roughness"] = torch.empty(n, dtype=torch.float32, device=dev)
            out["valid"] = torch.empty(n, dtype=torch.int32, device=dev)
            b.d_out_dir, b.d_out_eta = out["dir"].data_ptr(), out["eta"].data_ptr()
            b.d_out_roughness, b.d_out_valid = out["roughness"].data_ptr(), out["valid"].data_ptr()
        self.check(lib().lj_gpu_bsdf_batch(self.h, C.byref(b), n, stream))
        return out

    def phase(self, kind, g, dir_in, dir_out, rnd, stream=None):
        import torch
        n = dir_in.shape[0]
        dev = dir_in.device
        val = torch.empty(n, dtype=torch.float32, device=dev)
        pdf = torch.empty(n, dtype=torch.float32, device=dev)
        d = torch.empty((n, 3), dtype=torch.float32, device=dev)
        self.check(lib().lj_gpu_phase_batch(self.h, kind, g, _ptr(dir_in), _ptr(dir_out), _ptr(rnd),
                                            _ptr(val), _ptr(pdf), _ptr(d), n, stream))
        return val, pdf, d


def create_scenes(ctx, scene_list):
    """GpuScenes for several scenes.Scene descriptions at once
    (lj_gpu_scene_create_many: the same scenes as one GpuScene each, their
    copies, device builds and host tables overlapped)."""
    scene_list = list(scene_list)
    n = len(scene_list)
    if not ctx.h:
        raise LjError(abi.LJ_ERR_INVALID_ARG, "context is closed")
    made = [s.desc() for s in scene_list]   # (desc, arrays it points into)
    descs = (C.POINTER(abi.lj_scene_desc) * max(1, n))(*[C.pointer(d) for d, _ in made])
    outs = (C.c_void_p * max(1, n))()
    ctx.check(lib().lj_gpu_scene_create_many(ctx.h, n, descs, outs))
    res = []
    for s, h in zip(scene_list, outs[:n]):
        g = GpuScene.__new__(GpuScene)
        g.ctx, g.scene, g.h = ctx, s, C.c_void_p(h)
        ctx._scenes.add(g)
        res.append(g)
    del made
    return res


class GpuScene:
    """A scene resident on the device (BVH built there)."""

    def __init__(self, ctx, scene):
        self.ctx = ctx
        self.scene = scene
        desc, keep = scene.desc()
        self.h = C.c_void_p()
        if not ctx.h:
            raise LjError(abi.LJ_ERR_INVALID_ARG, "context is closed")
        ctx.check(lib().lj_gpu_scene_create(ctx.h, C.byref(desc), C.byref(self.h)))
        ctx._scenes.add(self)
        del keep

    def close(self):
        # a closed context has already destroyed its scenes
        if self.h and self.ctx.h:
            lib().lj_gpu_scene_destroy(self.h)
        self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update_mesh(self, shape_id, positions, normals=None, rebuild=False):
        """New vertex positions (and normals) of mesh `shape_id`; the BVH is
        refitted (or rebuilt) on the device.  The host-side scene
        description is not changed."""
        pos = np.ascontiguousarray(positions, np.float32)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
        self.ctx.check(lib().lj_gpu_scene_update_mesh(
            self.h, int(shape_id), pos.ctypes.data_as(C.c_void_p),
            None if nrm is None else nrm.ctypes.data_as(C.c_void_p), len(pos),
            abi.LJ_UPDATE_REBUILD if rebuild else abi.LJ_UPDATE_REFIT))

    def info(self):
        inf = abi.lj_scene_info()
        self.ctx.check(lib().lj_gpu_scene_info(self.h, C.byref(inf)))
        return inf

    def render(self, seed=0, spp=0, sample_offset=0, max_paths_in_flight=0):
        """Host-memory render (includes device->host copy).  Returns (image HxWx3 float32, stats)."""
        sc = self.scene
        out = np.zeros((sc.height, sc.width, 3), np.float32)
        p = abi.lj_render_params(seed=seed, spp=spp, sample_offset=sample_offset,
                                 max_paths_in_flight=max_paths_in_flight)
        st = abi.lj_stats()
        self.ctx.check(lib().lj_gpu_render(self.h, C.byref(p), out.ctypes.data_as(C.c_void_p), C.byref(st)))
        return out, st

    def render_device(self, out, seed=0, spp=0, sample_offset=0, max_paths_in_flight=0, stream=None,
                      stats=True, profile=False):
        """Render into a device tensor `out` (H*W*3 float32).  profile=True
        times each kernel class with CUDA events (stats.class_ms)."""
        p = abi.lj_render_params(seed=seed, spp=spp, sample_offset=sample_offset,
                                 max_paths_in_flight=max_paths_in_flight,
                                 flags=abi.LJ_RENDER_PROFILE if profile else 0)
        st = abi.lj_stats() if stats else None
        self.ctx.check(lib().lj_gpu_render_device(self.h, C.byref(p), _ptr(out), stream,
                                                  C.byref(st) if st is not None else None))
        return st

    def leaf_prims(self):
        """Primitive index of every BVH leaf record (int32 array, leaf order)."""
        n = C.c_int64()
        self.ctx.check(lib().lj_gpu_bvh_leaf_prims(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.int32)
        self.ctx.check(lib().lj_gpu_bvh_leaf_prims(self.h, out.ctypes.data_as(C.c_void_p), n.value, C.byref(n)))
        return out

    def render_job_device(self, out, job, stream=None, stats=False):
        """One job (lj_job_desc) through the single-scene renderer into the
        device tensor `out` (H*W*3 float32 at the job's resolution)."""
        st = abi.lj_stats() if stats else None
        self.ctx.check(lib().lj_gpu_render_job_device(self.h, C.byref(job), _ptr(out), stream,
                                                      C.byref(st) if st is not None else None))
        return st

    def trace_closest(self, rays, stream=None):
        """rays: (n, 8) float32 CUDA tensor -> (n, 4) hits (t, prim bits, u, v)."""
        import torch
        n = rays.shape[0]
        hits = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
        self.ctx.check(lib().lj_gpu_trace_closest(self.h, _ptr(rays), _ptr(hits), n, stream))
        return hits

    def trace_any(self, rays, stream=None):
        import torch
        n = rays.shape[0]
        occ = torch.empty(n, dtype=torch.uint8, device=rays.device)
        self.ctx.check(lib().lj_gpu_trace_any(self.h, _ptr(rays), _ptr(occ), n, stream))
        return occ

    def light_sample(self, ref_points, rnd, stream=None):
        import torch
        n = ref_points.shape[0]
        dev = ref_points.device
        lid = torch.empty(n, dtype=torch.int32, device=dev)
        pt = torch.empty((n, 3), dtype=torch.float32, device=dev)
        nr = torch.empty((n, 3), dtype=torch.float32, device=dev)
        pdf = torch.empty(n, dtype=torch.float32, device=dev)
        self.ctx.check(lib().lj_gpu_light_sample_batch(self.h, _ptr(ref_points), _ptr(rnd), _ptr(lid),
                                                       _ptr(pt), _ptr(nr), _ptr(pdf), n, stream))
        return lid, pt, nr, pdf

    def light_emission(self, light_ids, view_dirs, points, normals, stream=None):
        """emission(light, view_dir, footprint, point_on_light) per query
        (int32 ids, (n, 3) float32 tensors) -> (n, 3)."""
        import torch
        out = torch.empty((light_ids.shape[0], 3), dtype=torch.float32, device=light_ids.device)
        self.ctx.check(lib().lj_gpu_light_emission_batch(self.h, _ptr(light_ids), _ptr(view_dirs), _ptr(points),
                                                         _ptr(normals), _ptr(out), light_ids.shape[0], stream))
        return out

    def camera_rays(self, screen, stream=None):
        """sample_primary at (n, 2) screen positions -> (origins, directions)."""
        import torch
        n = screen.shape[0]
        org = torch.empty((n, 3), dtype=torch.float32, device=screen.device)
        d = torch.empty((n, 3), dtype=torch.float32, device=screen.device)
        self.ctx.check(lib().lj_gpu_camera_ray_batch(self.h, _ptr(screen), _ptr(org), _ptr(d), n, stream))
        return org, d

    def medium(self, medium_id, points, dirs, stream=None):
        """(sigma_a, sigma_s) at `points` and the majorant along rays
        (points, dirs) of medium `medium_id`, each (n, 3)."""
        import torch
        n = points.shape[0]
        out = [torch.empty((n, 3), dtype=torch.float32, device=points.device) for _ in range(3)]
        self.ctx.check(lib().lj_gpu_medium_batch(self.h, int(medium_id), _ptr(points), _ptr(dirs), _ptr(out[0]),
                                                 _ptr(out[1]), _ptr(out[2]), n, stream))
        return tuple(out)

    def trace_counters(self, rays, any_hit=False):
        """(nodes fetched, primitives tested) over a batch of rays."""
        nn, npr = C.c_int64(), C.c_int64()
        self.ctx.check(lib().lj_gpu_trace_counters(self.h, _ptr(rays), rays.shape[0], 1 if any_hit else 0,
                                                   C.byref(nn), C.byref(npr)))
        return nn.value, npr.value

    def prim_to_shape(self, prim):
        s, l = C.c_int32(), C.c_int32()
        self.ctx.check(lib().lj_gpu_prim_to_shape(self.h, int(prim), C.byref(s), C.byref(l)))
        return s.value, l.value


def job_desc(seed=0, spp=0, sample_offset=0, width=0, height=0, max_depth=None, rr_depth=None, profile=False,
             count_bvh=False):
    j = abi.lj_job_desc(seed=seed, spp=spp, sample_offset=sample_offset, width=width, height=height,
                        flags=(abi.LJ_RENDER_PROFILE if profile else 0) |
                        (abi.LJ_RENDER_COUNT_BVH if count_bvh else 0))
    if max_depth is not None:
        j.override_depth = 1
        j.max_depth = max_depth
        j.rr_depth = rr_depth if rr_depth is not None else 5
    return j


def server_options(hbm_budget_bytes=0, path_pool=0, block_size=0, max_live_jobs=0, max_queued_jobs=0,
                   waves_per_poll=0, policy=abi.LJ_SCHED_FIFO, use_graphs=True, profile=False,
                   one_shade_kernel=False, tune_objective=abi.LJ_TUNE_BALANCED):
    return abi.lj_server_options(hbm_budget_bytes=hbm_budget_bytes, path_pool=path_pool, block_size=block_size,
                                 max_live_jobs=max_live_jobs, max_queued_jobs=max_queued_jobs,
                                 waves_per_poll=waves_per_poll, policy=policy, use_graphs=1 if use_graphs else 0,
                                 flags=(abi.LJ_SERVER_PROFILE if profile else 0) |
                                 (abi.LJ_SERVER_ONE_SHADE_KERNEL if one_shade_kernel else 0),
                                 tune_objective=tune_objective)


class Server:
    """Continuous-batching render server (lj_gpu_server_*): jobs over
    resident scenes share one pool of wavefront queues."""

    def __init__(self, ctx, options=None):
        self.ctx = ctx
        self.h = C.c_void_p()
        opt = options if options is not None else server_options()
        ctx.check(lib().lj_gpu_server_start(ctx.h, C.byref(opt), C.byref(self.h)))
        self._sizes = {}
        ctx._servers.add(self)

    def check(self, rc):
        if rc != abi.LJ_OK:
            raise LjError(rc, lib().lj_gpu_server_last_error(self.h).decode())

    def submit(self, gscene, job=None, **kw):
        """Queues a render of GpuScene `gscene`; returns the job id."""
        j = job if job is not None else job_desc(**kw)
        jid = C.c_int64()
        self.check(lib().lj_gpu_server_submit(self.h, gscene.h, C.byref(j), C.byref(jid)))
        w = j.width or gscene.scene.width
        h = j.height or gscene.scene.height
        self._sizes[jid.value] = (h, w)
        return jid.value

    def poll(self, jid):
        st = abi.lj_job_status()
        self.check(lib().lj_gpu_server_poll(self.h, jid, C.byref(st)))
        return st

    def wait(self, jid, timeout=-1.0):
        """Blocks until the job ends; returns (image HxWx3 float32, status)."""
        h, w = self._sizes[jid]
        out = np.zeros((h, w, 3), np.float32)
        st = abi.lj_job_status()
        rc = lib().lj_gpu_server_wait(self.h, jid, float(timeout), out.ctypes.data_as(C.c_void_p), C.byref(st))
        if rc != abi.LJ_OK:
            raise LjError(rc, lib().lj_gpu_server_last_error(self.h).decode(), status=st)
        del self._sizes[jid]
        return out, st

    def cancel(self, jid):
        self.check(lib().lj_gpu_server_cancel(self.h, jid))

    def stats(self):
        st = abi.lj_server_stats()
        self.check(lib().lj_gpu_server_stats(self.h, C.byref(st)))
        return st

    def stop(self):
        # a closed context has already stopped its servers
        if self.h and self.ctx.h:
            rc = lib().lj_gpu_server_stop(self.h)
            self.h = C.c_void_p()
            if rc != abi.LJ_OK:
                raise LjError(rc, "server stopped after a device error")
        self.h = C.c_void_p()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop()


def autotune(ctx, gscenes, jobs, job_scene, cache_path=None, options=None):
    """Runs the job mix once per (path pool, block size) candidate and
    returns the options of the fastest (cached in `cache_path`)."""
    opt = options if options is not None else server_options()
    arr = (C.c_void_p * len(gscenes))(*[g.h.value for g in gscenes])
    jd = (abi.lj_job_desc * len(jobs))(*jobs)
    js = (C.c_int32 * len(jobs))(*job_scene)
    ctx.check(lib().lj_gpu_server_autotune(ctx.h, arr, jd, js, len(jobs),
                                           cache_path.encode() if cache_path else None, C.byref(opt)))
    return opt
