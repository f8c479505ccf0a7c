"""ORACLE / TEST INFRASTRUCTURE -- not part of the product.

ctypes loader for the C++ restatement of lajolla's path (lj_oracle.cpp, built
into oracle/_build/liblj_oracle.so by `make -C oracle port`).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np

from lajolla_public_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
# LJO_LIB selects another build of the port (e.g. `make asan`'s)
LIB_PATH = os.environ.get("LJO_LIB") or os.path.join(HERE, "_build", "liblj_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build():
    """Compile the port (always) -- the reference build is separate (build_ref)."""
    subprocess.run(["make", "-C", HERE, "-s", "port"], check=True)


def reference_dir():
    """Directory of the reference sources: $LJ_REFERENCE_DIR, else the
    default the oracle Makefile names.  None where no sources are there (the
    reference exists only in the development container)."""
    d = os.environ.get("LJ_REFERENCE_DIR")
    if not d:
        m = re.search(r"^LJ_REFERENCE_DIR \?= *(\S+)", open(os.path.join(HERE, "Makefile")).read(), re.M)
        d = m.group(1) if m else ""
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


def build_ref():
    """Compile the reference renderer + golden harness from the reference
    sources (reference_dir(); development container only)."""
    subprocess.run(["make", "-C", HERE, "-s", "-j8", "ref"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, i64, i32, u64 = C.c_void_p, C.c_int64, C.c_int32, C.c_uint64
        L.ljo_scene_create.restype = vp
        L.ljo_scene_create.argtypes = [C.POINTER(abi.lj_scene_desc)]
        L.ljo_scene_destroy.argtypes = [vp]
        L.ljo_scene_bounds.argtypes = [vp, vp]
        L.ljo_render.argtypes = [vp, C.c_int, u64, C.c_int, C.c_int, C.c_int, C.c_int, vp]
        L.ljo_render_samples.argtypes = [vp, u64, vp, i64, C.c_int, C.c_int, C.c_int, vp]
        L.ljo_trace_closest.argtypes = [vp, vp, vp, i64, C.c_int, vp, C.c_int]
        L.ljo_trace_any.argtypes = [vp, vp, vp, i64, C.c_int, C.c_int]
        L.ljo_morton.argtypes = [vp, i64, vp, vp]
        L.ljo_bsdf_batch.argtypes = [C.c_int, C.c_int, C.c_int] + [vp] * 10 + [i64]
        L.ljo_light_sample_batch.argtypes = [vp, vp, vp, vp, vp, vp, vp, i64]
        L.ljo_phase_batch.argtypes = [C.c_int, C.c_double, vp, vp, vp, vp, vp, vp, i64]
        L.ljo_table1d.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp]
        L.ljo_table2d.argtypes = [vp, C.c_int, C.c_int, vp, C.c_int, vp, vp]
        L.ljo_pcg.argtypes = [u64, u64, C.c_int, vp]
        L.ljo_pcg_keyed.argtypes = [u64, u64, u64, C.c_int, vp]
        L.ljo_mipmap_lookup.argtypes = [vp, C.c_int, C.c_int, vp, i64, vp, vp]
        L.ljo_filter_sample.argtypes = [C.c_int, C.c_double, vp, i64, vp]
        L.ljo_camera_batch.argtypes = [C.POINTER(abi.lj_camera_desc), vp, i64, vp]
        L.ljo_light_emission_batch.argtypes = [vp, vp, vp, vp, vp, i64, vp]
        L.ljo_medium_batch.argtypes = [vp, C.c_int, vp, vp, i64, vp, vp, vp]
        L.ljo_render_job_samples.argtypes = [vp, C.POINTER(abi.lj_camera_desc), u64, C.c_int, C.c_int, C.c_int,
                                             C.c_int, vp, vp, i64, C.c_int, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleScene:
    def __init__(self, scene):
        self.scene = scene
        self._desc, self._keep = scene.desc()
        self.h = lib().ljo_scene_create(C.byref(self._desc))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ljo_scene_destroy(self.h)
            self.h = None

    def bounds(self):
        out = np.zeros(4)
        lib().ljo_scene_bounds(self.h, _p(out))
        return out

    def render(self, mode="keyed", seed=0, spp=0, sample_offset=0, nthreads=0, yx_order=True):
        sc = self.scene
        out = np.zeros((sc.height, sc.width, 3))
        lib().ljo_render(self.h, 0 if mode == "tile" else 1, seed, spp, sample_offset, nthreads,
                         1 if yx_order else 0, _p(out))
        return out

    def render_samples(self, pixels, spp, seed=0, sample_offset=0, nthreads=0):
        pixels = np.ascontiguousarray(pixels, np.int32)
        out = np.zeros((len(pixels), spp, 3))
        lib().ljo_render_samples(self.h, seed, _p(pixels), len(pixels), spp, sample_offset,
                                 nthreads, _p(out))
        return out

    def render_job_samples(self, seed, width, height, max_depth, rr_depth, pixels, samples, nthreads=0):
        """Radiance of (pixel, sample index) keys of a render job at its own
        resolution and depth options (the GPU's keyed samples): (n, 3)."""
        px = np.ascontiguousarray(pixels, np.int32)
        sm = np.ascontiguousarray(samples, np.int32)
        out = np.zeros((len(px), 3))
        lib().ljo_render_job_samples(self.h, C.byref(self._desc.camera), seed, width, height, max_depth, rr_depth,
                                     _p(px), _p(sm), len(px), nthreads, _p(out))
        return out

    def trace_closest(self, rays, brute=False, nthreads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        hits = np.zeros((n, 4), np.float32)
        ties = np.zeros(n, np.int32)
        lib().ljo_trace_closest(self.h, _p(rays), _p(hits), n, 1 if brute else 0, _p(ties), nthreads)
        t = hits[:, 0].copy()
        prim = hits[:, 1].view(np.int32).copy()
        return t, prim, hits[:, 2].copy(), hits[:, 3].copy(), ties

    def trace_any(self, rays, brute=False, nthreads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        occ = np.zeros(len(rays), np.uint8)
        lib().ljo_trace_any(self.h, _p(rays), _p(occ), len(rays), 1 if brute else 0, nthreads)
        return occ

    def light_sample(self, ref_points, rnd):
        ref_points = np.ascontiguousarray(ref_points, np.float32)
        rnd = np.ascontiguousarray(rnd, np.float32)
        n = len(ref_points)
        lid = np.zeros(n, np.int32)
        pt, nr, pdf = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        lib().ljo_light_sample_batch(self.h, _p(ref_points), _p(rnd), _p(lid), _p(pt), _p(nr), _p(pdf), n)
        return lid, pt, nr, pdf

    def light_emission(self, light_ids, view_dirs, points, normals):
        lid = np.ascontiguousarray(light_ids, np.int32)
        v, p, nr = (np.ascontiguousarray(a, np.float64) for a in (view_dirs, points, normals))
        out = np.zeros((len(lid), 3))
        lib().ljo_light_emission_batch(self.h, _p(lid), _p(v), _p(p), _p(nr), len(lid), _p(out))
        return out

    def medium(self, medium_id, points, dirs):
        """(sigma_a, sigma_s, majorant) of a medium, as lj_gpu_medium_batch."""
        p, d = np.ascontiguousarray(points, np.float64), np.ascontiguousarray(dirs, np.float64)
        out = [np.zeros((len(p), 3)) for _ in range(3)]
        lib().ljo_medium_batch(self.h, int(medium_id), _p(p), _p(d), len(p), _p(out[0]), _p(out[1]), _p(out[2]))
        return tuple(out)


def morton(tri_vertices):
    v = np.ascontiguousarray(tri_vertices, np.float32).reshape(-1, 9)
    n = len(v)
    codes = np.zeros(n, np.uint32)
    order = np.zeros(n, np.uint32)
    lib().ljo_morton(_p(v), n, _p(codes), _p(order))
    return codes, order


def bsdf(material_type, op, params, dir_in, dir_out=None, rnd=None, to_view=False):
    params = np.ascontiguousarray(params, np.float32)
    dir_in = np.ascontiguousarray(dir_in, np.float32)
    n = len(dir_in)
    dir_out = np.ascontiguousarray(dir_out if dir_out is not None else np.zeros((n, 3)), np.float32)
    rnd = np.ascontiguousarray(rnd if rnd is not None else np.zeros((n, 3)), np.float32)
    val, pdf, d = np.zeros((n, 3)), np.zeros(n), np.zeros((n, 3))
    eta, rough, valid = np.zeros(n), np.zeros(n), np.zeros(n, np.int32)
    rc = lib().ljo_bsdf_batch(material_type, op, 1 if to_view else 0, _p(params), _p(dir_in),
                              _p(dir_out), _p(rnd), _p(val), _p(pdf), _p(d), _p(eta), _p(rough),
                              _p(valid), n)
    assert rc == 0
    return dict(value=val, pdf=pdf, dir=d, eta=eta, roughness=rough, valid=valid)


def phase(kind, g, dir_in, dir_out, rnd):
    dir_in = np.ascontiguousarray(dir_in, np.float32)
    dir_out = np.ascontiguousarray(dir_out, np.float32)
    rnd = np.ascontiguousarray(rnd, np.float32)
    n = len(dir_in)
    val, pdf, d = np.zeros(n), np.zeros(n), np.zeros((n, 3))
    lib().ljo_phase_batch(kind, g, _p(dir_in), _p(dir_out), _p(rnd), _p(val), _p(pdf), _p(d), n)
    return val, pdf, d


def pcg(stream, seed, k):
    out = np.zeros(k, np.uint32)
    lib().ljo_pcg(stream, seed, k, _p(out))
    return out


def camera_rays(matrix, fov, width, height, filter_kind, filter_param, screen):
    """Primary rays (org, dir) per screen position, as an (n, 6) array."""
    c = abi.lj_camera_desc()
    c.cam_to_world[:] = [float(x) for x in np.asarray(matrix, np.float64).reshape(-1)]
    c.fov, c.width, c.height = float(fov), int(width), int(height)
    c.filter_kind, c.filter_param, c.medium_id = int(filter_kind), float(filter_param), -1
    screen = np.ascontiguousarray(screen, np.float64).reshape(-1, 2)
    out = np.zeros((len(screen), 6))
    lib().ljo_camera_batch(C.byref(c), _p(screen), len(screen), _p(out))
    return out


def mipmap_lookup(img, uvl):
    """Trilinear lookups (n, 3) of the mipmap of img (h, w, 3) at (u, v,
    level) triples; also returns the number of levels."""
    img = np.ascontiguousarray(img, np.float32)
    h, w = img.shape[:2]
    uvl = np.ascontiguousarray(uvl, np.float64).reshape(-1, 3)
    out = np.zeros((len(uvl), 3))
    nl = C.c_int(0)
    lib().ljo_mipmap_lookup(_p(img), w, h, _p(uvl), len(uvl), _p(out), C.byref(nl))
    return out, nl.value


def filter_sample(kind, param, u):
    """Pixel-filter offsets (n, 2) for random pairs u (n, 2)."""
    u = np.ascontiguousarray(u, np.float64).reshape(-1, 2)
    out = np.zeros_like(u)
    lib().ljo_filter_sample(int(kind), float(param), _p(u), len(u), _p(out))
    return out


def pcg_keyed(job_seed, pixel, sample, k):
    out = np.zeros(k, np.uint32)
    lib().ljo_pcg_keyed(job_seed, pixel, sample, k, _p(out))
    return out


def read_pfm(path):
    with open(path, "rb") as f:
        header = f.readline().strip()
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4")
    ch = 3 if header == b"PF" else 1
    # the reference writes rows top to bottom (src/image.cpp:137-149), not
    # in PFM's usual bottom-to-top order
    return data.reshape(h, w, ch).copy()


def run_reference(xml_path, out_pfm, threads=8):
    """Run the reference `lajolla` binary (oracle/_ref/lajolla)."""
    exe = os.path.join(REF_DIR, "lajolla")
    r = subprocess.run([exe, "-t", str(threads), "-o", out_pfm, xml_path],
                       capture_output=True, text=True, cwd=os.path.dirname(xml_path))
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    secs = [float(l.split("Took")[1].split()[0]) for l in r.stdout.splitlines() if "Took" in l]
    return read_pfm(out_pfm), secs
