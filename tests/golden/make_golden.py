"""Generate the golden fixtures in tests/golden/ from the REFERENCE itself.

Runs in the development container only (needs the reference sources): it
builds oracle/_ref/{lajolla,golden_harness} from the unmodified reference
sources (oracle/Makefile, target `ref`), feeds seeded inputs to the
reference's own functions and renderer, and stores inputs + outputs as small
.npz files.  Tests compare the oracle port and the GPU path against them.

    python tests/golden/make_golden.py
"""
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lajolla_public_gb300 import abi, scenes  # noqa: E402
from oracle import ljo  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "golden_harness")


def harness(mode, inp, extra=()):
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        np.asarray(inp, np.float64).tofile(fi)
        subprocess.run([HARNESS, mode, fi, fo] + list(extra), check=True)
        return np.fromfile(fo, np.float64)


def f32(a):
    return np.asarray(a, np.float32).astype(np.float64)


def hemisphere(rng, n, z_min=0.02):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    v[:, 2] = np.abs(v[:, 2]) + z_min
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def sphere_dirs(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def make_bsdf(rng):
    """Lambertian / RoughPlastic / RoughDielectric (the reference's implemented
    materials), incl. the reference test's own configuration
    (src/tests/materials.cpp:55-185)."""
    recs = []
    n_per = 400
    for t in (0, 1, 2):
        for i in range(n_per):
            kd = rng.uniform(0.05, 0.95, 3)
            ks = rng.uniform(0.05, 0.95, 3)
            rough = rng.uniform(0.01, 1.0)
            eta = rng.uniform(1.1, 2.0)
            if t == 0:
                params = list(kd) + [0, 0, 0, 0, 0]
            else:
                params = list(kd) + list(ks) + [rough, eta]
            wi = hemisphere(rng, 1)[0]
            if t == 2 and i % 3 == 0:
                wi[2] = -wi[2]                      # from inside the dielectric
            if t == 2 and i % 2 == 1:
                wo = sphere_dirs(rng, 1)[0]         # reflection and refraction
            else:
                wo = hemisphere(rng, 1)[0]
            u = rng.uniform(0, 1, 3)
            recs.append([t] + params + list(wi) + list(wo) + list(u))
    # the reference test's setup: dir_in = normalize(0.3, 0.4, 0.5), rnd (0.3, 0.4)
    wi = np.array([0.3, 0.4, 0.5]) / np.linalg.norm([0.3, 0.4, 0.5])
    for t, params in ((0, [0.5, 0.5, 0.5, 0, 0, 0, 0, 0]),
                      (1, [0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.3, 1.5]),
                      (2, [0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.3, 1.5])):
        for w in (0.0, 0.6, 1.0):
            recs.append([t] + params + list(wi) + list(wi[[1, 0, 2]]) + [0.3, 0.4, w])
    recs = f32(np.array(recs))
    recs[:, 0] = np.round(recs[:, 0])
    out = harness("bsdf", recs.reshape(-1)).reshape(len(recs), 13)
    return dict(inputs=recs, outputs=out)


def make_phase(rng):
    n = 600
    g = rng.choice([-0.9, -0.3, 0.0005, 0.3, 0.7, 0.95], n)
    wi, wo = sphere_dirs(rng, n), sphere_dirs(rng, n)
    u = rng.uniform(0, 1, (n, 2))
    recs = f32(np.concatenate([g[:, None], wi, wo, u], axis=1))
    out = harness("phase", recs.reshape(-1)).reshape(n, 5)
    return dict(inputs=recs, outputs=out)


def make_table(rng):
    f1 = np.concatenate([rng.uniform(0, 1, 37), [0.0, 0.0], rng.uniform(0, 5, 11)])
    u1 = np.concatenate([rng.uniform(0, 1, 300), [0.0, 1.0, 0.5]])
    w, h = 24, 12
    f2 = rng.uniform(0, 1, (h, w)) ** 3
    f2[3] = 0.0   # an all-black row
    u2 = rng.uniform(0, 1, (300, 2))
    inp = np.concatenate([[len(f1)], f1, [len(u1)], u1, [w, h], f2.reshape(-1), [len(u2)], u2.reshape(-1)])
    out = harness("table", inp)
    m1, m2 = len(u1), len(u2)
    k = 0
    idx = out[k:k + m1]; k += m1
    pmf = out[k:k + m1]; k += m1
    xy = out[k:k + 2 * m2].reshape(m2, 2); k += 2 * m2
    pdf = out[k:k + m2]
    return dict(f1=f1, u1=u1, f2=f2, u2=u2, idx1=idx, pmf1=pmf, xy2=xy, pdf2=pdf)


def make_pcg():
    streams = [0, 1, 7, 12345, 2 ** 31 - 1]
    k = 16
    inp = np.array([[s, k] for s in streams], np.float64)
    out = harness("pcg", inp.reshape(-1)).reshape(len(streams), 2, k)
    return dict(streams=np.array(streams, np.int64), raw=out[:, 0].astype(np.uint32), real=out[:, 1])


def rotate(angle_deg, axis):
    """src/transform.cpp:21-56."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    s, c = math.sin(math.radians(angle_deg)), math.cos(math.radians(angle_deg))
    m = np.eye(4)
    m[0, 0] = a[0] * a[0] + (1 - a[0] * a[0]) * c
    m[0, 1] = a[0] * a[1] * (1 - c) - a[2] * s
    m[0, 2] = a[0] * a[2] * (1 - c) + a[1] * s
    m[1, 0] = a[0] * a[1] * (1 - c) + a[2] * s
    m[1, 1] = a[1] * a[1] + (1 - a[1] * a[1]) * c
    m[1, 2] = a[1] * a[2] * (1 - c) - a[0] * s
    m[2, 0] = a[0] * a[2] * (1 - c) - a[1] * s
    m[2, 1] = a[1] * a[2] * (1 - c) + a[0] * s
    m[2, 2] = a[2] * a[2] + (1 - a[2] * a[2]) * c
    return m


def light_scene_env(rng):
    ew, eh = 16, 8
    env = (rng.uniform(0, 1, (eh, ew, 3)) ** 2 * 4).astype(np.float32)
    env[2, 5] = [40, 30, 20]
    return env


def make_light(rng):
    env = light_scene_env(rng)
    n = 600
    ref = rng.uniform(-1.5, 1.5, (n, 3))
    ref[:, 1] = rng.uniform(-1, 1.5, n)
    u = rng.uniform(0, 1, (n, 4))
    recs = f32(np.concatenate([ref, u], axis=1))
    eh, ew = env.shape[:2]
    inp = np.concatenate([[ew, eh], env.astype(np.float64).reshape(-1), recs.reshape(-1)])
    out = harness("light", inp).reshape(n, 11)
    return dict(env=env, to_world=rotate(30, [0.2, 1, 0.1]), inputs=recs, outputs=out)


def make_camera(rng):
    m = scenes.look_at([0.3, 1.1, 3.4], [0, 0.9, 0], [0, 1, 0])
    out = {}
    for fk, fp, w, h in ((abi.LJ_FILTER_BOX, 1.0, 64, 48), (abi.LJ_FILTER_TENT, 2.0, 40, 40),
                         (abi.LJ_FILTER_GAUSSIAN, 0.5, 33, 57)):
        s = f32(rng.uniform(0, 1, (200, 2)))
        inp = np.concatenate([m.reshape(-1), [40.0, w, h, fk, fp], s.reshape(-1)])
        o = harness("camera", inp).reshape(-1, 6)
        out["f%d" % fk] = dict(matrix=m, fov=40.0, w=w, h=h, filter=fk, param=fp, screen=s, rays=o)
    flat = {}
    for k, v in out.items():
        for kk, vv in v.items():
            flat[k + "_" + kk] = np.asarray(vv)
    return flat


def make_medium(rng):
    """get_sigma_a / get_sigma_s / get_majorant (src/medium.cpp:27-37) of two
    heterogeneous media over grid volumes read by the reference's .vol loader
    (src/volume.cpp:6-104) from files written by scenes.write_vol, and one
    homogeneous medium.  Medium 0: a one-channel density grid (the loader
    repeats it into three channels) with scale s0 and a constant albedo;
    medium 1: a three-channel density grid with scale s1 and a three-channel
    albedo grid on a box of its own.  Half the points fill a box larger than
    the grids' (many fall outside: zero density), half a box mostly inside
    them; directions are uniform on the
    sphere, and each majorant is taken along the ray (point, direction)."""
    grids = {
        "d1": dict(data=f32(rng.uniform(0.1, 3.0, (6, 5, 7, 1))), p_min=f32([-0.6, -0.3, -0.4]),
                   p_max=f32([0.7, 0.5, 0.9])),
        "d3": dict(data=f32(rng.uniform(0.1, 3.0, (4, 6, 5, 3))), p_min=f32([-0.5, -0.6, -0.5]),
                   p_max=f32([0.6, 0.4, 0.3])),
        "a3": dict(data=f32(rng.uniform(0.1, 0.95, (5, 4, 4, 3))), p_min=f32([-0.7, -0.5, -0.6]),
                   p_max=f32([0.5, 0.6, 0.5])),
    }
    s0, s1 = 2.5, 0.75   # exact in FP32, the type lj_volume_desc.scale has
    albedo0 = f32(rng.uniform(0.2, 0.9, 3))
    sigma_a, sigma_s = f32(rng.uniform(0.1, 2.0, 3)), f32(rng.uniform(0.1, 2.0, 3))
    n = 800
    pts = f32(np.concatenate([rng.uniform(-1.0, 1.0, (n // 2, 3)), rng.uniform(-0.5, 0.5, (n - n // 2, 3))]))
    dirs = f32(sphere_dirs(rng, n))
    header = np.concatenate([[s0, s1], albedo0, sigma_a, sigma_s])
    with tempfile.TemporaryDirectory() as d:
        paths = []
        for k in ("d1", "d3", "a3"):
            paths.append(os.path.join(d, k + ".vol"))
            scenes.write_vol(paths[-1], grids[k]["data"], grids[k]["p_min"], grids[k]["p_max"])
        out = harness("medium", np.concatenate([header, np.concatenate([pts, dirs], 1).reshape(-1)]), paths)
    out = out.reshape(n, 3, 9)
    flat = dict(points=pts, dirs=dirs, s0=s0, s1=s1, albedo0=albedo0, sigma_a=sigma_a, sigma_s=sigma_s,
                outputs=out)
    for k, g in grids.items():
        for kk, vv in g.items():
            flat[k + "_" + kk] = vv
    return flat


def medium_scene(g):
    """A scene holding the three media of the `medium` golden (a single
    triangle and no lights: only the media are queried)."""
    sc = scenes.Scene(8, 8, 1, 2, np.eye(4), 45.0, integrator=abi.LJ_INTEGRATOR_VOLPATH, vol_path_version=6)
    m = sc.add_material(scenes.lambertian([0.5, 0.5, 0.5]))
    sc.add_mesh(np.array([[5, 5, 5], [6, 5, 5], [5, 6, 5]], np.float32), np.array([[0, 1, 2]]), m)

    def grid(k, scale=1.0):
        return dict(kind=abi.LJ_VOL_GRID, data=g[k + "_data"], p_min=list(g[k + "_p_min"]),
                    p_max=list(g[k + "_p_max"]), scale=float(scale))
    sc.media.append(dict(kind=abi.LJ_MEDIUM_HETEROGENEOUS, phase_kind=abi.LJ_PHASE_HG, g=0.3,
                         albedo=dict(kind=abi.LJ_VOL_CONST, value=list(g["albedo0"])),
                         density=grid("d1", g["s0"])))
    sc.media.append(dict(kind=abi.LJ_MEDIUM_HETEROGENEOUS, phase_kind=abi.LJ_PHASE_HG, g=0.3,
                         albedo=grid("a3"), density=grid("d3", g["s1"])))
    sc.media.append(dict(kind=abi.LJ_MEDIUM_HOMOGENEOUS, phase_kind=abi.LJ_PHASE_ISOTROPIC,
                         sigma_a=list(g["sigma_a"]), sigma_s=list(g["sigma_s"])))
    return sc


def mixed_scene(seed, w, h, spp, max_depth):
    """Cornell box whose boxes are RoughPlastic / RoughDielectric, plus a
    sphere light: exercises every implemented reference material."""
    sc = scenes.cornell_box(seed=seed, width=w, height=h, spp=spp, max_depth=max_depth)
    sc.materials[5] = scenes.roughplastic([0.6, 0.3, 0.2], [0.8, 0.8, 0.8], 0.2, 1.5)
    sc.materials[6] = scenes.roughdielectric([0.9, 0.9, 0.9], [0.95, 0.9, 0.85], 0.15, 1.45)
    # lift the glass box off the floor: a bottom face coplanar with the floor
    # would make which of the two a refracted ray hits depend on the last
    # bits of its direction (FP32 on the GPU, FP64 in the oracle)
    sc.shapes[6]["positions"] = sc.shapes[6]["positions"] + np.float32([0, 1e-3, 0])
    m = sc.add_material(scenes.lambertian([0.2, 0.7, 0.3]))
    sc.add_sphere([0.55, 1.45, -0.45], 0.12, m, emission=[6, 8, 10])
    return sc


RENDER_CASES = {
    "cbox": lambda: scenes.cornell_box(seed=1, width=40, height=32, spp=16, max_depth=6),
    "cbox_rr": lambda: scenes.cornell_box(seed=2, width=24, height=24, spp=8, max_depth=-1),
    "mixed": lambda: mixed_scene(3, 32, 32, 16, 8),
    # image and checkerboard textures, vertex normals, UVs; the reference's
    # Disney materials are stubs, so this path case has none
    "textured": lambda: scenes.textured_scene(4, 40, 32, 16, 6, clearcoat=False),
    # a rotated HDR envmap (miss-path emission, table_dist sampling) beside a
    # quad light, over Lambertian and RoughPlastic surfaces
    "envmap": lambda: scenes.envmap_scene(5, 40, 32, 16, 6),
}

# aux_render (src/render.cpp:12-69), one case per auxiliary integrator
AUX_CASES = {
    name: (lambda integ=integ: scenes.textured_scene(5, 48, 40, 1, 6, integrator=integ))
    for name, integ in (("depth", abi.LJ_INTEGRATOR_DEPTH), ("shading_normal", abi.LJ_INTEGRATOR_SHADING_NORMAL),
                        ("mean_curvature", abi.LJ_INTEGRATOR_MEAN_CURVATURE),
                        ("ray_differential", abi.LJ_INTEGRATOR_RAY_DIFFERENTIAL),
                        ("mipmap_level", abi.LJ_INTEGRATOR_MIPMAP_LEVEL))
}


def make_renders(cases=RENDER_CASES):
    out = {}
    for name, mk in cases.items():
        sc = mk()
        with tempfile.TemporaryDirectory() as d:
            xml = sc.write_mitsuba(d, name)
            img, _ = ljo.run_reference(xml, os.path.join(d, "out.pfm"), threads=8)
        out[name] = img.astype(np.float32)
    return out


# The reference's own scene files, parsed by the reference's parser and
# flattened by the adapter (lajolla_public_gb300/adapter) as a lajolla build
# with the GPU path would: file under scenes/, and the reduced resolution
# and sample count of the fixture.
REF_SCENES = {
    "cbox": ("cbox/cbox.xml", 128, 128, 64),
    "veach_mi": ("veach_mi/mi.xml", 192, 128, 64),
    "pixel_filter": ("pixel_filter_test/pixel_filter_test.xml", 160, 120, 64),
}
ADAPTER = os.path.join(ROOT, "oracle", "_ref", "adapter_check")


def reference_scene_variant(rel, w, h, spp, directory):
    """The reference's scene file with another film size and sample count,
    written into `directory`; relative file names point back at the
    original's directory."""
    import re
    src = os.path.join(ljo.reference_dir(), "scenes", rel)
    xml = open(src).read()
    for name, v in (("width", w), ("height", h), ("sampleCount", spp)):
        xml = re.sub(r'(<integer name="%s" value=")\d+' % name, r"\g<1>%d" % v, xml)
    base = os.path.dirname(src)
    xml = re.sub(r'value="((?!/)[^"]+\.(?:obj|ply|serialized|exr|hdr|png|jpg|tga|vol))"',
                 lambda m: 'value="%s"' % os.path.join(base, m.group(1)), xml)
    out = os.path.join(directory, os.path.basename(rel))
    open(out, "w").write(xml)
    return out


def flatten_reference_scene(xml):
    """adapter_check flatten: the flattened descriptor's bytes."""
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "scene.flat")
        subprocess.run([ADAPTER, "flatten", xml, f], check=True, capture_output=True)
        return open(f, "rb").read()


def make_refscenes():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s", "-j8", "adapter"], check=True)
    out = {}
    for name, (rel, w, h, spp) in REF_SCENES.items():
        with tempfile.TemporaryDirectory() as d:
            xml = reference_scene_variant(rel, w, h, spp, d)
            out[name + "_flat"] = np.frombuffer(flatten_reference_scene(xml), np.uint8)
            img, _ = ljo.run_reference(xml, os.path.join(d, "out.pfm"), threads=8)
        out[name + "_render"] = img.astype(np.float32)
    return out


def main(which=()):
    """Regenerates every fixture, or only those named (e.g. `medium renders`):
    the functions share one seeded stream in a fixed order, so each fixture
    comes out the same whichever subset is written."""
    ljo.build_ref()
    rng = np.random.default_rng(20261203)
    makers = [("bsdf", lambda: make_bsdf(rng)), ("phase", lambda: make_phase(rng)),
              ("table", lambda: make_table(rng)), ("pcg", make_pcg), ("light", lambda: make_light(rng)),
              ("camera", lambda: make_camera(rng)), ("renders", make_renders),
              ("aux", lambda: make_renders(AUX_CASES)),
              ("medium", lambda: make_medium(np.random.default_rng(20261204))),
              ("refscenes", make_refscenes)]
    for name, mk in makers:
        data = mk()
        if not which or name in which:
            np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main(sys.argv[1:])
