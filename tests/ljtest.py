"""Shared helpers for the test suite (fixtures, scenes matching the golden
harness, tolerance checks)."""
import os

import numpy as np

from lajolla_public_gb300 import abi, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def bsdf_params(rec):
    """Golden bsdf record -> packed lj_gpu_bsdf_batch parameters."""
    t = int(rec[0])
    p = rec[1:9]
    if t == abi.LJ_MAT_LAMBERTIAN:
        return t, list(p[0:3]) + [1.0]
    return t, list(p[0:8])


def light_scene(env, to_world):
    """The scene of golden_harness.cpp's `light` mode: quad mesh light, sphere
    light and a rotated envmap (scale 0.5)."""
    sc = scenes.Scene(8, 8, 1, 2, np.eye(4), 45.0)
    m = sc.add_material(scenes.lambertian([0.5, 0.5, 0.5]))
    pos = np.array([[-1, 2, -1], [1, 2, -1], [1, 2.5, 1], [-1, 2, 1.5]], np.float32)
    idx = np.array([[0, 2, 1], [0, 3, 2]], np.int32)
    sc.add_mesh(pos, idx, m, emission=[5, 4, 3])
    sc.add_sphere([2, 1, 0.5], 0.5, m, emission=[2, 3, 4])
    sc.images.append(np.asarray(env, np.float32))
    tw = np.asarray(to_world, np.float64)
    sc.lights.append(dict(kind=abi.LJ_LIGHT_ENVMAP, image_id=0, scale=0.5, to_world=tw,
                          to_local=np.linalg.inv(tw)))
    sc.envmap_light_id = len(sc.lights) - 1
    return sc


def rel_err(a, b, floor):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def emission_queries(g):
    """(light ids, points, normals, view directions) of the light golden's
    samples, with the view direction its harness used: from the reference
    point's side for area lights, the stored "from light" direction for the
    envmap (golden_harness.cpp, mode light)."""
    out = g["outputs"]
    ref = g["inputs"][:, 0:3].astype(np.float64)
    lid = out[:, 0].astype(np.int32)
    pt, nr = out[:, 1:4], out[:, 4:7]
    d = ref - pt
    view = d / np.linalg.norm(d, axis=1, keepdims=True)
    env = lid == 2
    view[env] = nr[env]
    return lid, pt, nr, view


def load_flat(data):
    """scenes.Scene from the flattened descriptor oracle/adapter_check writes
    (the layout its header gives): what the reference's parser made of a
    scene file, as the adapter hands it to the library."""
    import ctypes as C
    assert data[:4] == b"LJF1"
    off = 4

    def take(ctype):
        nonlocal off
        v = ctype.from_buffer_copy(data, off)
        off += C.sizeof(ctype)
        return v

    def arr(dtype, shape):
        nonlocal off
        n = int(np.prod(shape))
        a = np.frombuffer(data, dtype, n, off).reshape(shape).copy()
        off += a.nbytes
        return a

    d = take(abi.lj_scene_desc)
    cam, o = d.camera, d.options
    sc = scenes.Scene(cam.width, cam.height, o.samples_per_pixel, o.max_depth,
                      np.array(cam.cam_to_world[:], np.float64).reshape(4, 4), cam.fov,
                      filter_kind=cam.filter_kind, filter_param=cam.filter_param, rr_depth=o.rr_depth,
                      integrator=o.integrator, vol_path_version=o.vol_path_version,
                      max_null_collisions=o.max_null_collisions, camera_medium=cam.medium_id)
    for _ in range(d.num_shapes):
        s = take(abi.lj_shape_desc)
        has_n, has_uv = arr(np.int32, (2,))
        sh = dict(kind=s.kind, material_id=s.material_id, area_light_id=s.area_light_id,
                  interior_medium_id=s.interior_medium_id, exterior_medium_id=s.exterior_medium_id)
        if s.kind == abi.LJ_SHAPE_MESH:
            sh["positions"] = arr(np.float32, (s.num_vertices, 3))
            sh["indices"] = arr(np.int32, (s.num_triangles, 3))
            sh["normals"] = arr(np.float32, (s.num_vertices, 3)) if has_n else None
            sh["uvs"] = arr(np.float32, (s.num_vertices, 2)) if has_uv else None
        else:
            sh["center"], sh["radius"] = list(s.center), s.radius
        sc.shapes.append(sh)
    for _ in range(d.num_materials):
        m = take(abi.lj_material_desc)
        sc.materials.append(dict(type=m.type, eta=m.eta, tex=[
            dict(kind=t.kind, image_id=t.image_id, value0=list(t.value0), value1=list(t.value1), uscale=t.uscale,
                 vscale=t.vscale, uoffset=t.uoffset, voffset=t.voffset) for t in m.tex]))
    for _ in range(d.num_lights):
        l = take(abi.lj_light_desc)
        sc.lights.append(dict(kind=l.kind, shape_id=l.shape_id, intensity=list(l.intensity), image_id=l.image_id,
                              scale=l.scale, to_world=np.array(l.to_world[:]).reshape(4, 4),
                              to_local=np.array(l.to_local[:]).reshape(4, 4)))
    for _ in range(d.num_images):
        im = take(abi.lj_image_desc)
        sc.images.append(arr(np.float32, (im.height, im.width, im.channels)))

    def volume(v):
        out = dict(kind=v.kind, scale=v.scale, channel_scale=list(v.channel_scale))
        if v.kind == abi.LJ_VOL_CONST:
            out["value"] = list(v.value)
        else:
            out.update(p_min=list(v.p_min), p_max=list(v.p_max),
                       data=arr(np.float32, (v.res[2], v.res[1], v.res[0], v.channels)))
        return out
    for _ in range(d.num_media):
        m = take(abi.lj_medium_desc)
        med = dict(kind=m.kind, phase_kind=m.phase_kind, g=m.g, sigma_a=list(m.sigma_a), sigma_s=list(m.sigma_s))
        med["albedo"] = volume(m.albedo)
        med["density"] = volume(m.density)
        sc.media.append(med)
    sc.envmap_light_id = d.envmap_light_id
    assert off == len(data), (off, len(data))
    return sc
