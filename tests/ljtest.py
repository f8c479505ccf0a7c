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
