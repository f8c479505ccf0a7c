"""Moved geometry on a resident scene (lj_gpu_scene_update_mesh): after a
refit or a rebuild the BVH answers closest-hit and any-hit queries exactly
like brute force over the new triangles (ids identical except genuine ties,
triangle t bit-identical), and the scene renders bit-identically to a scene
created from the new positions (same hits, bounds, shadow epsilon, emitter
areas and light table).  Embree's counterpart is rtcUpdateGeometryBuffer +
rtcCommitScene; the reference builds its scene once (src/scene.cpp:19-34)."""
import copy

import numpy as np
import pytest
import torch

from lajolla_public_gb300 import abi, gpu, scenes
from oracle import ljo

pytestmark = pytest.mark.gpu


def moved(sc, shape_id, rng, sigma):
    out = copy.deepcopy(sc)
    p = out.shapes[shape_id]["positions"]
    out.shapes[shape_id]["positions"] = (p + rng.normal(0, sigma, p.shape)).astype(np.float32)
    return out


@pytest.mark.parametrize("rebuild", [False, True])
def test_updated_bvh_traces_like_brute_force(ctx, rebuild):
    rng = np.random.default_rng(3)
    sc = scenes.soup_scene(5, 20000)
    g = gpu.GpuScene(ctx, sc)
    for step in range(3):                      # updates compound
        sc = moved(sc, 0, rng, 0.02)
        g.update_mesh(0, sc.shapes[0]["positions"], rebuild=rebuild)
        rays = scenes.random_rays(10 + step, 50000)
        hits = g.trace_closest(torch.from_numpy(rays).cuda()).cpu().numpy()
        occ = g.trace_any(torch.from_numpy(rays).cuda()).cpu().numpy()
        o = ljo.OracleScene(sc)
        t_o, p_o, _, _, ties = o.trace_closest(rays, brute=True)
        p_g = hits[:, 1].view(np.int32)
        assert np.all((p_g == p_o) | (ties > 1)), (step, int(((p_g != p_o) & (ties <= 1)).sum()))
        hit = (p_o >= 0) & (ties <= 1)
        np.testing.assert_array_equal(hits[hit, 0], t_o[hit].astype(np.float32))
        np.testing.assert_array_equal(occ, o.trace_any(rays, brute=True))
    info = g.info()
    lo, hi = np.array(info.bounds_lower), np.array(info.bounds_upper)
    p = sc.shapes[0]["positions"]
    np.testing.assert_array_equal(lo, p.min(axis=0))
    np.testing.assert_array_equal(hi, p.max(axis=0))


@pytest.mark.parametrize("rebuild", [False, True])
def test_updated_scene_renders_like_a_fresh_one(ctx, rebuild):
    """A Cornell box whose light quad and tall box move: the area light's
    triangle areas and power, the scene bounds (shadow epsilon) all change."""
    rng = np.random.default_rng(4)
    sc = scenes.cornell_box(seed=2, width=32, height=32, spp=8)
    g = gpu.GpuScene(ctx, sc)
    light = len(sc.shapes) - 1
    new = copy.deepcopy(sc)
    lp = new.shapes[light]["positions"]
    new.shapes[light]["positions"] = (lp * np.float32([1.6, 1.0, 1.3]) + np.float32([0.1, -0.2, 0.0])).astype(np.float32)
    new = moved(new, 5, rng, 0.05)
    g.update_mesh(light, new.shapes[light]["positions"], rebuild=rebuild)
    g.update_mesh(5, new.shapes[5]["positions"], rebuild=rebuild)
    got, _ = g.render(seed=9)
    want, _ = gpu.GpuScene(ctx, new).render(seed=9)
    np.testing.assert_array_equal(got, want)
    old, _ = gpu.GpuScene(ctx, sc).render(seed=9)
    assert np.abs(old - want).max() > 1e-3


def test_update_with_normals_and_refused_requests(ctx):
    sc = scenes.textured_scene(1, 16, 16, 2, 4)
    g = gpu.GpuScene(ctx, sc)
    mesh = next(i for i, s in enumerate(sc.shapes) if s["kind"] == abi.LJ_SHAPE_MESH and s["normals"] is not None)
    p, n = sc.shapes[mesh]["positions"], sc.shapes[mesh]["normals"]
    g.update_mesh(mesh, p * 1.01, normals=-n)
    sphere = next(i for i, s in enumerate(sc.shapes) if s["kind"] == abi.LJ_SHAPE_SPHERE)
    bad = [dict(shape_id=sphere, positions=p), dict(shape_id=mesh, positions=p[:-1]),
           dict(shape_id=0, positions=sc.shapes[0]["positions"], normals=np.zeros_like(sc.shapes[0]["positions"])),
           dict(shape_id=mesh, positions=np.where(np.arange(p.size).reshape(p.shape) == 4, np.nan, p)),
           dict(shape_id=999, positions=p)]
    for kw in bad:
        with pytest.raises(gpu.LjError) as e:
            g.update_mesh(**kw)
        assert e.value.code == abi.LJ_ERR_INVALID_ARG
    with pytest.raises(gpu.LjError):
        gpu.lib()
        ctx.check(gpu.lib().lj_gpu_scene_update_mesh(g.h, mesh, p.ctypes.data, None, len(p), 7))
