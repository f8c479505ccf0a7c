"""GPU ray casting (LBVH -> compressed 8-wide BVH) against the CPU oracle's
brute-force closest hit / any hit, which uses the same FP32 triangle test.
Contract: primitive ids identical, including ties (equal t go to the lower
primitive index on both sides, whatever the traversal order), hit distances
identical for triangles (same arithmetic) and within 1e-6 relative for
spheres; any-hit flags identical."""
import numpy as np
import pytest
import torch

from lajolla_public_gb300 import gpu, scenes
from oracle import ljo

pytestmark = pytest.mark.gpu


def _soup_with_spheres(seed, n_tris, n_spheres):
    sc = scenes.soup_scene(seed, n_tris)
    rng = np.random.default_rng(seed + 100)
    m = sc.add_material(scenes.lambertian([0.5, 0.5, 0.5]))
    for c, r in zip(rng.uniform(0, 1, (n_spheres, 3)), rng.uniform(0.005, 0.05, n_spheres)):
        sc.add_sphere(c, r, m)
    return sc


def _check_closest(sc, rays, ctx, sphere_start):
    g = gpu.GpuScene(ctx, sc)
    hits = g.trace_closest(torch.from_numpy(rays).cuda()).cpu().numpy()
    t_g, p_g = hits[:, 0], hits[:, 1].view(np.int32)
    o = ljo.OracleScene(sc)
    t_o, p_o, _, _, ties = o.trace_closest(rays, brute=True)
    hit = p_o >= 0
    assert np.array_equal(p_g >= 0, hit), "hit/miss disagreement"
    same = p_g == p_o
    assert same.all(), np.nonzero(~same)[0][:10]
    tri = hit & (p_o < sphere_start)
    np.testing.assert_array_equal(t_g[tri], t_o[tri])
    sph = hit & (p_o >= sphere_start)
    if sph.any():
        np.testing.assert_allclose(t_g[sph], t_o[sph], rtol=1e-6)
    occ_g = g.trace_any(torch.from_numpy(rays).cuda()).cpu().numpy()
    np.testing.assert_array_equal(occ_g, o.trace_any(rays, brute=True))
    return g, hit.mean()


def test_closest_and_any_match_brute_force(ctx):
    sc = _soup_with_spheres(1, 20000, 40)
    rays = scenes.random_rays(2, 100000)
    g, frac = _check_closest(sc, rays, ctx, sc.num_triangles)
    assert 0.05 < frac < 0.95
    info = g.info()
    assert info.num_prims == 20040 and info.num_wide_nodes > 0


@pytest.mark.parametrize("make", [lambda: _soup_with_spheres(1, 20000, 40), lambda: scenes.tied_soup_scene(7, 4000),
                                  lambda: scenes.cornell_box(seed=1)])
def test_bvh_holds_every_primitive_once(ctx, make):
    sc = make()
    g = gpu.GpuScene(ctx, sc)
    leaves = g.leaf_prims()
    n = g.info().num_prims
    assert len(leaves) == n
    assert np.array_equal(np.sort(leaves), np.arange(n, dtype=np.int32))


def test_ties_resolve_to_lowest_index(ctx):
    sc = scenes.tied_soup_scene(7, 4000)
    rays = scenes.random_rays(8, 40000)
    _, p_o, _, _, ties = ljo.OracleScene(sc).trace_closest(rays, brute=True)
    assert (ties > 1).sum() > 1000
    _check_closest(sc, rays, ctx, sc.num_triangles)


def test_segment_rays_and_axis_aligned_directions(ctx):
    sc = _soup_with_spheres(3, 5000, 10)
    rays = scenes.random_rays(4, 20000)
    rng = np.random.default_rng(5)
    rays[:, 3] = rng.uniform(0, 0.5, len(rays))          # tnear
    rays[:, 7] = rays[:, 3] + rng.uniform(0, 2, len(rays))  # finite tfar
    axis = rng.integers(0, 3, 5000)
    rays[:5000, 4:7] = 0.0
    rays[np.arange(5000), 4 + axis] = rng.choice([-1.0, 1.0], 5000)
    rays[-10:, 7] = rays[-10:, 3] * 0.5                    # empty segments
    _check_closest(sc, rays, ctx, sc.num_triangles)


def test_single_triangle_scene_reference_known_answer(ctx):
    """src/tests/intersection.cpp:4-42: triangle (-1,-1,-1) (1,-1,-1) (0,1,-1),
    ray from the origin along -z hits (0, 0, -1)."""
    sc = scenes.Scene(4, 4, 1, 2, np.eye(4), 45.0)
    m = sc.add_material(scenes.lambertian([0.5, 0.5, 0.5]))
    sc.add_mesh(np.array([[-1, -1, -1], [1, -1, -1], [0, 1, -1]], np.float32), np.array([[0, 1, 2]]), m)
    g = gpu.GpuScene(ctx, sc)
    rays = np.array([[0, 0, 0, 0, 0, 0, -1, np.inf]], np.float32)
    h = g.trace_closest(torch.from_numpy(rays).cuda()).cpu().numpy()
    assert h[0, 1].view(np.int32) == 0
    p = rays[0, :3] + rays[0, 4:7] * h[0, 0]
    assert np.linalg.norm(p - np.array([0, 0, -1])) < 1e-3


def test_empty_batch_and_bad_arguments(ctx):
    sc = scenes.soup_scene(1, 100)
    g = gpu.GpuScene(ctx, sc)
    empty = torch.zeros((0, 8), dtype=torch.float32, device="cuda")
    assert g.trace_closest(empty).shape == (0, 4)
    with pytest.raises(gpu.LjError):
        g.ctx.check(gpu.lib().lj_gpu_trace_closest(g.h, None, None, 5, None))


def test_large_soup_properties(ctx):
    """1M-triangle soup (the microbenchmark's triangle distribution): hits
    agree with the CPU oracle's own BVH on a subsample of the rays."""
    sc = scenes.soup_scene(7, 1 << 20)
    g = gpu.GpuScene(ctx, sc)
    rays = scenes.random_rays(8, 1 << 20)
    hits = g.trace_closest(torch.from_numpy(rays).cuda()).cpu().numpy()
    sub = np.arange(0, len(rays), 64)
    o = ljo.OracleScene(sc)
    t_o, p_o, _, _, _ = o.trace_closest(rays[sub], brute=False)
    p_g = hits[sub, 1].view(np.int32)
    agree = (p_g == p_o) | (hits[sub, 0] == t_o)
    assert agree.all()
    np.testing.assert_array_equal(hits[sub, 0][p_o >= 0], t_o[p_o >= 0])


def test_morton_codes_and_sort_order_bit_exact(ctx):
    for n in (1, 2, 777, 300000):
        pos, idx = scenes.triangle_soup(n, n)
        tri = pos[idx].reshape(-1, 9).copy()
        if n > 10:
            tri[5] = tri[3]   # equal codes -> ties resolved by index
        codes, order = ctx.morton_sort(torch.from_numpy(tri).cuda())
        c_o, o_o = ljo.morton(tri)
        np.testing.assert_array_equal(codes.cpu().numpy().view(np.uint32), c_o)
        np.testing.assert_array_equal(order.cpu().numpy().view(np.uint32), o_o)
