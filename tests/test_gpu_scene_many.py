"""Several scenes at once (lj_gpu_scene_create_many): each is the scene one
lj_gpu_scene_create makes -- the same BVH (node counts, leaves, bounds), the
same hits and a bit-identical image -- although their copies, device
builds and host tables ran at the same time; a bad description among them
leaves no scene behind and is named by its index.  The reference constructs
one Scene per scene file (src/scene.cpp:4-53)."""
import copy

import numpy as np
import pytest
import torch

from lajolla_public_gb300 import abi, gpu, scenes

pytestmark = pytest.mark.gpu


def pool():
    return [
        scenes.cornell_box(seed=2, width=48, height=32, spp=4),
        scenes.resized_terrain_scene(seed=1, n_tris=60000, width=40, height=24, spp=2),
        scenes.resized_volume_scene(seed=3, n_tris=5000, width=32, height=32, spp=2, grid=32),
        scenes.soup_scene(4, 30000),
        scenes.with_three_channel_density(scenes.volume_scene(width=16, height=16, spp=2, grid=16)),
    ]


def test_scenes_created_together_equal_scenes_created_alone(ctx):
    scs = pool()
    alone = [gpu.GpuScene(ctx, s) for s in scs]
    together = gpu.create_scenes(ctx, scs)
    rays = torch.from_numpy(scenes.random_rays(7, 20000)).cuda()
    for a, b in zip(alone, together):
        ia, ib = a.info(), b.info()
        for f in ("num_triangles", "num_prims", "num_wide_nodes", "num_binary_nodes", "device_bytes",
                  "bsphere_radius"):
            assert getattr(ia, f) == getattr(ib, f), f
        assert list(ia.bounds_lower) == list(ib.bounds_lower) and list(ia.bounds_upper) == list(ib.bounds_upper)
        # the collapse claims node and leaf-record slots with atomics, so any two
        # builds (together or not) may lay the same tree out in another order;
        # its leaves and every query's answer are the same
        np.testing.assert_array_equal(np.sort(a.leaf_prims()), np.sort(b.leaf_prims()))
        # hit records compared as bits (a miss holds the prim index -1, a NaN as a float)
        assert torch.equal(a.trace_closest(rays).view(torch.int32), b.trace_closest(rays).view(torch.int32))
        assert torch.equal(a.trace_any(rays), b.trace_any(rays))
        if a.scene.width * a.scene.height <= 48 * 32:
            ima, _ = a.render(seed=5)
            imb, _ = b.render(seed=5)
            np.testing.assert_array_equal(ima, imb)
    for g in alone + together:
        g.close()


def test_one_description_twice(ctx):
    # both creations copy the same caller's density grid (8 MB, page-locked
    # for its copy) at once: two equal scenes
    sc = scenes.volume_scene(width=24, height=24, spp=2, grid=128)
    a, b = gpu.create_scenes(ctx, [sc, sc])
    assert a.info().num_wide_nodes == b.info().num_wide_nodes
    np.testing.assert_array_equal(a.render(seed=3)[0], b.render(seed=3)[0])
    a.close()
    b.close()


def test_a_bad_description_keeps_no_scene(ctx):
    scs = pool()[:3]
    bad = copy.deepcopy(scs[1])
    bad.shapes[0]["material_id"] = 1000
    with pytest.raises(gpu.LjError) as e:
        gpu.create_scenes(ctx, [scs[0], bad, scs[2]])
    assert e.value.code == abi.LJ_ERR_INVALID_ARG
    assert "description 1" in str(e.value)
    assert gpu.create_scenes(ctx, []) == []
    # the context still creates scenes as before
    g = gpu.create_scenes(ctx, scs[:1])[0]
    img, _ = g.render(seed=1)
    ref = gpu.GpuScene(ctx, scs[0])
    np.testing.assert_array_equal(img, ref.render(seed=1)[0])
    g.close()
    ref.close()
