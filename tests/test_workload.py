"""The benchmark workload's generators (CPU): the serving scene pool holds
Cornell-box, terrain and volumetric scenes in turn with triangle counts in
the stated range, and the job stream is deterministic per seed with
arrival times, resolutions, spp and depths from the stated sets."""
import numpy as np

from lajolla_public_gb300 import abi, scenes


def test_serving_scene_pool():
    pool = scenes.serving_scenes(0, 6, volume_grid=16)
    assert len(pool) == 6
    for k, sc in enumerate(pool):
        assert 9000 <= sc.num_triangles <= 2_100_000, (k, sc.num_triangles)
        if k % 3 == 2:
            assert sc.integrator == abi.LJ_INTEGRATOR_VOLPATH and sc.vol_path_version == 6
            dens = sc.media[0]["density"]
            assert dens["data"].shape == (16, 16, 16, 1)
            assert list(dens["channel_scale"]) == [np.float32(1.05), np.float32(0.9), np.float32(0.8)]
            assert abs(float(dens["data"].max()) - 20.0) < 1e-4
        else:
            assert sc.integrator == abi.LJ_INTEGRATOR_PATH
    # the terrain scenes are lit by an envmap, the Cornell boxes by an area light
    assert pool[1].envmap_light_id >= 0 and pool[0].envmap_light_id < 0


def test_serving_jobs_are_deterministic_and_in_range():
    a = scenes.serving_jobs(seed=1000, n_jobs=32, n_scenes=6, rate=200.0)
    b = scenes.serving_jobs(seed=1000, n_jobs=32, n_scenes=6, rate=200.0)
    assert a == b
    t = [j["arrival_s"] for j in a]
    assert t[0] == 0.0 and all(x <= y for x, y in zip(t, t[1:]))
    assert 0.05 < t[-1] < 0.5   # 31 gaps of mean 5 ms
    for j in a:
        assert j["width"] == j["height"] and j["width"] in (128, 256, 512, 1024)
        assert j["spp"] in (4, 16, 64, 256)
        assert 6 <= j["max_depth"] <= 64 and j["rr_depth"] == 5
        assert 0 <= j["scene"] < 6
    assert scenes.serving_jobs(seed=1001, n_jobs=32, n_scenes=6) != a


def test_three_channel_form_of_a_one_channel_grid():
    sc = scenes.volume_scene(width=8, height=8, spp=1, grid=8, max_depth=4)
    d1 = sc.media[0]["density"]["data"].copy()
    cs = np.asarray(sc.media[0]["density"]["channel_scale"], np.float32)
    sc3 = scenes.with_three_channel_density(sc)
    d3 = sc3.media[0]["density"]["data"]
    assert d3.shape == d1.shape[:3] + (3,)
    np.testing.assert_array_equal(d3, (d1 * cs).astype(np.float32))
    assert sc3.media[0]["density"]["channel_scale"] is None
