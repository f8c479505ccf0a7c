"""The continuous-batching render server (lj_gpu_server_*).

Contract: a job's image is the mean of the same keyed samples the
single-scene renderer traces (PCG keyed on seed, pixel, sample), summed in
64-bit fixed point; so (1) it equals lj_gpu_render's image to FP32
summation rounding (rtol 1e-5) -- except that the two renderers may run
kernel instances compiled for different material sets, whose last-bit
rounding can flip a rare Russian-roulette decision, so at most 0.2% of the
pixels (at least one) may differ -- and (2) it is bit-identical whether the
job runs alone or beside other jobs, with CUDA graphs or plain launches,
under either scheduling policy and any block size."""
import numpy as np
import pytest

from golden import make_golden
from lajolla_public_gb300 import abi, gpu, scenes

pytestmark = pytest.mark.gpu


def small_opts(**kw):
    kw.setdefault("path_pool", 1 << 18)
    return gpu.server_options(**kw)


def assert_matches_plain(img, ref, rtol=1e-5, atol=1e-6):
    close = np.isclose(img, ref, rtol=rtol, atol=atol).all(axis=2)
    bad = int((~close).sum())
    assert bad <= max(1, int(0.002 * close.size)), (bad, close.size)


def render_alone(ctx, gscene, opts=None, **job):
    with gpu.Server(ctx, opts or small_opts()) as srv:
        jid = srv.submit(gscene, **job)
        img, st = srv.wait(jid, timeout=120)
    return img, st


def test_single_job_matches_plain_render(ctx):
    sc = scenes.cornell_box(seed=3, width=64, height=48, spp=16, max_depth=6)
    g = gpu.GpuScene(ctx, sc)
    ref, _ = g.render(seed=9)
    img, st = render_alone(ctx, g, seed=9)
    assert st.state == abi.LJ_JOB_DONE and st.samples_total == 64 * 48 * 16
    assert st.samples_dropped == 0
    assert_matches_plain(img, ref, atol=1e-7)
    assert st.finish_ms >= st.admit_ms >= st.submit_ms


def test_textured_and_glossy_scenes_match_plain_render(ctx):
    for case in ("mixed", "textured"):
        sc = make_golden.RENDER_CASES[case]()
        g = gpu.GpuScene(ctx, sc)
        ref, _ = g.render(seed=4, spp=8)
        img, _ = render_alone(ctx, g, seed=4, spp=8)
        assert_matches_plain(img, ref)


def test_resolution_and_depth_overrides(ctx):
    base = scenes.cornell_box(seed=5, width=64, height=64, spp=4, max_depth=6)
    g = gpu.GpuScene(ctx, base)
    img, _ = render_alone(ctx, g, seed=2, width=40, height=24, max_depth=3, rr_depth=2)
    other = scenes.cornell_box(seed=5, width=40, height=24, spp=4, max_depth=3, rr_depth=2)
    ref, _ = gpu.GpuScene(ctx, other).render(seed=2)
    assert_matches_plain(img, ref, atol=1e-7)


@pytest.mark.parametrize("case", ["homogeneous_dielectric", "heterogeneous_sphere"])
def test_volpath_job_matches_plain_render(ctx, case):
    sc = {"homogeneous_dielectric": lambda: scenes.homogeneous_box_scene(width=32, height=24, spp=8,
                                                                         index_matched=False),
          "heterogeneous_sphere": lambda: scenes.volume_scene(width=32, height=32, spp=4, grid=32,
                                                              max_depth=24)}[case]()
    g = gpu.GpuScene(ctx, sc)
    ref, _ = g.render(seed=11)
    img, st = render_alone(ctx, g, seed=11)
    assert st.state == abi.LJ_JOB_DONE and st.samples_total == sc.width * sc.height * sc.spp
    assert_matches_plain(img, ref)


@pytest.mark.parametrize("kind", ["path", "volpath"])
def test_render_job_device_traces_the_server_jobs_samples(ctx, kind):
    """lj_gpu_render_job_device with resolution and depth overrides renders
    the same image as a server job of that description."""
    import torch
    sc = (scenes.cornell_box(seed=7, width=48, height=48, spp=4, max_depth=8) if kind == "path" else
          scenes.homogeneous_box_scene(width=48, height=48, spp=4, index_matched=False))
    g = gpu.GpuScene(ctx, sc)
    job = dict(seed=21, spp=8, width=40, height=24, max_depth=5, rr_depth=3)
    img, _ = render_alone(ctx, g, **job)
    out = torch.zeros(24 * 40 * 3, dtype=torch.float32, device="cuda")
    st = g.render_job_device(out, gpu.job_desc(**job), stats=True)
    torch.cuda.synchronize()
    assert st.samples == 40 * 24 * 8
    assert_matches_plain(img, out.cpu().numpy().reshape(24, 40, 3))


def _mix(ctx):
    gs = [gpu.GpuScene(ctx, scenes.cornell_box(seed=s, width=w, height=h, spp=4, max_depth=d))
          for s, w, h, d in ((1, 32, 32, 6), (2, 80, 40, 4), (3, 48, 64, 8), (4, 16, 16, -1))]
    gs.append(gpu.GpuScene(ctx, make_golden.RENDER_CASES["mixed"]()))
    # Disney materials and an envmap: the other shade kernel instance
    gs.append(gpu.GpuScene(ctx, scenes.resized_terrain_scene(seed=3, n_tris=20000, width=48, height=32, spp=4,
                                                             env_size=(64, 32))))
    # volumetric path jobs: the third path class
    gs.append(gpu.GpuScene(ctx, scenes.homogeneous_box_scene(width=24, height=24, spp=4, index_matched=True)))
    rng = np.random.default_rng(0)
    jobs = []
    for k in range(14):
        gi = int(rng.integers(len(gs)))
        jobs.append((gi, dict(seed=int(rng.integers(1 << 30)), spp=int(rng.choice([1, 4, 16])))))
    return gs, jobs


def test_job_is_identical_alone_and_in_the_mix(ctx):
    gs, jobs = _mix(ctx)
    target = (2, dict(seed=12345, spp=16))
    alone, _ = render_alone(ctx, gs[target[0]], **target[1])
    with gpu.Server(ctx, small_opts()) as srv:
        ids = []
        for k, (gi, j) in enumerate(jobs):
            ids.append(srv.submit(gs[gi], **j))
            if k == 5:
                tid = srv.submit(gs[target[0]], **target[1])
        mixed, st = srv.wait(tid, timeout=120)
        outs = [srv.wait(i, timeout=120)[0] for i in ids]
        stats = srv.stats()
    assert np.array_equal(alone, mixed)
    assert stats.jobs_done == len(jobs) + 1 and stats.jobs_failed == 0
    # every job of the mix equals its plain render
    for (gi, j), img in zip(jobs, outs):
        ref, _ = gs[gi].render(seed=j["seed"], spp=j["spp"])
        assert_matches_plain(img, ref)


@pytest.mark.parametrize("opts", [dict(use_graphs=False), dict(policy=abi.LJ_SCHED_SRPT),
                                  dict(block_size=64), dict(block_size=256, path_pool=1 << 16),
                                  dict(waves_per_poll=2)])
def test_launch_modes_and_policies_give_identical_images(ctx, opts):
    gs, jobs = _mix(ctx)
    jobs = jobs[:6]

    def run(o):
        with gpu.Server(ctx, small_opts(**o)) as srv:
            ids = [srv.submit(gs[gi], **j) for gi, j in jobs]
            return [srv.wait(i, timeout=120)[0] for i in ids]

    a, b = run({}), run(opts)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_cancel_and_reuse(ctx):
    big = gpu.GpuScene(ctx, scenes.cornell_box(seed=1, width=256, height=256, spp=1024))
    small = gpu.GpuScene(ctx, scenes.cornell_box(seed=2, width=16, height=16, spp=4))
    with gpu.Server(ctx, small_opts()) as srv:
        jid = srv.submit(big, seed=1)
        srv.cancel(jid)
        with pytest.raises(gpu.LjError) as e:
            srv.wait(jid, timeout=120)
        assert e.value.code == abi.LJ_ERR_CANCELLED
        assert e.value.status.state == abi.LJ_JOB_CANCELLED
        img, st = srv.wait(srv.submit(small, seed=3), timeout=120)
        ref, _ = small.render(seed=3)
        assert_matches_plain(img, ref, atol=1e-7)
        assert srv.stats().jobs_cancelled == 1


def test_admission_limits(ctx):
    big = gpu.GpuScene(ctx, scenes.cornell_box(seed=1, width=256, height=256, spp=1024))
    with gpu.Server(ctx, small_opts(max_live_jobs=1, max_queued_jobs=1)) as srv:
        a = srv.submit(big, seed=1)
        st = srv.poll(a)
        assert st.state in (abi.LJ_JOB_QUEUED, abi.LJ_JOB_RUNNING)
        ids = [a]
        with pytest.raises(gpu.LjError) as e:
            for k in range(3):   # the second or third waits for the single job slot
                ids.append(srv.submit(big, seed=2 + k))
        assert e.value.code == abi.LJ_ERR_QUEUE_FULL
        for i in ids:
            srv.cancel(i)
    # a budget below the path pool alone is refused at start
    with pytest.raises(gpu.LjError) as e:
        gpu.Server(ctx, small_opts(hbm_budget_bytes=1 << 20))
    assert e.value.code == abi.LJ_ERR_OUT_OF_MEMORY
    # a job larger than what the budget leaves is refused at submit
    with gpu.Server(ctx, small_opts(path_pool=1 << 16, hbm_budget_bytes=64 << 20)) as srv:
        huge = gpu.GpuScene(ctx, scenes.cornell_box(seed=1, width=4096, height=4096, spp=1))
        with pytest.raises(gpu.LjError) as e:
            srv.submit(huge, seed=1)
        assert e.value.code == abi.LJ_ERR_OUT_OF_MEMORY


def test_bad_requests(ctx):
    vol_sc = scenes.homogeneous_box_scene(width=8, height=8, spp=1)
    vol_sc.vol_path_version = 3   # volpath versions 1-5 are not served
    vol = gpu.GpuScene(ctx, vol_sc)
    cb = gpu.GpuScene(ctx, scenes.cornell_box(seed=1, width=8, height=8, spp=1))
    with gpu.Server(ctx, small_opts()) as srv:
        with pytest.raises(gpu.LjError) as e:
            srv.submit(vol, seed=1)
        assert e.value.code == abi.LJ_ERR_UNSUPPORTED
        with pytest.raises(gpu.LjError) as e:
            srv.submit(cb, seed=1, spp=-3)
        assert e.value.code == abi.LJ_ERR_INVALID_ARG
        with pytest.raises(gpu.LjError) as e:
            srv.poll(987654)
        assert e.value.code == abi.LJ_ERR_NOT_FOUND


def test_scene_kept_alive_while_registered(ctx):
    sc = scenes.cornell_box(seed=6, width=24, height=24, spp=4)
    g = gpu.GpuScene(ctx, sc)
    ref, _ = g.render(seed=1)
    srv = gpu.Server(ctx, small_opts())
    srv.submit(g, seed=1)
    h = g.h
    gpu.lib().lj_gpu_scene_destroy(h)        # refused: the server holds the scene
    img, _ = srv.wait(srv.submit(g, seed=1), timeout=120)
    assert_matches_plain(img, ref, atol=1e-7)
    srv.stop()


def test_autotune_picks_a_candidate_and_caches_it(ctx, tmp_path):
    gs = [gpu.GpuScene(ctx, scenes.cornell_box(seed=1, width=32, height=32, spp=4))]
    jobs = [gpu.job_desc(seed=k, spp=4) for k in range(4)]
    cache = str(tmp_path / "tune.json")
    opt = gpu.autotune(ctx, gs, jobs, [0] * 4, cache_path=cache)
    assert opt.path_pool in (1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24) and opt.block_size in (64, 128, 256)
    assert opt.waves_per_poll in (4, 8, 16)
    text = open(cache).read()
    assert "path_pool" in text and "block_size" in text and "median_latency_ms" in text
    again = gpu.autotune(ctx, gs, jobs, [0] * 4, cache_path=cache)
    assert (again.path_pool, again.block_size, again.waves_per_poll) == \
        (opt.path_pool, opt.block_size, opt.waves_per_poll)
    # another objective is another cache entry
    lat = gpu.autotune(ctx, gs, jobs, [0] * 4, cache_path=cache,
                       options=gpu.server_options(tune_objective=abi.LJ_TUNE_LATENCY))
    assert lat.block_size in (64, 128, 256)
    assert open(cache).read().count("|obj") == 2
    with pytest.raises(gpu.LjError):
        gpu.autotune(ctx, gs, jobs, [0] * 4, options=gpu.server_options(tune_objective=9))
