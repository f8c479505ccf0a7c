"""The oracle (C++ restatement, oracle/lj_oracle.cpp) pinned against golden
vectors and renders produced by the reference's own code
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

import ljtest
from lajolla_public_gb300 import abi, scenes
from oracle import ljo
from golden import make_golden


def test_pcg_matches_reference():
    g = ljtest.golden("pcg")
    for i, s in enumerate(g["streams"]):
        raw = ljo.pcg(int(s), 0x31e241f862a1fb5e, g["raw"].shape[1])
        np.testing.assert_array_equal(raw, g["raw"][i])
        np.testing.assert_array_equal(raw.astype(np.float64) / 2.0 ** 32, g["real"][i])


def test_table_dist_matches_reference():
    g = ljtest.golden("table")
    L = ljo.lib()
    f1, u1 = np.ascontiguousarray(g["f1"]), np.ascontiguousarray(g["u1"])
    idx = np.zeros(len(u1), np.int32)
    pmf = np.zeros(len(u1))
    L.ljo_table1d(ljo._p(f1), len(f1), ljo._p(u1), len(u1), ljo._p(idx), ljo._p(pmf))
    np.testing.assert_array_equal(idx, g["idx1"].astype(np.int32))
    np.testing.assert_allclose(pmf, g["pmf1"], rtol=1e-14, atol=0)
    f2 = np.ascontiguousarray(g["f2"])
    u2 = np.ascontiguousarray(g["u2"])
    xy = np.zeros((len(u2), 2))
    pdf = np.zeros(len(u2))
    h, w = f2.shape
    L.ljo_table2d(ljo._p(f2), w, h, ljo._p(u2), len(u2), ljo._p(xy), ljo._p(pdf))
    np.testing.assert_allclose(xy, g["xy2"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(pdf, g["pdf2"], rtol=1e-13, atol=0)


def test_camera_matches_reference():
    """sample_primary (src/camera.cpp:23-47) with the box, tent and Gaussian
    pixel filters (src/filters/*.inl) at non-square resolutions: ray origins
    and directions equal the reference's to FP64 rounding."""
    g = ljtest.golden("camera")
    for fk in (abi.LJ_FILTER_BOX, abi.LJ_FILTER_TENT, abi.LJ_FILTER_GAUSSIAN):
        k = "f%d_" % fk
        rays = ljo.camera_rays(g[k + "matrix"], g[k + "fov"], g[k + "w"], g[k + "h"], g[k + "filter"],
                               g[k + "param"], g[k + "screen"])
        assert rays.shape == g[k + "rays"].shape == (200, 6)
        np.testing.assert_allclose(rays, g[k + "rays"], rtol=1e-12, atol=1e-13)


def test_filter_sampling_jacobian_reference_method():
    """The reference's filter test (src/tests/filter.cpp:15-68) on the
    oracle's filter sampling: the determinant of the sampling map's
    finite-difference Jacobian equals the inverse of the normalised filter
    kernel at the sample (width 2 box and tent, standard deviation 2
    Gaussian), at the reference's point (0.3, 0.4) and at more points."""
    eps = 1e-6
    pts = np.array([[0.3, 0.4], [0.1, 0.8], [0.7, 0.2], [0.55, 0.45], [0.9, 0.95]])
    for kind, w in ((abi.LJ_FILTER_BOX, 2.0), (abi.LJ_FILTER_TENT, 2.0), (abi.LJ_FILTER_GAUSSIAN, 2.0)):
        s = ljo.filter_sample(kind, w, pts)
        su = ljo.filter_sample(kind, w, pts + [eps, 0])
        sv = ljo.filter_sample(kind, w, pts + [0, eps])
        du, dv = (su - s) / eps, (sv - s) / eps
        det = np.abs(du[:, 0] * dv[:, 1] - du[:, 1] * dv[:, 0])
        if kind == abi.LJ_FILTER_BOX:
            inv_kernel = np.full(len(pts), w * w)
        elif kind == abi.LJ_FILTER_TENT:
            h = w / 2
            inv_kernel = 1 / (((1 - np.abs(s[:, 0]) / h) / h) * ((1 - np.abs(s[:, 1]) / h) / h))
        else:
            r2 = (s ** 2).sum(1)
            inv_kernel = 1 / (np.exp(-r2 / (w * w) / 2) / (w * w * 2 * np.pi))
        np.testing.assert_allclose(det, inv_kernel, rtol=1e-3, atol=1e-3)


def test_mipmap_reference_known_answer_and_box_pyramid():
    """The reference's mipmap test (src/tests/mipmap.cpp:5-30) on the
    oracle's mipmap: a constant 64x64 image looks up to 1 at every texel
    centre of every level l + 0.5.  And for a random 64x32 image: level 0 at
    texel centres returns the texels, an integer level k returns the mean of
    the 2^k x 2^k block, and levels past the last clamp to it."""
    xs = (np.arange(64) + 0.5) / 64
    uu, vv = np.meshgrid(xs, xs)
    ones = np.ones((64, 64, 3), np.float32)
    _, nl = ljo.mipmap_lookup(ones, np.zeros((1, 3)))
    assert nl == 7
    for lvl in range(nl):
        q = np.stack([uu.ravel(), vv.ravel(), np.full(uu.size, lvl + 0.5)], 1)
        out, _ = ljo.mipmap_lookup(ones, q)
        assert np.abs(out - 1).max() <= 1e-3
    rng = np.random.default_rng(3)
    img = rng.uniform(0, 1, (32, 64, 3)).astype(np.float32)
    for k in range(4):
        bw, bh = 64 >> k, 32 >> k
        block = img.astype(np.float64).reshape(bh, 1 << k, bw, 1 << k, 3).mean(axis=(1, 3))
        u, v = np.meshgrid((np.arange(bw) + 0.5) / bw, (np.arange(bh) + 0.5) / bh)
        q = np.stack([u.ravel(), v.ravel(), np.full(u.size, float(k))], 1)
        out, nl = ljo.mipmap_lookup(img, q)
        np.testing.assert_allclose(out, block.reshape(-1, 3), rtol=1e-12, atol=1e-12)
    last = img.astype(np.float64).mean(axis=(0, 1))   # 64x32 -> 7 levels, the last 1x1 holds the mean
    out, nl = ljo.mipmap_lookup(img, [[0.3, 0.6, 50.0]])
    assert nl == 7
    np.testing.assert_allclose(out[0], last, rtol=1e-12)


def test_bsdf_matches_reference():
    g = ljtest.golden("bsdf")
    rec, out = g["inputs"], g["outputs"]
    for t in (0, 1, 2):
        sel = rec[:, 0] == t
        r, o = rec[sel], out[sel]
        params = np.array([ljtest.bsdf_params(x)[1] for x in r], np.float32)
        wi, wo, rnd = r[:, 9:12], r[:, 12:15], r[:, 15:18]
        ev = ljo.bsdf(t, abi.LJ_BSDF_OP_EVAL, params, wi, wo)
        evv = ljo.bsdf(t, abi.LJ_BSDF_OP_EVAL, params, wi, wo, to_view=True)
        pd = ljo.bsdf(t, abi.LJ_BSDF_OP_PDF, params, wi, wo)
        sm = ljo.bsdf(t, abi.LJ_BSDF_OP_SAMPLE, params, wi, rnd=rnd)
        np.testing.assert_allclose(ev["value"], o[:, 0:3], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(evv["value"], o[:, 3:6], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(pd["pdf"], o[:, 6], rtol=1e-12, atol=1e-14)
        np.testing.assert_array_equal(sm["valid"], o[:, 7].astype(np.int32))
        v = sm["valid"] == 1
        np.testing.assert_allclose(sm["dir"][v], o[v, 8:11], rtol=1e-12, atol=1e-13)
        np.testing.assert_allclose(sm["eta"][v], o[v, 11], rtol=1e-12)
        np.testing.assert_allclose(sm["roughness"][v], o[v, 12], rtol=1e-12)


def test_phase_matches_reference():
    g = ljtest.golden("phase")
    r, o = g["inputs"], g["outputs"]
    for gval in np.unique(r[:, 0]):
        sel = r[:, 0] == gval
        val, pdf, d = ljo.phase(abi.LJ_PHASE_HG, float(gval), r[sel, 1:4], r[sel, 4:7], r[sel, 7:9])
        np.testing.assert_allclose(val, o[sel, 0], rtol=1e-12)
        np.testing.assert_allclose(pdf, o[sel, 1], rtol=1e-12)
        np.testing.assert_allclose(d, o[sel, 2:5], rtol=1e-10, atol=1e-12)


def test_light_sampling_matches_reference():
    g = ljtest.golden("light")
    sc = ljtest.light_scene(g["env"], g["to_world"])
    o = ljo.OracleScene(sc)
    r, out = g["inputs"], g["outputs"]
    lid, pt, nr, pdf = o.light_sample(r[:, 0:3], r[:, [3, 4, 5, 6]])
    np.testing.assert_array_equal(lid, out[:, 0].astype(np.int32))
    np.testing.assert_allclose(pt, out[:, 1:4], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(nr, out[:, 4:7], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(pdf, out[:, 7], rtol=1e-9)


def test_light_emission_matches_reference():
    """emission (src/light.cpp:56-77) of the reference's sampled light points:
    one-sided area-light radiance and the envmap's lookup
    (src/lights/envmap.inl:44-73), on the light golden's outputs."""
    g = ljtest.golden("light")
    o = ljo.OracleScene(ljtest.light_scene(g["env"], g["to_world"]))
    lid, pt, nr, view = ljtest.emission_queries(g)
    np.testing.assert_allclose(o.light_emission(lid, view, pt, nr), g["outputs"][:, 8:11], rtol=1e-9, atol=1e-12)
    assert (g["outputs"][lid == 2, 8:11] > 0).all()   # envmap samples are lit


def test_medium_matches_reference():
    """get_sigma_a / get_sigma_s / get_majorant (src/medium.cpp:27-37) with
    the GridVolume lookup and slab test (src/volume.h:44-144) on grids the
    reference's .vol loader read, and a homogeneous medium."""
    g = ljtest.golden("medium")
    o = ljo.OracleScene(make_golden.medium_scene(g))
    for k in range(3):
        sa, ss, mj = o.medium(k, g["points"], g["dirs"])
        want = g["outputs"][:, k]
        np.testing.assert_allclose(sa, want[:, 0:3], rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(ss, want[:, 3:6], rtol=1e-6, atol=1e-12)
        np.testing.assert_array_equal(mj, want[:, 6:9])


@pytest.mark.parametrize("case", sorted(make_golden.RENDER_CASES))
def test_render_matches_reference_sample_for_sample(case):
    """Tile-mode RNG reproduces the reference renderer's own image exactly
    (up to its FP32 PFM output rounding)."""
    ref = ljtest.golden("renders")[case]
    sc = make_golden.RENDER_CASES[case]()
    img = ljo.OracleScene(sc).render(mode="tile", yx_order=True)
    np.testing.assert_allclose(img, ref, rtol=2e-7, atol=2e-7)


@pytest.mark.parametrize("name", sorted(make_golden.REF_SCENES))
def test_flattened_reference_scene_renders_like_the_reference(name):
    """The reference's own scene files (cbox.xml, veach_mi/mi.xml,
    pixel_filter_test.xml), parsed by the reference and flattened by the
    adapter into the FP32 descriptor: the oracle's tile-mode render equals
    the reference's render of the same file sample for sample, except where
    the FP32 rounding of material and light values flips a Russian-roulette
    or light-selection decision (a few paths of cbox's roulette-only paths
    and of the MIS scene's glossy plates); their image means agree."""
    g = ljtest.golden("refscenes")
    sc = ljtest.load_flat(g[name + "_flat"].tobytes())
    ref = g[name + "_render"].astype(np.float64)
    img = ljo.OracleScene(sc).render(mode="tile", yx_order=True)
    rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    assert (rel <= 1e-6).all(axis=2).mean() >= 0.98, (rel > 1e-6).mean()
    np.testing.assert_allclose(img.mean(axis=(0, 1)), ref.mean(axis=(0, 1)), rtol=2e-3)


def test_morton_sort_is_stable_and_sorted():
    pos, idx = scenes.triangle_soup(5, 20000)
    tri = pos[idx].reshape(-1, 9)
    tri[100] = tri[7]          # duplicate codes -> order by index
    codes, order = ljo.morton(tri)
    assert codes.max() < (1 << 30)
    s = codes[order]
    assert np.all(np.diff(s.astype(np.int64)) >= 0)
    ties = np.diff(s.astype(np.int64)) == 0
    assert np.all(np.diff(order.astype(np.int64))[ties] > 0)
    np.testing.assert_array_equal(np.sort(order), np.arange(len(tri)))


def test_single_triangle_reference_known_answer_cpu():
    """src/tests/intersection.cpp:4-42 on the oracle: triangle (-1,-1,-1)
    (1,-1,-1) (0,1,-1); a ray from the origin along -z hits (0, 0, -1), one
    along +z misses."""
    sc = scenes.Scene(4, 4, 1, 2, np.eye(4), 45.0)
    m = sc.add_material(scenes.lambertian([0.5, 0.5, 0.5]))
    sc.add_mesh(np.array([[-1, -1, -1], [1, -1, -1], [0, 1, -1]], np.float32), np.array([[0, 1, 2]]), m)
    o = ljo.OracleScene(sc)
    rays = np.array([[0, 0, 0, 0, 0, 0, -1, np.inf], [0, 0, 0, 0, 0, 0, 1, np.inf]], np.float32)
    for brute in (True, False):
        t, prim, _, _, _ = o.trace_closest(rays, brute=brute)
        assert prim[0] == 0 and prim[1] < 0
        p = rays[0, :3] + rays[0, 4:7] * t[0]
        assert np.linalg.norm(p - np.array([0, 0, -1])) < 1e-3
        np.testing.assert_array_equal(o.trace_any(rays, brute=brute), [1, 0])


def test_bvh_matches_brute_force_cpu():
    """The oracle's own BVH traversal agrees with brute force (CPU twin of
    the GPU trace parity test)."""
    sc = scenes.soup_scene(3, 3000)
    o = ljo.OracleScene(sc)
    rays = scenes.random_rays(4, 4000)
    t0, p0, _, _, ties = o.trace_closest(rays, brute=True)
    t1, p1, _, _, _ = o.trace_closest(rays, brute=False)
    assert np.array_equal(p0, p1)
    np.testing.assert_array_equal(t0[p0 >= 0], t1[p0 >= 0])
    np.testing.assert_array_equal(o.trace_any(rays, brute=True), o.trace_any(rays, brute=False))


@pytest.mark.parametrize("case", sorted(make_golden.AUX_CASES))
def test_aux_render_matches_reference(case):
    """aux_render (src/render.cpp:12-69): one deterministic ray per pixel."""
    ref = ljtest.golden("aux")[case]
    sc = make_golden.AUX_CASES[case]()
    img = ljo.OracleScene(sc).render(mode="tile")
    np.testing.assert_allclose(img, ref, rtol=1e-6, atol=1e-6)
    assert np.abs(ref).max() > 0


def test_bvh_ties_resolve_to_lowest_index_cpu():
    """Equal-t hits go to the lower primitive index whatever the traversal
    order (the rule the GPU traversal follows too)."""
    sc = scenes.tied_soup_scene(7, 2000)
    o = ljo.OracleScene(sc)
    rays = scenes.random_rays(8, 20000)
    t0, p0, _, _, ties = o.trace_closest(rays, brute=True)
    t1, p1, _, _, _ = o.trace_closest(rays, brute=False)
    assert (ties > 1).sum() > 500
    assert np.array_equal(p0, p1)
    np.testing.assert_array_equal(t0, t1)
