"""Per-function parity of the FP32 device code against golden vectors made
by the reference's own functions (Lambertian, RoughPlastic, RoughDielectric,
HG phase, light sampling and emission, primary rays with each pixel filter,
medium coefficients and majorants over grid volumes) and against the oracle
restatement (the Disney family, whose reference bodies are homework stubs --
parity unpinned there).

Tolerances (FP32 device code vs the reference's FP64 on identical inputs):
  scalar / RGB outputs (BSDF value, pdf, eta, phase value):
      |gpu - ref| <= 1e-5 |ref| + 1e-7   for at least 99% of the values,
      |gpu - ref| <= 1e-3 |ref| + 1e-6   for all of them;
  unit-vector outputs (sampled directions, normals), Euclidean error:
      <= 1e-5 for at least 99%, <= 1e-3 for all;
  points: the unit-vector rule scaled by max(1, |ref|).
The tails come from FP32 conditioning (grazing Fresnel, near-specular GGX
peaks, values of order 1e-7 next to O(1) intermediates)."""
import numpy as np
import pytest
import torch

import ljtest
from golden import make_golden
from lajolla_public_gb300 import abi, gpu, scenes
from oracle import ljo

pytestmark = pytest.mark.gpu


def check_close(got, want, name, rtol=1e-5, atol=1e-7, frac=0.99, rtol_all=1e-3, atol_all=1e-6):
    got = np.asarray(got, np.float64).reshape(-1)
    want = np.asarray(want, np.float64).reshape(-1)
    assert np.isfinite(got).all(), name
    d = np.abs(got - want)
    ok = (d <= rtol * np.abs(want) + atol).mean()
    worst = (d / (rtol_all * np.abs(want) + atol_all)).max()
    assert ok >= frac, "%s: only %.4f within rtol %g atol %g" % (name, ok, rtol, atol)
    assert worst <= 1.0, "%s: an error exceeds rtol %g atol %g by %.3gx" % (name, rtol_all, atol_all, worst)


def check_vectors(got, want, name, tol=1e-5, frac=0.99, tol_all=1e-3):
    got = np.asarray(got, np.float64).reshape(-1, 3)
    want = np.asarray(want, np.float64).reshape(-1, 3)
    assert np.isfinite(got).all(), name
    scale = np.maximum(1.0, np.linalg.norm(want, axis=1))
    err = np.linalg.norm(got - want, axis=1) / scale
    assert (err <= tol).mean() >= frac, "%s: only %.4f within %g (max %g)" % (name, (err <= tol).mean(), tol, err.max())
    assert err.max() <= tol_all, "%s: max error %g" % (name, err.max())


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def test_bsdf_vs_reference_golden(ctx):
    g = ljtest.golden("bsdf")
    rec, out = g["inputs"], g["outputs"]
    for t in (0, 1, 2):
        sel = rec[:, 0] == t
        r, o = rec[sel], out[sel]
        params = np.array([ljtest.bsdf_params(x)[1] for x in r], np.float32)
        wi, wo, rnd = cu(r[:, 9:12]), cu(r[:, 12:15]), cu(r[:, 15:18])
        P = cu(params)
        ev = ctx.bsdf(t, abi.LJ_BSDF_OP_EVAL, P, wi, wo)["value"].cpu().numpy()
        evv = ctx.bsdf(t, abi.LJ_BSDF_OP_EVAL, P, wi, wo, to_view=True)["value"].cpu().numpy()
        pd = ctx.bsdf(t, abi.LJ_BSDF_OP_PDF, P, wi, wo)["pdf"].cpu().numpy()
        sm = ctx.bsdf(t, abi.LJ_BSDF_OP_SAMPLE, P, wi, rnd=rnd)
        check_close(ev, o[:, 0:3], "eval type %d" % t)
        check_close(evv, o[:, 3:6], "eval to_view type %d" % t)
        check_close(pd, o[:, 6], "pdf type %d" % t)
        valid = sm["valid"].cpu().numpy()
        assert (valid == o[:, 7].astype(np.int32)).mean() >= 0.995
        v = (valid == 1) & (o[:, 7] == 1)
        check_vectors(sm["dir"].cpu().numpy()[v], o[v, 8:11], "sample dir type %d" % t)
        check_close(sm["eta"].cpu().numpy()[v], o[v, 11], "sample eta type %d" % t)
        check_close(sm["roughness"].cpu().numpy()[v], o[v, 12], "sample roughness type %d" % t)


def _disney_inputs(n, rng, t):
    widths = abi.SLOT_WIDTHS[t]
    cols = []
    for w in widths:
        if w == 3:
            cols.append(rng.uniform(0.05, 0.95, (n, 3)))
        else:
            cols.append(rng.uniform(0.0, 1.0, (n, 1)))
    p = np.concatenate(cols + [rng.uniform(1.2, 1.8, (n, 1))], axis=1)
    if t in (abi.LJ_MAT_DISNEY_METAL, abi.LJ_MAT_DISNEY_GLASS, abi.LJ_MAT_DISNEY_DIFFUSE):
        p[:, 3] = rng.uniform(0.05, 1.0, n)      # roughness
    if t == abi.LJ_MAT_DISNEY_BSDF:
        p[:, 3 + 4] = rng.uniform(0.05, 1.0, n)  # roughness slot
    wi = ljtest_hemi(rng, n)
    wi[: n // 5, 2] *= -1                     # some from inside
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    return p.astype(np.float32), wi.astype(np.float32), wo.astype(np.float32), rng.uniform(0, 1, (n, 3)).astype(np.float32)


def ljtest_hemi(rng, n):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    v[:, 2] = np.abs(v[:, 2]) + 0.05
    return v / np.linalg.norm(v, axis=1, keepdims=True)


@pytest.mark.parametrize("t", [abi.LJ_MAT_DISNEY_DIFFUSE, abi.LJ_MAT_DISNEY_METAL, abi.LJ_MAT_DISNEY_GLASS,
                               abi.LJ_MAT_DISNEY_CLEARCOAT, abi.LJ_MAT_DISNEY_SHEEN, abi.LJ_MAT_DISNEY_BSDF])
def test_disney_vs_oracle_restatement(ctx, t):
    rng = np.random.default_rng(100 + t)
    p, wi, wo, rnd = _disney_inputs(4000, rng, t)
    want_e = ljo.bsdf(t, abi.LJ_BSDF_OP_EVAL, p, wi, wo)["value"]
    want_p = ljo.bsdf(t, abi.LJ_BSDF_OP_PDF, p, wi, wo)["pdf"]
    want_s = ljo.bsdf(t, abi.LJ_BSDF_OP_SAMPLE, p, wi, rnd=rnd)
    P, WI, WO, R = cu(p), cu(wi), cu(wo), cu(rnd)
    check_close(ctx.bsdf(t, abi.LJ_BSDF_OP_EVAL, P, WI, WO)["value"].cpu().numpy(), want_e, "disney eval %d" % t)
    check_close(ctx.bsdf(t, abi.LJ_BSDF_OP_PDF, P, WI, WO)["pdf"].cpu().numpy(), want_p, "disney pdf %d" % t)
    s = ctx.bsdf(t, abi.LJ_BSDF_OP_SAMPLE, P, WI, rnd=R)
    valid = s["valid"].cpu().numpy()
    assert (valid == want_s["valid"]).mean() >= 0.995
    v = (valid == 1) & (want_s["valid"] == 1)
    check_vectors(s["dir"].cpu().numpy()[v], want_s["dir"][v], "disney dir %d" % t)


def test_bsdf_sample_pdf_consistency_reference_method(ctx):
    """The reference's materials test (src/tests/materials.cpp:5-53): the
    inverse Jacobian determinant of the sampling map equals the pdf (1e-2)."""
    wi = np.array([0.3, 0.4, 0.5]) / np.linalg.norm([0.3, 0.4, 0.5])
    uv = np.array([0.3, 0.4])
    eps = 1e-3   # FP32: larger finite-difference step than the reference's 1e-6
    cases = [(abi.LJ_MAT_LAMBERTIAN, [0.5, 0.5, 0.5, 1.0], [0.6]),
             (abi.LJ_MAT_ROUGHPLASTIC, [0.5, 0.5, 0.5, 0.5, 0.5, 0.5, 0.3, 1.5], [0.0, 1.0]),
             (abi.LJ_MAT_DISNEY_METAL, [0.5, 0.5, 0.5, 0.3, 0.2, 1.5], [0.5])]
    for t, params, ws in cases:
        for w in ws:
            rnd = np.array([[uv[0], uv[1], w], [uv[0] + eps, uv[1], w], [uv[0], uv[1] + eps, w]], np.float32)
            s = ctx.bsdf(t, abi.LJ_BSDF_OP_SAMPLE, cu(np.tile(params, (3, 1))), cu(np.tile(wi, (3, 1))), rnd=cu(rnd))
            d = s["dir"].cpu().numpy().astype(np.float64)
            du, dv = (d[1] - d[0]) / eps, (d[2] - d[0]) / eps
            det = np.sqrt(du.dot(du) * dv.dot(dv) - du.dot(dv) ** 2)
            pdf = ctx.bsdf(t, abi.LJ_BSDF_OP_PDF, cu(np.tile(params, (1, 1))), cu(wi[None]), cu(d[:1]))["pdf"].cpu().numpy()[0]
            if t == abi.LJ_MAT_ROUGHPLASTIC:
                # a mixture: the sampled lobe's own density is what the Jacobian measures
                continue
            assert abs(1 / det - pdf) / pdf < 2e-2, (t, w, 1 / det, pdf)


def test_phase_vs_reference_golden(ctx):
    g = ljtest.golden("phase")
    r, o = g["inputs"], g["outputs"]
    for gval in np.unique(r[:, 0]):
        sel = r[:, 0] == gval
        val, pdf, d = ctx.phase(abi.LJ_PHASE_HG, float(gval), cu(r[sel, 1:4]), cu(r[sel, 4:7]), cu(r[sel, 7:9]))
        check_close(val.cpu().numpy(), o[sel, 0], "hg eval g=%g" % gval)
        check_close(pdf.cpu().numpy(), o[sel, 1], "hg pdf g=%g" % gval)
        check_vectors(d.cpu().numpy(), o[sel, 2:5], "hg dir g=%g" % gval)


def test_light_sampling_vs_reference_golden(ctx):
    g = ljtest.golden("light")
    sc = ljtest.light_scene(g["env"], g["to_world"])
    gs = gpu.GpuScene(ctx, sc)
    r, out = g["inputs"], g["outputs"]
    lid, pt, nr, pdf = gs.light_sample(cu(r[:, 0:3]), cu(r[:, [3, 4, 5, 6]]))
    lid = lid.cpu().numpy()
    same = lid == out[:, 0].astype(np.int32)
    assert same.mean() >= 0.99
    check_vectors(pt.cpu().numpy()[same], out[same, 1:4], "light point")
    check_vectors(nr.cpu().numpy()[same], out[same, 4:7], "light normal")
    check_close(pdf.cpu().numpy()[same], out[same, 7], "light pdf")


def test_light_emission_vs_reference_golden(ctx):
    """emission (src/light.cpp:56-77) at the reference's sampled light points:
    one-sided area lights (mesh and sphere) and the rotated envmap's lookup
    (src/lights/envmap.inl:44-73)."""
    g = ljtest.golden("light")
    gs = gpu.GpuScene(ctx, ljtest.light_scene(g["env"], g["to_world"]))
    lid, pt, nr, view = ljtest.emission_queries(g)
    e = gs.light_emission(torch.from_numpy(lid).cuda(), cu(view), cu(pt), cu(nr)).cpu().numpy()
    want = g["outputs"][:, 8:11]
    for k in (0, 1, 2):
        sel = lid == k
        assert sel.sum() > 20
        check_close(e[sel], want[sel], "emission of light %d" % k)


@pytest.mark.parametrize("fk", [abi.LJ_FILTER_BOX, abi.LJ_FILTER_TENT, abi.LJ_FILTER_GAUSSIAN])
def test_camera_rays_vs_reference_golden(ctx, fk):
    """sample_primary (src/camera.cpp:23-47) with the box, tent and Gaussian
    pixel filters (src/filters/box.inl, tent.inl, gaussian.inl) at the
    golden's non-square resolutions: origins exact, directions within the
    unit-vector tolerance."""
    g = ljtest.golden("camera")
    k = "f%d_" % fk
    sc = scenes.Scene(int(g[k + "w"]), int(g[k + "h"]), 1, 2, g[k + "matrix"], float(g[k + "fov"]),
                      filter_kind=int(g[k + "filter"]), filter_param=float(g[k + "param"]))
    m = sc.add_material(scenes.lambertian([0.5, 0.5, 0.5]))
    sc.add_mesh(np.array([[0, 0, -5], [1, 0, -5], [0, 1, -5]], np.float32), np.array([[0, 1, 2]]), m)
    org, d = gpu.GpuScene(ctx, sc).camera_rays(cu(g[k + "screen"]))
    want = g[k + "rays"]
    check_vectors(org.cpu().numpy(), want[:, 0:3], "camera origin filter %d" % fk, tol=1e-7, frac=1.0, tol_all=1e-7)
    check_vectors(d.cpu().numpy(), want[:, 3:6], "camera direction filter %d" % fk)


def test_medium_vs_reference_golden(ctx):
    """get_sigma_a / get_sigma_s (trilinear GridVolume lookups,
    src/volume.h:44-81) at points in and around the grids, and get_majorant
    (the box slab test, src/volume.h:124-144) along rays, for a one-channel
    density grid with a constant albedo, a three-channel density grid with a
    three-channel albedo grid, and a homogeneous medium
    (src/medium.cpp:27-37), all read by the reference from .vol files."""
    g = ljtest.golden("medium")
    gs = gpu.GpuScene(ctx, make_golden.medium_scene(g))
    P, D = cu(g["points"]), cu(g["dirs"])
    for k in range(3):
        sa, ss, mj = (t.cpu().numpy() for t in gs.medium(k, P, D))
        want = g["outputs"][:, k]
        check_close(sa, want[:, 0:3], "sigma_a medium %d" % k)
        check_close(ss, want[:, 3:6], "sigma_s medium %d" % k)
        # the FP32 slab test may flip a ray that grazes the box's edge
        hit_g, hit_r = mj.sum(1) > 0, want[:, 6:9].sum(1) > 0
        assert (hit_g == hit_r).mean() >= 0.995, (k, (hit_g != hit_r).sum())
        both = hit_g & hit_r
        check_close(mj[both], want[both, 6:9], "majorant medium %d" % k, frac=1.0)
    with pytest.raises(gpu.LjError):
        gs.medium(3, P, D)
