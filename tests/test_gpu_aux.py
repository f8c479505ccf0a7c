"""Auxiliary integrators (aux_render, src/render.cpp:12-69) on the GPU
against the oracle and the reference's own aux images (tests/golden/aux.npz).

The camera ray is computed in FP32 on the GPU and in FP64 in the oracle, so
a ray through a corner where two surfaces meet may pick the other surface
(both at the same distance); at least 99% of the pixels must agree within
the per-quantity tolerance below, and every pixel that does not must still
agree on the hit distance (a corner, not a different object)."""
import numpy as np
import pytest

import ljtest
from golden import make_golden
from lajolla_public_gb300 import gpu
from oracle import ljo

pytestmark = pytest.mark.gpu

# (rtol, atol) per integrator: depth and normals are FP32 rounding only;
# mean curvature differentiates interpolated normals over small triangles;
# the mipmap level is a log2 of a product of FP32 terms.
TOL = {
    "depth": (1e-5, 1e-6),
    "shading_normal": (0.0, 1e-4),
    "mean_curvature": (1e-3, 1e-4),
    "ray_differential": (1e-6, 1e-7),
    "mipmap_level": (0.0, 1e-3),
}


@pytest.mark.parametrize("case", sorted(make_golden.AUX_CASES))
def test_aux_matches_oracle_and_reference(ctx, case):
    sc = make_golden.AUX_CASES[case]()
    img_g, st = gpu.GpuScene(ctx, sc).render(seed=1)
    img_o = ljo.OracleScene(sc).render(mode="tile")
    ref = ljtest.golden("aux")[case]
    rtol, atol = TOL[case]
    depth_sc = make_golden.AUX_CASES["depth"]()
    d_g, _ = gpu.GpuScene(ctx, depth_sc).render(seed=1)
    d_o = ljo.OracleScene(depth_sc).render(mode="tile")
    for other in (img_o, ref):
        ok = (np.abs(img_g - other) <= atol + rtol * np.abs(other)).all(axis=2)
        assert ok.mean() >= 0.99, (case, ok.mean())
        np.testing.assert_allclose(d_g[~ok], d_o[~ok], rtol=1e-5, atol=1e-6, err_msg=case)
    assert st.samples == sc.width * sc.height and st.kernel_launches == 1


def test_aux_ignores_seed_and_spp(ctx):
    sc = make_golden.AUX_CASES["depth"]()
    g = gpu.GpuScene(ctx, sc)
    a, _ = g.render(seed=1, spp=1)
    b, _ = g.render(seed=99, spp=7)
    np.testing.assert_array_equal(a, b)
