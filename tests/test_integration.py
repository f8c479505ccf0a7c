"""The reference-side adapter (lajolla_public_gb300/adapter/render_gpu.cpp)
linked with the reference's own parser and scene code and liblj_gpu.so
(oracle/Makefile, target `adapter`) and run: every scene file the reference
ships parses, flattens and passes the library's checks; the flattened
descriptor of a scene written by lajolla_public_gb300.scenes equals the
generator's own description field by field; and an image written through
the adapter (image_from_rgb + the reference's imwrite) is byte-identical to
the file the reference renderer writes for the same pixels.  Needs the
reference sources, so it runs in the development container only (skipped
elsewhere); the GPU half of this path is tests/test_gpu_render.py's
reference-scene test."""
import glob
import os
import subprocess
import tempfile

import numpy as np
import pytest

import ljtest
from golden import make_golden
from lajolla_public_gb300 import abi, build, gpu
from oracle import ljo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = ljo.reference_dir()
pytestmark = pytest.mark.skipif(REF is None, reason="reference sources not present")


@pytest.fixture(scope="module")
def adapter():
    build.build()
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s", "-j8", "adapter"], check=True,
                   capture_output=True)
    return make_golden.ADAPTER


def flatten(adapter, xml):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "s.flat")
        r = subprocess.run([adapter, "flatten", xml, out], capture_output=True, text=True,
                           cwd=os.path.dirname(xml))
        assert r.returncode == 0, (xml, r.stderr[-2000:])
        return ljtest.load_flat(open(out, "rb").read())


def test_every_reference_scene_parses_flattens_and_validates(adapter):
    xmls = sorted(glob.glob(os.path.join(REF, "scenes", "*", "*.xml")))
    assert len(xmls) >= 20
    kinds = set()
    for xml in xmls:
        sc = flatten(adapter, xml)
        gpu.validate_scene(sc)
        kinds |= {m["type"] for m in sc.materials} | {("light", l["kind"]) for l in sc.lights}
        kinds |= {("medium", m["kind"]) for m in sc.media} | {("filter", sc.filter_kind)}
    # the reference's scenes exercise every material, both light kinds, both
    # media and every pixel filter
    assert set(range(abi.LJ_MAT_COUNT)) <= kinds
    assert {("light", 0), ("light", 1), ("medium", 0), ("medium", 1)} <= kinds
    assert {("filter", 0), ("filter", 1), ("filter", 2)} & kinds


# materials with an index of refraction in the reference (src/material.h)
ETA_MATERIALS = (abi.LJ_MAT_ROUGHPLASTIC, abi.LJ_MAT_ROUGHDIELECTRIC, abi.LJ_MAT_DISNEY_GLASS, abi.LJ_MAT_DISNEY_BSDF)


def corners(sh, key, width):
    a = sh[key]
    return None if a is None else a[sh["indices"]].reshape(-1, width)


def assert_same_scene(a, b):
    """a: the generator's scene; b: the adapter's flattening of its XML."""
    assert (a.width, a.height, a.spp, a.integrator) == (b.width, b.height, b.spp, b.integrator)
    if a.integrator >= abi.LJ_INTEGRATOR_PATH:   # the parser reads depths for these only
        assert (a.max_depth, a.rr_depth) == (b.max_depth, b.rr_depth)
    assert a.filter_kind == b.filter_kind and a.filter_param == b.filter_param
    np.testing.assert_allclose(b.cam_to_world, a.cam_to_world, rtol=0, atol=1e-7)
    assert abs(a.fov - b.fov) <= 1e-5 * a.fov
    assert len(a.shapes) == len(b.shapes)
    for sa, sb in zip(a.shapes, b.shapes):
        for k in ("kind", "material_id", "area_light_id", "interior_medium_id", "exterior_medium_id"):
            assert sa[k] == sb[k], k
        if sa["kind"] == abi.LJ_SHAPE_MESH:
            # the OBJ loader may renumber vertices: compare triangle corners
            np.testing.assert_array_equal(corners(sb, "positions", 9), corners(sa, "positions", 9))
            for key, w in (("normals", 9), ("uvs", 6)):
                ca, cb = corners(sa, key, w), corners(sb, key, w)
                assert (ca is None) == (cb is None), key
                if ca is not None:
                    np.testing.assert_allclose(cb, ca, rtol=0, atol=1e-7)
        else:
            np.testing.assert_array_equal(np.float32(sb["center"]), np.float32(sa["center"]))
            assert np.float32(sb["radius"]) == np.float32(sa["radius"])
    assert len(a.materials) == len(b.materials)
    for ma, mb in zip(a.materials, b.materials):
        assert ma["type"] == mb["type"]
        if ma["type"] in ETA_MATERIALS:
            assert np.float32(ma["eta"]) == np.float32(mb["eta"])
        for k, ta in enumerate(ma["tex"]):
            tb = mb["tex"][k]
            assert ta.get("kind", abi.LJ_TEX_CONST) == tb["kind"]
            width = abi.SLOT_WIDTHS[ma["type"]][k]
            for key in ("value0", "value1"):
                np.testing.assert_array_equal(np.float32(tb[key][:width]), np.float32(ta.get(key, [0, 0, 0])[:width]))
            for key, dflt in (("uscale", 1), ("vscale", 1), ("uoffset", 0), ("voffset", 0)):
                assert np.float32(tb[key]) == np.float32(ta.get(key, dflt)), key
            if tb["kind"] == abi.LJ_TEX_IMAGE:
                np.testing.assert_array_equal(b.images[tb["image_id"]], a.images[ta["image_id"]])
    assert len(a.lights) == len(b.lights) and a.envmap_light_id == b.envmap_light_id
    for la, lb in zip(a.lights, b.lights):
        assert la["kind"] == lb["kind"]
        if la["kind"] == abi.LJ_LIGHT_AREA:
            assert la["shape_id"] == lb["shape_id"]
            np.testing.assert_array_equal(np.float32(lb["intensity"]), np.float32(la["intensity"]))
        else:
            assert np.float32(la.get("scale", 1.0)) == np.float32(lb["scale"])
            np.testing.assert_array_equal(lb["to_world"], np.asarray(la["to_world"]))
            np.testing.assert_allclose(lb["to_local"], np.asarray(la["to_local"]), rtol=0, atol=1e-12)
            np.testing.assert_array_equal(b.images[lb["image_id"]], a.images[la["image_id"]])


@pytest.mark.parametrize("case", sorted(make_golden.RENDER_CASES) + sorted(make_golden.AUX_CASES))
def test_adapter_flattening_equals_the_generators_scene(adapter, case):
    sc = {**make_golden.RENDER_CASES, **make_golden.AUX_CASES}[case]()
    with tempfile.TemporaryDirectory() as d:
        flat = flatten(adapter, sc.write_mitsuba(d, case))
    assert_same_scene(sc, flat)


@pytest.mark.parametrize("ext", ["pfm", "exr"])
def test_image_written_through_the_adapter_is_byte_identical(adapter, ext):
    """The reference renders a scene to PFM and to EXR (FP16); the adapter
    turns the PFM's FP32 pixels (the form the library returns) into an
    Image3 and writes it with the reference's imwrite: same bytes."""
    sc = make_golden.RENDER_CASES["mixed"]()
    with tempfile.TemporaryDirectory() as d:
        xml = sc.write_mitsuba(d, "s")
        ljo.run_reference(xml, os.path.join(d, "ref.pfm"), threads=8)
        want = os.path.join(d, "ref." + ext)
        if ext != "pfm":   # same tile-keyed samples, same image, written as FP16 EXR
            subprocess.run([os.path.join(ljo.REF_DIR, "lajolla"), "-t", "8", "-o", want, xml], check=True,
                           capture_output=True, cwd=d)
        got = os.path.join(d, "got." + ext)
        subprocess.run([adapter, "write", os.path.join(d, "ref.pfm"), got], check=True)
        assert open(got, "rb").read() == open(want, "rb").read()
