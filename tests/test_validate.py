"""lj_gpu_scene_validate (CPU): the checks lj_gpu_scene_create makes before
it touches the device.  Every scene the generators make for the tests and
the benchmark passes them; descriptions with out-of-range indices, unknown
kinds or empty images are refused with a reason."""
import ctypes as C

import numpy as np
import pytest

from lajolla_public_gb300 import abi, gpu, scenes
from golden import make_golden


def valid_scenes():
    out = {
        "cornell_box": scenes.cornell_box(seed=0, width=16, height=16, spp=1),
        "textured": scenes.textured_scene(4, 16, 16, 1, 6),
        "textured_no_clearcoat": scenes.textured_scene(4, 16, 16, 1, 6, clearcoat=False),
        "soup": scenes.soup_scene(1, 500),
        "tied_soup": scenes.tied_soup_scene(2, 64),
        "terrain": scenes.terrain_scene(seed=1, width=16, height=16, spp=1, grid=(32, 16)),
        "resized_terrain": scenes.resized_terrain_scene(seed=2, n_tris=20000, width=16, height=16, spp=1),
        "volume": scenes.volume_scene(width=16, height=16, spp=1, grid=8),
        "volume_three_channel": scenes.with_three_channel_density(scenes.volume_scene(width=16, height=16,
                                                                                       spp=1, grid=8)),
        "homogeneous_matched": scenes.homogeneous_box_scene(width=8, height=8, index_matched=True),
        "homogeneous_dielectric": scenes.homogeneous_box_scene(width=8, height=8, index_matched=False),
    }
    dark = scenes.cornell_box(seed=1, width=8, height=8, spp=2)   # no lights at all
    dark.shapes[-1]["area_light_id"] = -1
    dark.lights = []
    out["no_lights"] = dark
    single = scenes.Scene(4, 4, 1, 2, np.eye(4), 45.0)              # one triangle, no lights
    single.add_mesh(np.array([[-1, -1, -1], [1, -1, -1], [0, 1, -1]], np.float32), np.array([[0, 1, 2]]),
                    single.add_material(scenes.lambertian([0.5, 0.5, 0.5])))
    out["single_triangle"] = single
    for k, f in make_golden.RENDER_CASES.items():
        out["golden_" + k] = f()
    for k, f in make_golden.AUX_CASES.items():
        out["aux_" + k] = f()
    for k, sc in enumerate(scenes.serving_scenes(0, 6, max_tris=50000, volume_grid=8)):
        out["serving_%d" % k] = sc
    return out


def validate_desc(desc):
    buf = C.create_string_buffer(256)
    rc = gpu.lib().lj_gpu_scene_validate(C.byref(desc), buf, len(buf))
    return rc, buf.value.decode()


def test_generated_scenes_are_valid():
    for name, sc in valid_scenes().items():
        desc, keep = sc.desc()
        rc, msg = validate_desc(desc)
        assert rc == abi.LJ_OK, (name, msg)


def test_null_description_and_short_message_buffer():
    buf = C.create_string_buffer(8)
    assert gpu.lib().lj_gpu_scene_validate(None, buf, len(buf)) == abi.LJ_ERR_INVALID_ARG
    assert buf.value == b"null sc"           # truncated, NUL-terminated
    assert gpu.lib().lj_gpu_scene_validate(None, None, 0) == abi.LJ_ERR_INVALID_ARG


def _bad(mutate, reason):
    sc = scenes.textured_scene(4, 16, 16, 1, 6)
    desc, keep = sc.desc()
    mutate(desc, keep)
    rc, msg = validate_desc(desc)
    assert rc == abi.LJ_ERR_INVALID_ARG and reason in msg, msg


def _first_image_slot(desc):
    for i in range(desc.num_materials):
        for k in range(abi.LJ_MAT_SLOTS):
            if desc.materials[i].tex[k].kind == abi.LJ_TEX_IMAGE:
                return desc.materials[i].tex[k]
    raise AssertionError("no image texture")


@pytest.mark.parametrize("case", ["grid_res", "grid_channels", "grid_data", "volume_kind"])
def test_invalid_grid_volumes_are_refused(case):
    sc = scenes.volume_scene(width=8, height=8, spp=1, grid=8)
    desc, keep = sc.desc()
    i = next(k for k in range(desc.num_media) if desc.media[k].kind == abi.LJ_MEDIUM_HETEROGENEOUS)
    v = desc.media[i].density
    assert v.kind == abi.LJ_VOL_GRID
    if case == "grid_res":
        v.res[0], v.res[1] = -8, -8         # a positive product of negative sizes
    elif case == "grid_channels":
        v.channels = 4
    elif case == "grid_data":
        v.data = None
    else:
        v.kind = 2
    rc, msg = validate_desc(desc)
    assert rc == abi.LJ_ERR_INVALID_ARG and "medium %d" % i in msg, msg


@pytest.mark.parametrize("case", ["tex_image_id", "tex_kind", "image_channels", "image_size", "image_data",
                                  "light_kind", "shape_light", "shape_medium", "envmap_id", "material_type",
                                  "index_range", "camera"])
def test_invalid_descriptions_are_refused(case):
    def set_(obj, field, value):
        setattr(obj, field, value)

    if case == "tex_image_id":
        _bad(lambda d, k: set_(_first_image_slot(d), "image_id", d.num_images), "texture image id")
    elif case == "tex_kind":
        _bad(lambda d, k: set_(d.materials[0].tex[0], "kind", 7), "texture kind")
    elif case == "image_channels":
        _bad(lambda d, k: set_(d.images[0], "channels", 2), "image 0")
    elif case == "image_size":
        _bad(lambda d, k: set_(d.images[0], "width", 0), "image 0")
    elif case == "image_data":
        _bad(lambda d, k: set_(d.images[0], "data", None), "image 0")
    elif case == "light_kind":
        _bad(lambda d, k: set_(d.lights[0], "kind", 5), "unknown kind")
    elif case == "shape_light":
        _bad(lambda d, k: set_(d.shapes[0], "area_light_id", -2), "light id")
    elif case == "shape_medium":
        _bad(lambda d, k: set_(d.shapes[0], "interior_medium_id", -3), "medium id")
    elif case == "envmap_id":
        _bad(lambda d, k: set_(d, "envmap_light_id", -2), "envmap light id")
    elif case == "material_type":
        _bad(lambda d, k: set_(d.materials[0], "type", abi.LJ_MAT_COUNT), "unknown type")
    elif case == "index_range":
        def bump(d, k):
            idx = np.ctypeslib.as_array(C.cast(d.shapes[0].indices, C.POINTER(C.c_int32)),
                                        (d.shapes[0].num_triangles * 3,))
            idx[0] = d.shapes[0].num_vertices
        _bad(bump, "vertex index")
    else:
        _bad(lambda d, k: set_(d.camera, "width", 0), "camera")


def test_validate_scene_helper_raises():
    sc = scenes.cornell_box(seed=0, width=8, height=8, spp=1)
    gpu.validate_scene(sc)
    sc.width = 0
    with pytest.raises(gpu.LjError):
        gpu.validate_scene(sc)
