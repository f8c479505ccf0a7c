"""Scene description + seeded synthetic scene generators.

A `Scene` holds the flat, FP32 view of lajolla's `Scene` (src/scene.h:42-82)
that the C ABI takes (`lj_scene_desc`, include/lj_gpu.h).  Every value a
generator produces is float32-exact, so the same scene written out as Mitsuba
XML + OBJ (`write_mitsuba`) parses in the reference renderer (whose parser
reads numbers with std::stof, src/parsers/parse_scene.cpp:85-116) to exactly
the same numbers the GPU path receives.

Generators (seeded, deterministic):
  cornell_box      5 wall quads + 2 y-rotated boxes + ceiling quad light
                   (17, 12, 4), Lambertian albedos U[0.1, 0.8]^3, fov 40,
                   box filter -- the 256x256 / 64 spp / max depth 6 workload.
  triangle_soup    n triangles, centroids U[0,1]^3, vertex offsets N(0, 0.01)
  random_rays      origins U[-0.5, 1.5]^3, directions uniform on S^2
"""
import ctypes as C
import math
import os

import numpy as np

from . import abi


def f32(x):
    return float(np.float32(x))


def look_at(pos, target, up):
    """src/transform.cpp:64-90 (look_at), returned float32-exact (the parser
    reads matrices with std::stof)."""
    pos, target, up = (np.asarray(v, np.float64) for v in (pos, target, up))
    d = target - pos
    d = d / np.linalg.norm(d)
    upn = up / np.linalg.norm(up)
    left = np.cross(upn, d)
    left = left / np.linalg.norm(left)
    new_up = np.cross(d, left)
    m = np.zeros((4, 4))
    m[:3, 0] = left
    m[:3, 1] = new_up
    m[:3, 2] = d
    m[:3, 3] = pos
    m[3, 3] = 1
    return m.astype(np.float32).astype(np.float64)


def const_tex(v):
    v = [v, v, v] if np.isscalar(v) else list(v)
    return dict(kind=abi.LJ_TEX_CONST, value0=[f32(x) for x in v])


def checker_tex(c0, c1, uscale=1.0, vscale=1.0):
    c0 = [c0] * 3 if np.isscalar(c0) else list(c0)
    c1 = [c1] * 3 if np.isscalar(c1) else list(c1)
    return dict(kind=abi.LJ_TEX_CHECKER, value0=[f32(x) for x in c0],
                value1=[f32(x) for x in c1], uscale=f32(uscale), vscale=f32(vscale))


def image_tex(image_id, uscale=1.0, vscale=1.0, uoffset=0.0, voffset=0.0):
    return dict(kind=abi.LJ_TEX_IMAGE, image_id=int(image_id), uscale=f32(uscale), vscale=f32(vscale),
                uoffset=f32(uoffset), voffset=f32(voffset))


def rgbe_image(rng, h, w, exponent=128):
    """Random RGB image whose values survive a Radiance RGBE round trip
    exactly: each channel is k * 2^(exponent - 136) with k in [16, 255]
    (the decoder multiplies the byte by 2^(e - 136)).  k >= 16 also keeps
    every scanline from starting with the run-length marker bytes (2, 2)."""
    k = rng.integers(16, 256, size=(h, w, 3))
    return (k * 2.0 ** (exponent - 136)).astype(np.float32)


def rgbe_sky(rng, h, w, exponent=129):
    """Lat-long sky (y up, lajolla's mapping src/lights/envmap.inl:7-20)
    whose texels survive a Radiance RGBE round trip exactly: every channel is
    k * 2^(exponent - 136) with k in [16, 255].  A horizon-to-zenith gradient
    over a dim ground plus a seeded sun lobe at k = 255, 16x the darkest
    texel."""
    u = (np.arange(w) + 0.5) / w
    v = (np.arange(h) + 0.5) / h
    az, el = u * 2 * np.pi, v * np.pi
    dirs = np.stack([np.sin(az)[None, :] * np.sin(el)[:, None], np.cos(el)[:, None] * np.ones((1, w)),
                     -np.cos(az)[None, :] * np.sin(el)[:, None]], axis=-1)
    up = np.clip(dirs[..., 1], 0, 1)[..., None]
    sky = np.where(dirs[..., 1:2] > 0, np.array([120, 110, 100]) * (1 - up) + np.array([40, 70, 150]) * up,
                   np.array([24, 20, 16]))
    sun_el, sun_az = np.radians(rng.uniform(30, 60)), rng.uniform(0, 2 * np.pi)
    sd = np.array([np.sin(sun_az) * np.cos(sun_el), np.sin(sun_el), -np.cos(sun_az) * np.cos(sun_el)])
    lobe = np.exp(-(1 - np.clip(dirs @ sd, -1, 1)) / (1 - np.cos(np.radians(12.0))))[..., None]
    k = np.clip(np.rint(sky + (255 - sky) * lobe), 16, 255)
    return (k * 2.0 ** (exponent - 136)).astype(np.float32)


def write_hdr(path, img):
    """Flat (not run-length encoded) Radiance RGBE file of an image made by
    rgbe_image; row 0 of `img` is the first scanline."""
    img = np.asarray(img, np.float64)
    h, w, _ = img.shape
    m = img.max(axis=2)
    e = np.zeros((h, w), np.int64)
    nz = m > 0
    e[nz] = np.frexp(m[nz])[1] - 8 + 136   # largest channel's byte in [128, 256)
    # the file stores one exponent per pixel: use the image's own one
    ex = int(e[nz].max()) if nz.any() else 128
    k = np.rint(img / 2.0 ** (ex - 136)).astype(np.int64)
    if not np.array_equal(k * 2.0 ** (ex - 136), img) or k.max() > 255:
        raise ValueError("write_hdr: image is not exactly representable with one shared exponent")
    rgbe = np.concatenate([k, np.full((h, w, 1), ex, np.int64)], axis=2).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n")
        f.write(f"-Y {h} +X {w}\n".encode())
        f.write(rgbe.tobytes())


def write_vol(path, data, p_min, p_max):
    """Binary grid volume in the layout lajolla's loader reads
    (src/volume.cpp:6-104): 'VOL', version byte 3, int32 type 1 (FP32),
    int32 x, y, z resolution and channel count, the grid's box as six FP32
    (min xyz, max xyz), then the FP32 voxels, x fastest, channels
    interleaved.  `data` is (z, y, x, channels)."""
    data = np.ascontiguousarray(data, np.float32)
    if data.ndim == 3:
        data = data[..., None]
    nz, ny, nx, ch = data.shape
    with open(path, "wb") as f:
        f.write(b"VOL" + bytes([3]))
        f.write(np.array([1, nx, ny, nz, ch], "<i4").tobytes())
        f.write(np.array(list(p_min) + list(p_max), "<f4").tobytes())
        f.write(data.astype("<f4").tobytes())


def lambertian(rgb):
    return dict(type=abi.LJ_MAT_LAMBERTIAN, eta=1.0, tex=[const_tex(rgb)])


def roughplastic(kd, ks=(1, 1, 1), roughness=0.1, eta=1.49 / 1.000277):
    return dict(type=abi.LJ_MAT_ROUGHPLASTIC, eta=f32(eta),
                tex=[const_tex(kd), const_tex(ks), const_tex(roughness)])


def roughdielectric(ks=(1, 1, 1), kt=(1, 1, 1), roughness=0.1, eta=1.5046 / 1.000277):
    return dict(type=abi.LJ_MAT_ROUGHDIELECTRIC, eta=f32(eta),
                tex=[const_tex(ks), const_tex(kt), const_tex(roughness)])


def disney_bsdf(base_color, specular_transmission=0.0, metallic=0.0, subsurface=0.0,
                specular=0.5, roughness=0.5, specular_tint=0.0, anisotropic=0.0,
                sheen=0.0, sheen_tint=0.5, clearcoat=0.0, clearcoat_gloss=1.0, eta=1.5):
    vals = [specular_transmission, metallic, subsurface, specular, roughness, specular_tint,
            anisotropic, sheen, sheen_tint, clearcoat, clearcoat_gloss]
    return dict(type=abi.LJ_MAT_DISNEY_BSDF, eta=f32(eta),
                tex=[const_tex(base_color)] + [const_tex(v) for v in vals])


class Scene:
    """Flat scene: numpy arrays + dicts, convertible to lj_scene_desc."""

    def __init__(self, width, height, spp, max_depth, cam_to_world, fov,
                 filter_kind=abi.LJ_FILTER_BOX, filter_param=1.0, rr_depth=5,
                 integrator=abi.LJ_INTEGRATOR_PATH, vol_path_version=0,
                 max_null_collisions=1000, camera_medium=-1):
        self.width, self.height = int(width), int(height)
        self.spp, self.max_depth, self.rr_depth = int(spp), int(max_depth), int(rr_depth)
        self.integrator = integrator
        self.vol_path_version = vol_path_version
        self.max_null_collisions = max_null_collisions
        self.cam_to_world = np.asarray(cam_to_world, np.float64)
        self.fov = f32(fov)
        self.filter_kind, self.filter_param = filter_kind, f32(filter_param)
        self.camera_medium = camera_medium
        self.shapes, self.materials, self.lights, self.media, self.images = [], [], [], [], []
        self.envmap_light_id = -1

    # -- building ---------------------------------------------------------
    def add_material(self, m):
        self.materials.append(m)
        return len(self.materials) - 1

    def add_mesh(self, positions, indices, material_id, normals=None, uvs=None,
                 emission=None, interior_medium=-1, exterior_medium=-1):
        sh = dict(kind=abi.LJ_SHAPE_MESH,
                  positions=np.ascontiguousarray(positions, np.float32),
                  indices=np.ascontiguousarray(indices, np.int32),
                  normals=None if normals is None else np.ascontiguousarray(normals, np.float32),
                  uvs=None if uvs is None else np.ascontiguousarray(uvs, np.float32),
                  material_id=material_id, area_light_id=-1,
                  interior_medium_id=interior_medium, exterior_medium_id=exterior_medium)
        return self._add_shape(sh, emission)

    def add_sphere(self, center, radius, material_id, emission=None,
                   interior_medium=-1, exterior_medium=-1):
        sh = dict(kind=abi.LJ_SHAPE_SPHERE, center=[f32(c) for c in center],
                  radius=f32(radius), material_id=material_id, area_light_id=-1,
                  interior_medium_id=interior_medium, exterior_medium_id=exterior_medium)
        return self._add_shape(sh, emission)

    def _add_shape(self, sh, emission):
        sid = len(self.shapes)
        if emission is not None:
            sh["area_light_id"] = len(self.lights)
            self.lights.append(dict(kind=abi.LJ_LIGHT_AREA, shape_id=sid,
                                    intensity=[f32(e) for e in emission]))
        self.shapes.append(sh)
        return sid

    @property
    def num_triangles(self):
        return sum(len(s["indices"]) for s in self.shapes if s["kind"] == abi.LJ_SHAPE_MESH)

    # -- C ABI view -------------------------------------------------------
    def desc(self):
        """Returns (lj_scene_desc, keepalive); keep `keepalive` referenced
        while the descriptor is in use."""
        keep = []

        def ptr(arr, ctype):
            if arr is None:
                return None
            arr = np.ascontiguousarray(arr)
            keep.append(arr)
            return arr.ctypes.data_as(C.POINTER(ctype))

        d = abi.lj_scene_desc()
        cam = d.camera
        for i, v in enumerate(self.cam_to_world.reshape(-1)):
            cam.cam_to_world[i] = v
        cam.fov = self.fov
        cam.width, cam.height = self.width, self.height
        cam.filter_kind, cam.filter_param = self.filter_kind, self.filter_param
        cam.medium_id = self.camera_medium
        o = d.options
        o.integrator, o.samples_per_pixel = self.integrator, self.spp
        o.max_depth, o.rr_depth = self.max_depth, self.rr_depth
        o.vol_path_version, o.max_null_collisions = self.vol_path_version, self.max_null_collisions

        shapes = (abi.lj_shape_desc * max(1, len(self.shapes)))()
        for i, s in enumerate(self.shapes):
            t = shapes[i]
            t.kind, t.material_id, t.area_light_id = s["kind"], s["material_id"], s["area_light_id"]
            t.interior_medium_id, t.exterior_medium_id = s["interior_medium_id"], s["exterior_medium_id"]
            if s["kind"] == abi.LJ_SHAPE_MESH:
                t.num_vertices, t.num_triangles = len(s["positions"]), len(s["indices"])
                t.positions = ptr(s["positions"], C.c_float)
                t.indices = ptr(s["indices"], C.c_int32)
                t.normals = ptr(s["normals"], C.c_float)
                t.uvs = ptr(s["uvs"], C.c_float)
            else:
                for k in range(3):
                    t.center[k] = s["center"][k]
                t.radius = s["radius"]
        mats = (abi.lj_material_desc * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            mats[i].type, mats[i].eta = m["type"], m["eta"]
            for k, tx in enumerate(m["tex"]):
                td = mats[i].tex[k]
                td.kind = tx.get("kind", abi.LJ_TEX_CONST)
                td.image_id = tx.get("image_id", -1)
                for c in range(3):
                    td.value0[c] = tx.get("value0", [0, 0, 0])[c]
                    td.value1[c] = tx.get("value1", [0, 0, 0])[c]
                td.uscale, td.vscale = tx.get("uscale", 1.0), tx.get("vscale", 1.0)
                td.uoffset, td.voffset = tx.get("uoffset", 0.0), tx.get("voffset", 0.0)
        lights = (abi.lj_light_desc * max(1, len(self.lights)))()
        for i, l in enumerate(self.lights):
            t = lights[i]
            t.kind = l["kind"]
            t.shape_id = l.get("shape_id", -1)
            for c in range(3):
                t.intensity[c] = l.get("intensity", [0, 0, 0])[c]
            t.image_id = l.get("image_id", -1)
            t.scale = l.get("scale", 1.0)
            tw = np.asarray(l.get("to_world", np.eye(4)), np.float64).reshape(-1)
            tl = np.asarray(l.get("to_local", np.eye(4)), np.float64).reshape(-1)
            for k in range(16):
                t.to_world[k], t.to_local[k] = tw[k], tl[k]
        images = (abi.lj_image_desc * max(1, len(self.images)))()
        for i, im in enumerate(self.images):
            im = np.ascontiguousarray(im, np.float32)
            if im.ndim == 2:
                im = im[:, :, None]
            images[i].height, images[i].width, images[i].channels = im.shape
            images[i].data = ptr(im, C.c_float)
        media = (abi.lj_medium_desc * max(1, len(self.media)))()
        for i, m in enumerate(self.media):
            t = media[i]
            t.kind, t.phase_kind, t.g = m["kind"], m.get("phase_kind", 0), m.get("g", 0.0)
            for c in range(3):
                t.sigma_a[c] = m.get("sigma_a", [0, 0, 0])[c]
                t.sigma_s[c] = m.get("sigma_s", [0, 0, 0])[c]
            for key in ("albedo", "density"):
                v = m.get(key)
                if v is None:
                    continue
                vd = getattr(t, key)
                vd.kind = v["kind"]
                if v["kind"] == abi.LJ_VOL_CONST:
                    for c in range(3):
                        vd.value[c] = v["value"][c]
                    vd.channels = 3
                else:
                    data = np.ascontiguousarray(v["data"], np.float32)  # (z, y, x, ch)
                    vd.res[0], vd.res[1], vd.res[2] = data.shape[2], data.shape[1], data.shape[0]
                    vd.channels = data.shape[3]
                    for c in range(3):
                        vd.p_min[c], vd.p_max[c] = v["p_min"][c], v["p_max"][c]
                    vd.data = ptr(data, C.c_float)
                vd.scale = v.get("scale", 1.0)
                cs = v.get("channel_scale")
                for c in range(3):
                    vd.channel_scale[c] = 0.0 if cs is None else cs[c]
        d.num_shapes, d.num_materials = len(self.shapes), len(self.materials)
        d.num_lights, d.num_media, d.num_images = len(self.lights), len(self.media), len(self.images)
        d.envmap_light_id = self.envmap_light_id
        d.shapes = C.cast(shapes, C.POINTER(abi.lj_shape_desc))
        d.materials = C.cast(mats, C.POINTER(abi.lj_material_desc))
        d.lights = C.cast(lights, C.POINTER(abi.lj_light_desc))
        d.media = C.cast(media, C.POINTER(abi.lj_medium_desc))
        d.images = C.cast(images, C.POINTER(abi.lj_image_desc))
        keep += [shapes, mats, lights, images, media]
        return d, keep

    # -- Mitsuba XML for the reference renderer ---------------------------
    def write_mitsuba(self, directory, name="scene"):
        """Write <directory>/<name>.xml (+ OBJ meshes) in the subset of the
        Mitsuba 0.5 format lajolla's parser reads
        (src/parsers/parse_scene.cpp).  Supports what the generators emit:
        path integrator, perspective sensor, box filter, diffuse /
        roughplastic / roughdielectric BSDFs, OBJ meshes, spheres, area
        emitters."""
        os.makedirs(directory, exist_ok=True)
        r = repr

        def vec(v):
            return ", ".join(r(float(x)) for x in v)

        for i, im in enumerate(self.images):
            write_hdr(os.path.join(directory, f"{name}_img{i}.hdr"), im)

        def tex(t, pname):
            kind = t.get("kind", abi.LJ_TEX_CONST)
            if kind == abi.LJ_TEX_CONST:
                return [f'    <rgb name="{pname}" value="{vec(t["value0"])}"/>']
            uv = [f'      <float name="{k}" value="{r(float(t.get(k, d)))}"/>'
                  for k, d in (("uscale", 1.0), ("vscale", 1.0), ("uoffset", 0.0), ("voffset", 0.0))]
            if kind == abi.LJ_TEX_CHECKER:
                return ([f'    <texture type="checkerboard" name="{pname}">',
                         f'      <rgb name="color0" value="{vec(t["value0"])}"/>',
                         f'      <rgb name="color1" value="{vec(t["value1"])}"/>'] + uv + ['    </texture>'])
            fn = os.path.join(directory, f'{name}_img{t["image_id"]}.hdr')
            return ([f'    <texture type="bitmap" name="{pname}">',
                     f'      <string name="filename" value="{fn}"/>'] + uv + ['    </texture>'])

        itype = {abi.LJ_INTEGRATOR_PATH: "path", abi.LJ_INTEGRATOR_DEPTH: "depth",
                 abi.LJ_INTEGRATOR_SHADING_NORMAL: "shadingNormal",
                 abi.LJ_INTEGRATOR_MEAN_CURVATURE: "meanCurvature",
                 abi.LJ_INTEGRATOR_RAY_DIFFERENTIAL: "rayDifferential",
                 abi.LJ_INTEGRATOR_MIPMAP_LEVEL: "mipmapLevel"}[self.integrator]
        out = ['<?xml version="1.0" encoding="utf-8"?>', '<scene version="0.4.0">',
               f'  <integrator type="{itype}">',
               f'    <integer name="maxDepth" value="{self.max_depth}"/>',
               f'    <integer name="rrDepth" value="{self.rr_depth}"/>', '  </integrator>',
               '  <sensor type="perspective">',
               f'    <float name="fov" value="{r(self.fov)}"/>',
               '    <transform name="toWorld">',
               '      <matrix value="' + " ".join(r(float(x)) for x in self.cam_to_world.reshape(-1)) + '"/>',
               '    </transform>',
               f'    <sampler type="independent"><integer name="sampleCount" value="{self.spp}"/></sampler>',
               '    <film type="hdrfilm">',
               f'      <integer name="width" value="{self.width}"/>',
               f'      <integer name="height" value="{self.height}"/>']
        if self.filter_kind == abi.LJ_FILTER_BOX:
            out.append(f'      <rfilter type="box"><float name="width" value="{r(self.filter_param)}"/></rfilter>')
        elif self.filter_kind == abi.LJ_FILTER_TENT:
            out.append(f'      <rfilter type="tent"><float name="width" value="{r(self.filter_param)}"/></rfilter>')
        else:
            out.append(f'      <rfilter type="gaussian"><float name="stddev" value="{r(self.filter_param)}"/></rfilter>')
        out += ['    </film>', '  </sensor>']
        for i, m in enumerate(self.materials):
            tx = m["tex"]
            if m["type"] == abi.LJ_MAT_LAMBERTIAN:
                out += [f'  <bsdf type="diffuse" id="mat{i}">'] + tex(tx[0], "reflectance") + ['  </bsdf>']
            elif m["type"] == abi.LJ_MAT_ROUGHPLASTIC:
                out += ([f'  <bsdf type="roughplastic" id="mat{i}">'] + tex(tx[0], "diffuseReflectance") +
                        tex(tx[1], "specularReflectance")) + [
                        f'    <float name="roughness" value="{r(tx[2]["value0"][0])}"/>',
                        f'    <float name="intIOR" value="{r(m["eta"])}"/>',
                        '    <float name="extIOR" value="1"/>', '  </bsdf>']
            elif m["type"] == abi.LJ_MAT_ROUGHDIELECTRIC:
                out += ([f'  <bsdf type="roughdielectric" id="mat{i}">'] + tex(tx[0], "specularReflectance") +
                        tex(tx[1], "specularTransmittance")) + [
                        f'    <float name="roughness" value="{r(tx[2]["value0"][0])}"/>',
                        f'    <float name="intIOR" value="{r(m["eta"])}"/>',
                        '    <float name="extIOR" value="1"/>', '  </bsdf>']
            elif m["type"] == abi.LJ_MAT_DISNEY_CLEARCOAT:
                out += [f'  <bsdf type="disneyclearcoat" id="mat{i}">',
                        f'    <float name="clearcoatGloss" value="{r(tx[0]["value0"][0])}"/>', '  </bsdf>']
            else:
                raise ValueError("write_mitsuba: material type %d not supported" % m["type"])
        for i, s in enumerate(self.shapes):
            if s["kind"] == abi.LJ_SHAPE_MESH:
                fn = os.path.join(directory, f"{name}_shape{i}.obj")
                with open(fn, "w") as f:
                    for p in s["positions"]:
                        f.write("v %r %r %r\n" % tuple(float(x) for x in p))
                    if s["normals"] is not None:
                        for n in s["normals"]:
                            f.write("vn %r %r %r\n" % tuple(float(x) for x in n))
                    if s["uvs"] is not None:
                        # the parser stores (s, 1 - t) (src/parsers/parse_obj.cpp:117-120)
                        for u, v in s["uvs"]:
                            f.write("vt %r %r\n" % (float(u), 1.0 - float(v)))
                    vt = "" if s["uvs"] is None else "%d"
                    vn = "" if s["normals"] is None else "%d"
                    for t in s["indices"]:
                        ids = [int(x) + 1 for x in t]
                        if vt or vn:
                            f.write("f " + " ".join(f"{a}/{vt % a if vt else ''}/{vn % a if vn else ''}"
                                                    for a in ids) + "\n")
                        else:
                            f.write("f %d %d %d\n" % tuple(ids))
                out.append('  <shape type="obj">')
                out.append(f'    <string name="filename" value="{fn}"/>')
                if s["normals"] is None:
                    out.append('    <boolean name="faceNormals" value="true"/>')
            else:
                out.append('  <shape type="sphere">')
                out.append(f'    <point name="center" x="{r(s["center"][0])}" y="{r(s["center"][1])}" z="{r(s["center"][2])}"/>')
                out.append(f'    <float name="radius" value="{r(s["radius"])}"/>')
            out.append(f'    <ref id="mat{s["material_id"]}"/>')
            if s["area_light_id"] >= 0:
                em = self.lights[s["area_light_id"]]["intensity"]
                out.append(f'    <emitter type="area"><rgb name="radiance" value="{vec(em)}"/></emitter>')
            out.append('  </shape>')
        # the parser numbers lights in document order (area lights with their
        # shapes), so the envmap, the last light here, comes after the shapes
        if self.envmap_light_id >= 0:
            if self.envmap_light_id != len(self.lights) - 1:
                raise ValueError("write_mitsuba: the envmap must be the last light")
            l = self.lights[self.envmap_light_id]
            fn = os.path.join(directory, f'{name}_img{l["image_id"]}.hdr')
            out += ['  <emitter type="envmap">', f'    <string name="filename" value="{fn}"/>',
                    '    <transform name="toWorld">',
                    '      <matrix value="' + " ".join(r(float(x)) for x in np.asarray(l["to_world"]).reshape(-1))
                    + '"/>', '    </transform>', f'    <float name="scale" value="{r(float(l.get("scale", 1.0)))}"/>',
                    '  </emitter>']
        out.append('</scene>')
        path = os.path.join(directory, f"{name}.xml")
        with open(path, "w") as f:
            f.write("\n".join(out) + "\n")
        return path


def _quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3); normal = (p1-p0) x (p2-p0)."""
    return np.array([p0, p1, p2, p3], np.float32), np.array([[0, 1, 2], [0, 2, 3]], np.int32)


def _box(center, size, angle_deg):
    """Axis box rotated about +y; 12 outward-facing triangles."""
    cx, cy, cz = center
    sx, sy, sz = (s / 2 for s in size)
    c, s = math.cos(math.radians(angle_deg)), math.sin(math.radians(angle_deg))

    def P(x, y, z):
        return [cx + c * x + s * z, cy + y, cz - s * x + c * z]

    corners = {}
    for ix in (-1, 1):
        for iy in (-1, 1):
            for iz in (-1, 1):
                corners[(ix, iy, iz)] = P(ix * sx, iy * sy, iz * sz)
    faces = [  # each CCW seen from outside
        [(-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)],      # +z
        [(1, -1, -1), (-1, -1, -1), (-1, 1, -1), (1, 1, -1)],  # -z
        [(1, -1, 1), (1, -1, -1), (1, 1, -1), (1, 1, 1)],      # +x
        [(-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1)],  # -x
        [(-1, 1, 1), (1, 1, 1), (1, 1, -1), (-1, 1, -1)],      # +y
        [(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)],  # -y
    ]
    pos, idx = [], []
    for f in faces:
        b = len(pos)
        pos += [corners[k] for k in f]
        idx += [[b, b + 1, b + 2], [b, b + 2, b + 3]]
    return np.array(pos, np.float32), np.array(idx, np.int32)


def cornell_box(seed=0, width=256, height=256, spp=64, max_depth=6, rr_depth=5):
    """Seeded Cornell-like box: interior [-1,1] x [0,2] x [-1,1], open at +z."""
    rng = np.random.default_rng(seed)
    sc = Scene(width, height, spp, max_depth,
               look_at([0, 1, 3.4], [0, 1, 0], [0, 1, 0]), 40.0, rr_depth=rr_depth)

    def albedo():
        return [f32(x) for x in rng.uniform(0.1, 0.8, 3)]

    walls = [
        _quad([-1, 0, 1], [1, 0, 1], [1, 0, -1], [-1, 0, -1]),      # floor, normal +y
        _quad([-1, 2, -1], [1, 2, -1], [1, 2, 1], [-1, 2, 1]),      # ceiling, normal -y
        _quad([-1, 0, -1], [1, 0, -1], [1, 2, -1], [-1, 2, -1]),    # back, normal +z
        _quad([-1, 0, 1], [-1, 0, -1], [-1, 2, -1], [-1, 2, 1]),    # left, normal +x
        _quad([1, 0, -1], [1, 0, 1], [1, 2, 1], [1, 2, -1]),        # right, normal -x
    ]
    for pos, idx in walls:
        sc.add_mesh(pos, idx, sc.add_material(lambertian(albedo())))
    a1, a2 = (float(x) for x in rng.uniform(10, 35, 2))
    for center, size, ang in (([-0.35, 0.6, -0.3], [0.6, 1.2, 0.6], a1),
                              ([0.4, 0.3, 0.3], [0.6, 0.6, 0.6], -a2)):
        pos, idx = _box(center, size, ang)
        sc.add_mesh(pos, idx, sc.add_material(lambertian(albedo())))
    lpos, lidx = _quad([-0.25, 1.98, -0.25], [0.25, 1.98, -0.25], [0.25, 1.98, 0.25], [-0.25, 1.98, 0.25])
    sc.add_mesh(lpos, lidx, sc.add_material(lambertian([0.78, 0.78, 0.78])), emission=[17, 12, 4])
    return sc


def textured_scene(seed=0, width=64, height=64, spp=16, max_depth=6, integrator=abi.LJ_INTEGRATOR_PATH,
                   clearcoat=True):
    """Cornell box with textures and curved surfaces: an image-textured floor
    (dyadic UVs, so the OBJ round trip is exact), a checkerboard back wall,
    a smooth-shaded icosphere mesh (vertex normals: non-zero mean
    curvature), an image-textured analytic sphere and, with `clearcoat`, a
    DisneyClearcoat box (a material without a spectrum texture)."""
    rng = np.random.default_rng(seed)
    sc = cornell_box(seed=seed, width=width, height=height, spp=spp, max_depth=max_depth)
    sc.integrator = integrator
    sc.images.append(rgbe_image(rng, 32, 64))
    sc.images.append(rgbe_image(rng, 16, 16))
    floor, back, box2 = sc.shapes[0], sc.shapes[2], sc.shapes[6]
    floor["uvs"] = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    sc.materials[floor["material_id"]] = dict(type=abi.LJ_MAT_LAMBERTIAN, eta=1.0,
                                             tex=[image_tex(0, uscale=2.0, vscale=3.0, uoffset=0.25)])
    back["uvs"] = np.array([[0, 0], [0.5, 0], [0.5, 0.75], [0, 0.75]], np.float32)
    sc.materials[back["material_id"]] = dict(type=abi.LJ_MAT_LAMBERTIAN, eta=1.0,
                                            tex=[checker_tex([0.7, 0.2, 0.2], [0.2, 0.2, 0.7], 4.0, 4.0)])
    if clearcoat:
        sc.materials[box2["material_id"]] = dict(type=abi.LJ_MAT_DISNEY_CLEARCOAT, eta=1.5, tex=[const_tex(0.7)])
    v, f = icosphere(2)
    r = 0.3
    sc.add_mesh(v * r + np.array([0.45, 0.9, 0.3]), f, sc.add_material(lambertian([0.6, 0.6, 0.3])),
                normals=v)
    sc.add_sphere([-0.35, 1.45, -0.3], 0.22, sc.add_material(dict(type=abi.LJ_MAT_LAMBERTIAN, eta=1.0,
                                                                  tex=[image_tex(1, 3.0, 2.0)])))
    return sc


def envmap_scene(seed=0, width=64, height=48, spp=16, max_depth=6, with_area_light=True):
    """Seeded outdoor scene lit by a rotated HDR envmap (scale 2, an
    RGBE-exact sky from rgbe_sky) and, with `with_area_light`, a small quad
    light: a Lambertian ground quad, a RoughPlastic analytic sphere, a
    Lambertian box and a smooth-shaded RoughPlastic icosphere.  The camera
    sees the sky above the horizon, so the miss path's emission shows."""
    rng = np.random.default_rng(seed)
    sc = Scene(width, height, spp, max_depth, look_at([0.4, 1.2, 4.0], [0, 0.6, 0], [0, 1, 0]), 50.0)
    ground = sc.add_material(lambertian([f32(x) for x in rng.uniform(0.3, 0.7, 3)]))
    sc.add_mesh(*_quad([-4, 0, 4], [4, 0, 4], [4, 0, -4], [-4, 0, -4]), ground)
    plastic = sc.add_material(roughplastic([f32(x) for x in rng.uniform(0.2, 0.8, 3)], [0.8, 0.8, 0.8],
                                           f32(rng.uniform(0.05, 0.3)), 1.5))
    sc.add_sphere([-0.7, 0.5, 0.2], 0.5, plastic)
    pos, idx = _box([0.7, 0.35, -0.3], [0.7, 0.7, 0.7], float(rng.uniform(10, 40)))
    sc.add_mesh(pos, idx, sc.add_material(lambertian([f32(x) for x in rng.uniform(0.2, 0.8, 3)])))
    v, f = icosphere(2)
    sc.add_mesh(v * 0.3 + np.array([0.2, 0.3, 0.9]), f,
                sc.add_material(roughplastic([0.3, 0.5, 0.7], [0.9, 0.9, 0.9], 0.2, 1.45)), normals=v)
    if with_area_light:
        lpos, lidx = _quad([1.2, 2.0, 0.5], [1.6, 2.0, 0.5], [1.6, 2.0, 0.1], [1.2, 2.0, 0.1])
        sc.add_mesh(lpos, lidx, sc.add_material(lambertian([0.5, 0.5, 0.5])), emission=[12, 10, 8])
    sc.images.append(rgbe_sky(rng, 32, 64))
    # FP32 entries: lajolla's parser reads matrices with std::stof
    tw = _rotation(float(rng.uniform(20, 70)), [0.1, 1.0, 0.2]).astype(np.float32).astype(np.float64)
    sc.lights.append(dict(kind=abi.LJ_LIGHT_ENVMAP, image_id=len(sc.images) - 1, scale=2.0, to_world=tw,
                          to_local=np.linalg.inv(tw)))
    sc.envmap_light_id = len(sc.lights) - 1
    return sc


def _rotation(angle_deg, axis):
    """4x4 rotation about `axis` (src/transform.cpp:21-56's rotate)."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    s, c = np.sin(np.radians(angle_deg)), np.cos(np.radians(angle_deg))
    m = np.eye(4)
    m[:3, :3] = c * np.eye(3) + (1 - c) * np.outer(a, a) + s * np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]],
                                                                         [-a[1], a[0], 0]])
    return m


def triangle_soup(seed, n_tris, offset_sigma=0.01):
    """n triangles: centroids U[0,1]^3, each vertex = centroid + N(0, sigma)."""
    rng = np.random.default_rng(seed)
    cent = rng.uniform(0, 1, (n_tris, 1, 3))
    v = (cent + rng.normal(0, offset_sigma, (n_tris, 3, 3))).astype(np.float32)
    return v.reshape(-1, 3), np.arange(n_tris * 3, dtype=np.int32).reshape(-1, 3)


def tied_soup_scene(seed, n_tris):
    """Every soup triangle twice (the copies far apart in index order) plus
    coplanar quads facing both ways: many rays see two or more primitives at
    exactly the same distance."""
    sc = Scene(8, 8, 1, 1, np.eye(4), 45.0)
    rng = np.random.default_rng(seed)
    v, _ = triangle_soup(seed, n_tris)
    tri = v.reshape(n_tris, 3, 3)
    pos = np.concatenate([tri, tri[rng.permutation(n_tris)]]).reshape(-1, 3)
    m = sc.add_material(lambertian([0.5, 0.5, 0.5]))
    sc.add_mesh(pos, np.arange(len(pos), dtype=np.int32).reshape(-1, 3), m)
    for z in (0.25, 0.5, 0.75):
        q = np.array([[0, 0, z], [1, 0, z], [1, 1, z], [0, 1, z]], np.float32)
        sc.add_mesh(q, np.array([[0, 1, 2], [0, 2, 3]], np.int32), m)
        sc.add_mesh(q[::-1].copy(), np.array([[0, 1, 2], [0, 2, 3]], np.int32), m)
    return sc


def soup_scene(seed, n_tris):
    """A scene wrapping a triangle soup (one Lambertian mesh, one light)."""
    pos, idx = triangle_soup(seed, n_tris)
    sc = Scene(64, 64, 1, 2, look_at([0.5, 0.5, 3], [0.5, 0.5, 0.5], [0, 1, 0]), 40.0)
    m = sc.add_material(lambertian([0.5, 0.5, 0.5]))
    sc.add_mesh(pos, idx, m)
    return sc


def value_noise_2d(rng, nx, nz, octaves=5, base_cells=8):
    """Seeded fractal value noise on an (nz, nx) grid in [0, 1]: random
    lattice values, smoothstep-interpolated, octaves summed with gain 1/2."""
    h = np.zeros((nz, nx))
    amp, total = 1.0, 0.0
    xs, zs = np.linspace(0, 1, nx), np.linspace(0, 1, nz)
    for o in range(octaves):
        cells = base_cells * (2 ** o)
        lat = rng.uniform(0, 1, (cells + 2, cells + 2))
        fx, fz = xs * cells, zs * cells
        ix, iz = np.floor(fx).astype(int), np.floor(fz).astype(int)
        tx, tz = fx - ix, fz - iz
        tx, tz = tx * tx * (3 - 2 * tx), tz * tz * (3 - 2 * tz)
        a = lat[iz[:, None], ix[None, :]]
        b = lat[iz[:, None], ix[None, :] + 1]
        c = lat[iz[:, None] + 1, ix[None, :]]
        d = lat[iz[:, None] + 1, ix[None, :] + 1]
        top = a + (b - a) * tx[None, :]
        bot = c + (d - c) * tx[None, :]
        h += amp * (top + (bot - top) * tz[:, None])
        total += amp
        amp *= 0.5
    return h / total


def terrain_mesh(rng, nx, nz, size_x, size_z, height):
    """(nx x nz) quads -> 2 nx nz triangles, smooth vertex normals."""
    vx, vz = nx + 1, nz + 1
    hgt = value_noise_2d(rng, vx, vz) * height
    xs = np.linspace(-size_x / 2, size_x / 2, vx)
    zs = np.linspace(-size_z / 2, size_z / 2, vz)
    X, Z = np.meshgrid(xs, zs)
    pos = np.stack([X, hgt, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    gz, gx = np.gradient(hgt, zs, xs)
    n = np.stack([-gx, np.ones_like(gx), -gz], axis=-1).reshape(-1, 3)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    i = np.arange(nz)[:, None] * vx + np.arange(nx)[None, :]
    i = i.reshape(-1)
    # counter-clockwise seen from +y: normal (e1 x e2) points up
    t0 = np.stack([i, i + vx, i + 1], axis=1)
    t1 = np.stack([i + 1, i + vx, i + vx + 1], axis=1)
    idx = np.concatenate([t0, t1], axis=0).astype(np.int32)
    return pos, idx, n.astype(np.float32)


def icosphere(subdiv):
    """Unit icosphere: 20 * 4^subdiv triangles, outward winding."""
    t = (1 + 5 ** 0.5) / 2
    v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
         [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
         [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = f
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        faces = nf
    return np.array(verts, np.float64), np.array(faces, np.int32)


def sky_envmap(rng, w, h, sun_peak=5e3):
    """Procedural HDR lat-long sky (y up, lajolla's mapping envmap.inl:7-20):
    blue-to-white gradient over a dark ground plus a Gaussian sun lobe."""
    u = (np.arange(w) + 0.5) / w
    v = (np.arange(h) + 0.5) / h
    az, el = u * 2 * np.pi, v * np.pi
    dirs = np.stack([np.sin(az)[None, :] * np.sin(el)[:, None],
                     np.cos(el)[:, None] * np.ones((1, w)),
                     -np.cos(az)[None, :] * np.sin(el)[:, None]], axis=-1)
    up = np.clip(dirs[..., 1], 0, 1)
    horizon = np.array([0.9, 0.85, 0.8])
    zenith = np.array([0.2, 0.35, 0.8])
    sky = horizon * (1 - up[..., None]) + zenith * up[..., None]
    sky = np.where(dirs[..., 1:2] > 0, sky, np.array([0.05, 0.04, 0.03]))
    sun_el = np.radians(rng.uniform(25, 50))
    sun_az = rng.uniform(0, 2 * np.pi)
    sd = np.array([np.sin(sun_az) * np.sin(np.pi / 2 - sun_el), np.cos(np.pi / 2 - sun_el),
                   -np.cos(sun_az) * np.sin(np.pi / 2 - sun_el)])
    cosang = np.clip(dirs @ sd, -1, 1)
    lobe = np.exp(-(1 - cosang) / (1 - np.cos(np.radians(1.5))))
    sky = sky * 2 + sun_peak * lobe[..., None] * np.array([1.0, 0.95, 0.85])
    return sky.astype(np.float32)


def terrain_scene(seed=0, width=1920, height=1080, spp=256, max_depth=8, grid=(2048, 1024),
                  n_spheres=64, sphere_subdiv=5, env_size=(1024, 512)):
    """Seeded large-mesh scene: fractal terrain + icospheres with Disney BSDFs
    (roughness U[0.05,1], metallic Bernoulli(0.3), base color U[0,1]^3) under
    a procedural HDR envmap sampled through the 2D table."""
    rng = np.random.default_rng(seed)
    sx, sz, hh = 40.0, 20.0, 3.0
    sc = Scene(width, height, spp, max_depth,
               look_at([0, 7.5, 16], [0, 1.0, -2], [0, 1, 0]), 50.0)

    def disney():
        return disney_bsdf(rng.uniform(0, 1, 3), metallic=float(rng.uniform() < 0.3),
                           roughness=rng.uniform(0.05, 1.0))
    pos, idx, nrm = terrain_mesh(rng, grid[0], grid[1], sx, sz, hh)
    sc.add_mesh(pos, idx, sc.add_material(disney()), normals=nrm)
    hmap = pos.reshape(grid[1] + 1, grid[0] + 1, 3)
    uv, uf = icosphere(sphere_subdiv)
    for _ in range(n_spheres):
        r = rng.uniform(0.25, 0.8)
        gx, gz = rng.integers(0, grid[0] + 1), rng.integers(0, grid[1] // 2 + 1) + grid[1] // 4
        c = hmap[gz, gx] + np.array([0, r * 0.9, 0])
        p = (uv * r + c).astype(np.float32)
        sc.add_mesh(p, uf, sc.add_material(disney()), normals=uv.astype(np.float32))
    sc.images.append(sky_envmap(rng, env_size[0], env_size[1]))
    sc.lights.append(dict(kind=abi.LJ_LIGHT_ENVMAP, image_id=len(sc.images) - 1, scale=1.0,
                          to_world=np.eye(4), to_local=np.eye(4)))
    sc.envmap_light_id = len(sc.lights) - 1
    return sc


def value_noise_3d(rng, n, octaves=5, base_cells=4):
    """Seeded fractal value noise on an n^3 grid (z, y, x) in [0, 1]."""
    g = np.linspace(0, 1, n)
    out = np.zeros((n, n, n), np.float32)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = base_cells * (2 ** o)
        lat = rng.uniform(0, 1, (cells + 2,) * 3).astype(np.float32)
        f = g * cells
        i = np.floor(f).astype(int)
        t = (f - i).astype(np.float32)
        t = t * t * (3 - 2 * t)
        acc = np.zeros((n, n, n), np.float32)
        for dz in (0, 1):
            wz = t if dz else 1 - t
            for dy in (0, 1):
                wy = t if dy else 1 - t
                for dx in (0, 1):
                    wx = t if dx else 1 - t
                    v = lat[(i + dz)[:, None, None], (i + dy)[None, :, None], (i + dx)[None, None, :]]
                    acc += v * (wz[:, None, None] * wy[None, :, None] * wx[None, None, :])
        out += amp * acc
        total += amp
        amp *= 0.5
    return out / total


def volume_scene(seed=0, width=512, height=512, spp=256, max_depth=64, grid=256, max_density=20.0,
                 sigma_t_scale=(1.05, 0.9, 0.8), albedo=(0.952, 0.889, 0.75), g=0.7,
                 eta=1.33, roughness=0.1, floor_grid=1):
    """Seeded volumetric scene: a heterogeneous chromatic medium (5-octave
    value noise scaled to `max_density` as a one-channel FP32 density grid,
    sigma_t = sigma_t_scale * density through the grid's channel scale,
    constant albedo, HG g) inside a rough dielectric sphere, over a diffuse
    plane (split into floor_grid^2 quads), lit by one sphere area light."""
    rng = np.random.default_rng(seed)
    sc = Scene(width, height, spp, max_depth, look_at([0, 1.4, 4.2], [0, 0.9, 0], [0, 1, 0]), 35.0,
               integrator=abi.LJ_INTEGRATOR_VOLPATH, vol_path_version=6)
    noise = value_noise_3d(rng, grid)
    noise = noise - noise.min()
    noise = noise / noise.max() * max_density
    dens = noise[..., None].astype(np.float32)
    c, r = np.array([0.0, 1.0, 0.0]), 1.0
    sc.media.append(dict(kind=abi.LJ_MEDIUM_HETEROGENEOUS, phase_kind=abi.LJ_PHASE_HG, g=f32(g),
                         albedo=dict(kind=abi.LJ_VOL_CONST, value=[f32(a) for a in albedo]),
                         density=dict(kind=abi.LJ_VOL_GRID, data=dens, p_min=[f32(x) for x in c - r],
                                      p_max=[f32(x) for x in c + r],
                                      channel_scale=[f32(x) for x in sigma_t_scale])))
    diel = sc.add_material(roughdielectric([1, 1, 1], [1, 1, 1], roughness, eta))
    sc.add_sphere(c, r, diel, interior_medium=0, exterior_medium=-1)
    floor_m = sc.add_material(lambertian([0.6, 0.6, 0.6]))
    corners = ([-6, 0, 6], [6, 0, 6], [6, 0, -6], [-6, 0, -6])
    fpos, fidx = _quad(*corners) if floor_grid <= 1 else _subdivide_quad(*corners, floor_grid)
    sc.add_mesh(fpos, fidx, floor_m)
    lm = sc.add_material(lambertian([0.0, 0.0, 0.0]))
    sc.add_sphere([2.0, 3.5, 1.5], 0.5, lm, emission=[30, 28, 25])
    return sc


def homogeneous_box_scene(width=32, height=32, spp=16, max_depth=16, sigma_a=(0.3, 0.6, 0.9),
                          sigma_s=(1.2, 0.8, 0.5), g=0.5, index_matched=True):
    """Small test scene: a chromatic homogeneous medium inside a unit box
    (index-matching if `index_matched`, else a rough dielectric), over a
    diffuse floor, lit by a quad light."""
    sc = Scene(width, height, spp, max_depth, look_at([0, 1.2, 3.5], [0, 0.6, 0], [0, 1, 0]), 40.0,
               integrator=abi.LJ_INTEGRATOR_VOLPATH, vol_path_version=6)
    sc.media.append(dict(kind=abi.LJ_MEDIUM_HOMOGENEOUS, phase_kind=abi.LJ_PHASE_HG, g=f32(g),
                         sigma_a=[f32(x) for x in sigma_a], sigma_s=[f32(x) for x in sigma_s]))
    pos, idx = _box([0, 0.6, 0], [1.0, 1.0, 1.0], 20.0)
    m = -1 if index_matched else sc.add_material(roughdielectric([1, 1, 1], [1, 1, 1], 0.2, 1.33))
    sc.add_mesh(pos, idx, m, interior_medium=0, exterior_medium=-1)
    fm = sc.add_material(lambertian([0.5, 0.5, 0.5]))
    fpos, fidx = _quad([-3, 0, 3], [3, 0, 3], [3, 0, -3], [-3, 0, -3])
    sc.add_mesh(fpos, fidx, fm)
    lpos, lidx = _quad([-0.5, 2.5, -0.5], [0.5, 2.5, -0.5], [0.5, 2.5, 0.5], [-0.5, 2.5, 0.5])
    sc.add_mesh(lpos, lidx, sc.add_material(lambertian([0, 0, 0])), emission=[8, 8, 8])
    return sc


def random_rays(seed, n, tnear=0.0, tfar=np.inf):
    """Rays as an (n, 8) float32 array in lj_ray layout."""
    rng = np.random.default_rng(seed)
    org = rng.uniform(-0.5, 1.5, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.empty((n, 8), np.float32)
    r[:, 0:3] = org
    r[:, 3] = tnear
    r[:, 4:7] = d
    r[:, 7] = tfar
    return r


# ---- serving workload (Poisson-arriving render jobs over resident scenes) ----
def _subdivide_quad(p0, p1, p2, p3, k):
    """k x k grid over the quad (p0, p1, p2, p3); same winding as _quad."""
    p0, p1, p2, p3 = (np.asarray(p, np.float64) for p in (p0, p1, p2, p3))
    t = np.linspace(0.0, 1.0, k + 1)
    a = p0[None, :] * (1 - t)[:, None] + p1[None, :] * t[:, None]     # p0 -> p1
    b = p3[None, :] * (1 - t)[:, None] + p2[None, :] * t[:, None]     # p3 -> p2
    pos = a[None, :, :] * (1 - t)[:, None, None] + b[None, :, :] * t[:, None, None]   # [row j][col i]
    idx = []
    for j in range(k):
        for i in range(k):
            v00, v01 = j * (k + 1) + i, j * (k + 1) + i + 1
            v10, v11 = (j + 1) * (k + 1) + i, (j + 1) * (k + 1) + i + 1
            idx += [[v00, v01, v11], [v00, v11, v10]]
    return pos.reshape(-1, 3).astype(np.float32), np.array(idx, np.int32)


def tessellated_cornell_box(seed=0, n_tris=10000, width=256, height=256, spp=64, max_depth=6):
    """The seeded Cornell box with each wall quad split into a k x k grid so
    that the scene holds about n_tris triangles (same surfaces)."""
    sc = cornell_box(seed=seed, width=width, height=height, spp=spp, max_depth=max_depth)
    k = max(1, int(round(math.sqrt(max(1, n_tris - 26) / 10.0))))
    for w in range(5):
        pos = sc.shapes[w]["positions"]
        p, i = _subdivide_quad(pos[0], pos[1], pos[2], pos[3], k)
        sc.shapes[w]["positions"], sc.shapes[w]["indices"] = p, i
    return sc


def resized_terrain_scene(seed=0, n_tris=500000, width=256, height=256, spp=64, max_depth=8,
                          env_size=(256, 128)):
    """terrain_scene with its grid and sphere count scaled to about n_tris
    triangles (16 subdivision-3 icospheres, the rest terrain)."""
    n_spheres, subdiv = 16, 3
    rest = max(2000, n_tris - n_spheres * 20 * 4 ** subdiv)
    nz = max(8, int(round(math.sqrt(rest / 4.0))))
    return terrain_scene(seed=seed, width=width, height=height, spp=spp, max_depth=max_depth,
                         grid=(2 * nz, nz), n_spheres=n_spheres, sphere_subdiv=subdiv, env_size=env_size)


def with_three_channel_density(sc):
    """The same scene with every one-channel density grid that carries a
    channel scale stored as three channels (data * channel scale per voxel,
    FP32) and no channel scale: the reference's representation of a
    chromatic grid."""
    for m in sc.media:
        d = m.get("density")
        if d is None or d.get("data") is None or d.get("channel_scale") is None:
            continue
        data = np.asarray(d["data"], np.float32)
        if data.shape[-1] != 1:
            continue
        cs = np.asarray(d["channel_scale"], np.float32)
        d["data"] = (data * cs).astype(np.float32)
        d["channel_scale"] = None
    return sc


def resized_volume_scene(seed=0, n_tris=10000, width=256, height=256, spp=64, max_depth=64, grid=256):
    """volume_scene with its floor split into about n_tris triangles."""
    return volume_scene(seed=seed, width=width, height=height, spp=spp, max_depth=max_depth, grid=grid,
                        floor_grid=max(1, int(round(math.sqrt(n_tris / 2.0)))))


def serving_scenes(seed=0, n_scenes=6, min_tris=10000, max_tris=2000000, volume_grid=256):
    """Scene pool of the serving workload: Cornell-box, terrain and
    volumetric scenes in turn, with triangle counts log-uniform in
    [min_tris, max_tris]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenes):
        t = int(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris))))
        if k % 3 == 0:
            out.append(tessellated_cornell_box(seed=seed * 100 + k, n_tris=t))
        elif k % 3 == 1:
            out.append(resized_terrain_scene(seed=seed * 100 + k, n_tris=t))
        else:
            out.append(resized_volume_scene(seed=seed * 100 + k, n_tris=t, grid=volume_grid))
    return out


def serving_jobs(seed=0, n_jobs=32, n_scenes=6, rate=200.0, resolutions=(128, 256, 512, 1024),
                 spps=(4, 16, 64, 256), depth=(6, 64)):
    """Poisson arrivals (mean `rate` per second), scene uniform over the pool,
    square resolution, spp and max depth (RR from depth 5) uniform over the
    given choices.  Returns a list of dicts sorted by arrival time."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n_jobs))
    t -= t[0]
    jobs = []
    for k in range(n_jobs):
        r = int(rng.choice(resolutions))
        jobs.append(dict(arrival_s=float(t[k]), scene=int(rng.integers(n_scenes)), width=r, height=r,
                         spp=int(rng.choice(spps)), max_depth=int(rng.integers(depth[0], depth[1] + 1)),
                         rr_depth=5, seed=int(rng.integers(1 << 40))))
    return jobs
