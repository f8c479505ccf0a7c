// ORACLE / TEST INFRASTRUCTURE -- not part of the product.
//
// Drives the reference-side adapter (lajolla_public_gb300/adapter/render_gpu.cpp)
// with the UNMODIFIED reference parser, linked against liblj_gpu.so (see
// Makefile, target `adapter`; development container only).
//
//   adapter_check flatten scene.xml out.flat
//       parse_scene (src/parsers/parse_scene.cpp) -> flatten_scene ->
//       lj_gpu_scene_validate (no device); writes the flattened descriptor
//       (layout below) for tests/ljtest.py's load_flat.  Exit 3 and the
//       reason on stderr if the library refuses the scene.
//   adapter_check write in.pfm out.(pfm|exr)
//       an FP32 HWC image (read from a PFM as lajolla writes it) through
//       image_from_rgb and the reference's imwrite (src/image.cpp:135-173).
//   adapter_check render scene.xml out.(pfm|exr)
//       parse_scene -> render_gpu -> imwrite (needs a GB300).
//
// Flattened layout, little-endian: "LJF1"; the lj_scene_desc (pointers
// zeroed); per shape its lj_shape_desc (pointers zeroed), int32 has_normals,
// int32 has_uvs, then positions, indices, normals, uvs; each
// lj_material_desc; each lj_light_desc; per image its lj_image_desc and the
// pixels; per medium its lj_medium_desc and the grid data of albedo, then
// density (grids only).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "parsers/parse_scene.h"
#include "render_gpu.h"

namespace {

struct Out {
    FILE *f;
    void raw(const void *p, size_t n) { fwrite(p, 1, n, f); }
    template <typename T>
    void pod(T v) { raw(&v, sizeof(T)); }
};

template <typename T>
T nulled(T v);
template <>
lj_scene_desc nulled(lj_scene_desc d) {
    d.shapes = nullptr; d.materials = nullptr; d.lights = nullptr; d.media = nullptr; d.images = nullptr;
    return d;
}
template <>
lj_shape_desc nulled(lj_shape_desc d) {
    d.positions = nullptr; d.indices = nullptr; d.normals = nullptr; d.uvs = nullptr;
    return d;
}
template <>
lj_image_desc nulled(lj_image_desc d) {
    d.data = nullptr;
    return d;
}
template <>
lj_medium_desc nulled(lj_medium_desc d) {
    d.albedo.data = nullptr;
    d.density.data = nullptr;
    return d;
}

void write_volume_data(Out &o, const lj_volume_desc &v) {
    if (v.kind != LJ_VOL_GRID) return;
    o.raw(v.data, sizeof(float) * (size_t)v.res[0] * v.res[1] * v.res[2] * v.channels);
}

int flatten(const char *xml, const char *out_path) {
    RTCDevice dev = rtcNewDevice(nullptr);
    std::unique_ptr<Scene> scene = parse_scene(xml, dev);
    LjFlatScene flat;
    flatten_scene(*scene, flat);
    char msg[512];
    if (lj_gpu_scene_validate(&flat.desc, msg, sizeof(msg)) != LJ_OK) {
        fprintf(stderr, "invalid: %s\n", msg);
        return 3;
    }
    Out o{fopen(out_path, "wb")};
    if (!o.f) { perror(out_path); return 1; }
    const lj_scene_desc &d = flat.desc;
    o.raw("LJF1", 4);
    o.pod(nulled(d));
    for (int i = 0; i < d.num_shapes; i++) {
        const lj_shape_desc &s = d.shapes[i];
        o.pod(nulled(s));
        o.pod((int32_t)(s.normals != nullptr));
        o.pod((int32_t)(s.uvs != nullptr));
        if (s.kind != LJ_SHAPE_MESH) continue;
        o.raw(s.positions, sizeof(float) * 3 * s.num_vertices);
        o.raw(s.indices, sizeof(int32_t) * 3 * s.num_triangles);
        if (s.normals) o.raw(s.normals, sizeof(float) * 3 * s.num_vertices);
        if (s.uvs) o.raw(s.uvs, sizeof(float) * 2 * s.num_vertices);
    }
    for (int i = 0; i < d.num_materials; i++) o.pod(d.materials[i]);
    for (int i = 0; i < d.num_lights; i++) o.pod(d.lights[i]);
    for (int i = 0; i < d.num_images; i++) {
        const lj_image_desc &im = d.images[i];
        o.pod(nulled(im));
        o.raw(im.data, sizeof(float) * (size_t)im.width * im.height * im.channels);
    }
    for (int i = 0; i < d.num_media; i++) {
        const lj_medium_desc &m = d.media[i];
        o.pod(nulled(m));
        write_volume_data(o, m.albedo);
        write_volume_data(o, m.density);
    }
    fclose(o.f);
    rtcReleaseDevice(dev);
    return 0;
}

// PFM as src/image.cpp:137-149 writes it: "PF", "w h", "-1", then the
// pixels in the Image3's own row order.
bool read_pfm(const char *path, std::vector<float> &px, int &w, int &h) {
    std::ifstream f(path, std::ios::binary);
    std::string tag;
    double scale;
    if (!(f >> tag >> w >> h >> scale) || tag != "PF") return false;
    f.get();
    px.resize((size_t)w * h * 3);
    f.read((char *)px.data(), px.size() * sizeof(float));
    return (bool)f;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc == 4 && std::string(argv[1]) == "flatten") return flatten(argv[2], argv[3]);
    if (argc == 4 && std::string(argv[1]) == "write") {
        std::vector<float> px;
        int w = 0, h = 0;
        if (!read_pfm(argv[2], px, w, h)) {
            fprintf(stderr, "cannot read %s\n", argv[2]);
            return 1;
        }
        imwrite(argv[3], image_from_rgb(px.data(), w, h));
        return 0;
    }
    if (argc == 4 && std::string(argv[1]) == "render") {
        RTCDevice dev = rtcNewDevice(nullptr);
        std::unique_ptr<Scene> scene = parse_scene(argv[2], dev);
        imwrite(argv[3], render_gpu(*scene));
        rtcReleaseDevice(dev);
        return 0;
    }
    fprintf(stderr, "usage: adapter_check flatten scene.xml out.flat | write in.pfm out.(pfm|exr) | "
                    "render scene.xml out.(pfm|exr)\n");
    return 2;
}
