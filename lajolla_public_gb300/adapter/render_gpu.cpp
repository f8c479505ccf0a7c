// render_gpu.cpp -- flattens lajolla's Scene into lj_scene_desc and renders
// it with liblj_gpu.so (see render_gpu.h).
#include "render_gpu.h"

#include <cmath>
#include <map>
#include <mutex>
#include <stdexcept>
#include <type_traits>
#include <variant>

namespace {

struct Flattener {
    LjFlatScene &f;
    const TexturePool &pool;
    std::map<int, int> img3, img1;   // texture pool id -> flat image index

    const float *keep(std::vector<float> v) {
        f.floats.push_back(std::move(v));
        return f.floats.back().data();
    }
    const int32_t *keep(std::vector<int32_t> v) {
        f.ints.push_back(std::move(v));
        return f.ints.back().data();
    }

    int add_image(const Image3 &img) {
        std::vector<float> px(img.data.size() * 3);
        for (size_t i = 0; i < img.data.size(); i++)
            for (int c = 0; c < 3; c++) px[i * 3 + c] = (float)img.data[i][c];
        lj_image_desc d{};
        d.width = img.width;
        d.height = img.height;
        d.channels = 3;
        d.data = keep(std::move(px));
        f.images.push_back(d);
        return (int)f.images.size() - 1;
    }
    // mip level 0 of a texture of the pool (the library builds its own
    // pyramid from it, src/mipmap.h:25-50), once per texture
    int image3(int tid) {
        auto it = img3.find(tid);
        if (it != img3.end()) return it->second;
        return img3[tid] = add_image(get_img3(pool, tid).images[0]);
    }
    int image1(int tid) {
        auto it = img1.find(tid);
        if (it != img1.end()) return it->second;
        const Image1 &src = get_img1(pool, tid).images[0];
        Image3 rgb(src.width, src.height);
        for (size_t i = 0; i < src.data.size(); i++) rgb.data[i] = Vector3{src.data[i], src.data[i], src.data[i]};
        return img1[tid] = add_image(rgb);
    }

    // Texture<T> (src/texture.h:80-113): scalar textures fill all three values
    template <typename T>
    lj_texture_desc texture(const Texture<T> &t) {
        lj_texture_desc d{};
        d.uscale = d.vscale = 1;
        auto put = [](float *dst, const T &v) {
            if constexpr (std::is_same_v<T, Real>) {
                dst[0] = dst[1] = dst[2] = (float)v;
            } else {
                for (int c = 0; c < 3; c++) dst[c] = (float)v[c];
            }
        };
        if (auto *c = std::get_if<ConstantTexture<T>>(&t)) {
            d.kind = LJ_TEX_CONST;
            put(d.value0, c->value);
        } else if (auto *k = std::get_if<CheckerboardTexture<T>>(&t)) {
            d.kind = LJ_TEX_CHECKER;
            put(d.value0, k->color0);
            put(d.value1, k->color1);
            d.uscale = (float)k->uscale;
            d.vscale = (float)k->vscale;
            d.uoffset = (float)k->uoffset;
            d.voffset = (float)k->voffset;
        } else if (auto *im = std::get_if<ImageTexture<T>>(&t)) {
            d.kind = LJ_TEX_IMAGE;
            if constexpr (std::is_same_v<T, Real>) d.image_id = image1(im->texture_id);
            else d.image_id = image3(im->texture_id);
            d.uscale = (float)im->uscale;
            d.vscale = (float)im->vscale;
            d.uoffset = (float)im->uoffset;
            d.voffset = (float)im->voffset;
        }
        return d;
    }

    // Material (src/material.h:12-110); texture slots in struct member order
    lj_material_desc material(const Material &m) {
        lj_material_desc d{};
        d.eta = 1;
        std::visit([&](const auto &b) {
            using B = std::decay_t<decltype(b)>;
            if constexpr (std::is_same_v<B, Lambertian>) {
                d.type = LJ_MAT_LAMBERTIAN;
                d.tex[0] = texture(b.reflectance);
            } else if constexpr (std::is_same_v<B, RoughPlastic>) {
                d.type = LJ_MAT_ROUGHPLASTIC;
                d.eta = (float)b.eta;
                d.tex[0] = texture(b.diffuse_reflectance);
                d.tex[1] = texture(b.specular_reflectance);
                d.tex[2] = texture(b.roughness);
            } else if constexpr (std::is_same_v<B, RoughDielectric>) {
                d.type = LJ_MAT_ROUGHDIELECTRIC;
                d.eta = (float)b.eta;
                d.tex[0] = texture(b.specular_reflectance);
                d.tex[1] = texture(b.specular_transmittance);
                d.tex[2] = texture(b.roughness);
            } else if constexpr (std::is_same_v<B, DisneyDiffuse>) {
                d.type = LJ_MAT_DISNEY_DIFFUSE;
                d.tex[0] = texture(b.base_color);
                d.tex[1] = texture(b.roughness);
                d.tex[2] = texture(b.subsurface);
            } else if constexpr (std::is_same_v<B, DisneyMetal>) {
                d.type = LJ_MAT_DISNEY_METAL;
                d.tex[0] = texture(b.base_color);
                d.tex[1] = texture(b.roughness);
                d.tex[2] = texture(b.anisotropic);
            } else if constexpr (std::is_same_v<B, DisneyGlass>) {
                d.type = LJ_MAT_DISNEY_GLASS;
                d.eta = (float)b.eta;
                d.tex[0] = texture(b.base_color);
                d.tex[1] = texture(b.roughness);
                d.tex[2] = texture(b.anisotropic);
            } else if constexpr (std::is_same_v<B, DisneyClearcoat>) {
                d.type = LJ_MAT_DISNEY_CLEARCOAT;
                d.tex[0] = texture(b.clearcoat_gloss);
            } else if constexpr (std::is_same_v<B, DisneySheen>) {
                d.type = LJ_MAT_DISNEY_SHEEN;
                d.tex[0] = texture(b.base_color);
                d.tex[1] = texture(b.sheen_tint);
            } else {
                static_assert(std::is_same_v<B, DisneyBSDF>, "a Material alternative without a mapping");
                d.type = LJ_MAT_DISNEY_BSDF;
                d.eta = (float)b.eta;
                d.tex[0] = texture(b.base_color);
                d.tex[1] = texture(b.specular_transmission);
                d.tex[2] = texture(b.metallic);
                d.tex[3] = texture(b.subsurface);
                d.tex[4] = texture(b.specular);
                d.tex[5] = texture(b.roughness);
                d.tex[6] = texture(b.specular_tint);
                d.tex[7] = texture(b.anisotropic);
                d.tex[8] = texture(b.sheen);
                d.tex[9] = texture(b.sheen_tint);
                d.tex[10] = texture(b.clearcoat);
                d.tex[11] = texture(b.clearcoat_gloss);
            }
        }, m);
        return d;
    }

    // Volume<Spectrum> (src/volume.h:12-30).  channel_scale stays zero: the
    // reference's GridVolume, three values per voxel.
    lj_volume_desc volume(const VolumeSpectrum &v) {
        lj_volume_desc d{};
        d.scale = 1;
        if (auto *c = std::get_if<ConstantVolume<Spectrum>>(&v)) {
            d.kind = LJ_VOL_CONST;
            d.channels = 3;
            for (int k = 0; k < 3; k++) d.value[k] = (float)c->value[k];
        } else {
            const auto &g = std::get<GridVolume<Spectrum>>(v);
            d.kind = LJ_VOL_GRID;
            d.channels = 3;
            d.scale = (float)g.scale;
            for (int k = 0; k < 3; k++) {
                d.res[k] = g.resolution[k];
                d.p_min[k] = (float)g.p_min[k];
                d.p_max[k] = (float)g.p_max[k];
            }
            std::vector<float> data(g.data.size() * 3);
            for (size_t i = 0; i < g.data.size(); i++)
                for (int k = 0; k < 3; k++) data[i * 3 + k] = (float)g.data[i][k];
            d.data = keep(std::move(data));
        }
        return d;
    }
};

}  // namespace

void flatten_scene(const Scene &scene, LjFlatScene &out) {
    Flattener F{out, scene.texture_pool, {}, {}};
    // Shape (src/shape.h:21-54); positions etc. as FP32, the precision
    // Embree receives them in (src/shapes/triangle_mesh.inl:1-22)
    for (const Shape &s : scene.shapes) {
        lj_shape_desc d{};
        d.material_id = get_material_id(s);
        d.area_light_id = get_area_light_id(s);
        d.interior_medium_id = get_interior_medium_id(s);
        d.exterior_medium_id = get_exterior_medium_id(s);
        if (auto *sp = std::get_if<Sphere>(&s)) {
            d.kind = LJ_SHAPE_SPHERE;
            for (int k = 0; k < 3; k++) d.center[k] = (float)sp->position[k];
            d.radius = (float)sp->radius;
        } else {
            const TriangleMesh &m = std::get<TriangleMesh>(s);
            d.kind = LJ_SHAPE_MESH;
            std::vector<float> p, n, uv;
            std::vector<int32_t> idx;
            for (const Vector3 &v : m.positions)
                for (int k = 0; k < 3; k++) p.push_back((float)v[k]);
            for (const Vector3i &t : m.indices)
                for (int k = 0; k < 3; k++) idx.push_back(t[k]);
            for (const Vector3 &v : m.normals)
                for (int k = 0; k < 3; k++) n.push_back((float)v[k]);
            for (const Vector2 &v : m.uvs) {
                uv.push_back((float)v[0]);
                uv.push_back((float)v[1]);
            }
            d.num_vertices = (int32_t)m.positions.size();
            d.num_triangles = (int32_t)m.indices.size();
            d.positions = F.keep(std::move(p));
            d.indices = F.keep(std::move(idx));
            d.normals = m.normals.empty() ? nullptr : F.keep(std::move(n));
            d.uvs = m.uvs.empty() ? nullptr : F.keep(std::move(uv));
        }
        out.shapes.push_back(d);
    }
    for (const Material &m : scene.materials) out.materials.push_back(F.material(m));
    // Light (src/light.h:15-36)
    for (const Light &l : scene.lights) {
        lj_light_desc d{};
        d.image_id = -1;
        d.shape_id = -1;
        if (auto *a = std::get_if<DiffuseAreaLight>(&l)) {
            d.kind = LJ_LIGHT_AREA;
            d.shape_id = a->shape_id;
            for (int k = 0; k < 3; k++) d.intensity[k] = (float)a->intensity[k];
        } else {
            const Envmap &e = std::get<Envmap>(l);
            d.kind = LJ_LIGHT_ENVMAP;
            d.scale = (float)e.scale;
            d.image_id = F.texture(e.values).image_id;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) {
                    d.to_world[i * 4 + j] = e.to_world(i, j);
                    d.to_local[i * 4 + j] = e.to_local(i, j);
                }
        }
        out.lights.push_back(d);
    }
    // Medium (src/medium.h:10-22), PhaseFunction (src/phase_function.h:9-16)
    for (const Medium &m : scene.media) {
        lj_medium_desc d{};
        PhaseFunction pf = get_phase_function(m);
        if (auto *hg = std::get_if<HenyeyGreenstein>(&pf)) {
            d.phase_kind = LJ_PHASE_HG;
            d.g = (float)hg->g;
        } else {
            d.phase_kind = LJ_PHASE_ISOTROPIC;
        }
        if (auto *h = std::get_if<HomogeneousMedium>(&m)) {
            d.kind = LJ_MEDIUM_HOMOGENEOUS;
            for (int k = 0; k < 3; k++) {
                d.sigma_a[k] = (float)h->sigma_a[k];
                d.sigma_s[k] = (float)h->sigma_s[k];
            }
        } else {
            const auto &het = std::get<HeterogeneousMedium>(m);
            d.kind = LJ_MEDIUM_HETEROGENEOUS;
            d.albedo = F.volume(het.albedo);
            d.density = F.volume(het.density);
        }
        out.media.push_back(d);
    }

    lj_scene_desc &desc = out.desc;
    desc = lj_scene_desc{};
    const Camera &c = scene.camera;   // src/camera.h:9-25
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) desc.camera.cam_to_world[i * 4 + j] = c.cam_to_world(i, j);
    // cam_to_sample = scale(-1/2, -aspect/2, 1) * translate(-1, -1/aspect, 0)
    // * perspective(fov) (src/camera.cpp:7-21): entry (0, 0) is
    // -1 / (2 tan(fov / 2))
    desc.camera.fov = 2 * std::atan(1 / (-2 * c.cam_to_sample(0, 0))) * 180 / c_PI;
    desc.camera.width = c.width;
    desc.camera.height = c.height;
    desc.camera.medium_id = c.medium_id;
    if (auto *b = std::get_if<Box>(&c.filter)) {
        desc.camera.filter_kind = LJ_FILTER_BOX;
        desc.camera.filter_param = (float)b->width;
    } else if (auto *t = std::get_if<Tent>(&c.filter)) {
        desc.camera.filter_kind = LJ_FILTER_TENT;
        desc.camera.filter_param = (float)t->width;
    } else {
        desc.camera.filter_kind = LJ_FILTER_GAUSSIAN;
        desc.camera.filter_param = (float)std::get<Gaussian>(c.filter).stddev;
    }
    // RenderOptions (src/scene.h:13-31); the integrator enums share an order
    desc.options.integrator = (int32_t)scene.options.integrator;
    desc.options.samples_per_pixel = scene.options.samples_per_pixel;
    desc.options.max_depth = scene.options.max_depth;
    desc.options.rr_depth = scene.options.rr_depth;
    desc.options.vol_path_version = scene.options.vol_path_version;
    desc.options.max_null_collisions = scene.options.max_null_collisions;
    desc.num_shapes = (int32_t)out.shapes.size();
    desc.shapes = out.shapes.data();
    desc.num_materials = (int32_t)out.materials.size();
    desc.materials = out.materials.data();
    desc.num_lights = (int32_t)out.lights.size();
    desc.lights = out.lights.data();
    desc.num_media = (int32_t)out.media.size();
    desc.media = out.media.data();
    desc.num_images = (int32_t)out.images.size();
    desc.images = out.images.data();
    desc.envmap_light_id = scene.envmap_light_id;
}

Image3 image_from_rgb(const float *rgb, int width, int height) {
    Image3 img(width, height);
    for (size_t i = 0; i < img.data.size(); i++) img.data[i] = Vector3{rgb[i * 3], rgb[i * 3 + 1], rgb[i * 3 + 2]};
    return img;
}

Image3 render_gpu(const Scene &scene) {
    static std::mutex m;
    static lj_ctx *ctx = nullptr;   // one context per process, device 0
    std::lock_guard<std::mutex> lock(m);
    if (!ctx && lj_gpu_init(0, &ctx) != LJ_OK) throw std::runtime_error("render_gpu: no GB300-class GPU");
    LjFlatScene flat;
    flatten_scene(scene, flat);
    lj_scene *gs = nullptr;
    if (lj_gpu_scene_create(ctx, &flat.desc, &gs) != LJ_OK) throw std::runtime_error(lj_gpu_last_error(ctx));
    const int w = scene.camera.width, h = scene.camera.height;
    std::vector<float> rgb((size_t)w * h * 3);
    lj_render_params params{};
    int rc = lj_gpu_render(gs, &params, rgb.data(), nullptr);
    std::string msg = rc == LJ_OK ? "" : lj_gpu_last_error(ctx);
    lj_gpu_scene_destroy(gs);
    if (rc != LJ_OK) throw std::runtime_error(msg);
    return image_from_rgb(rgb.data(), w, h);
}
