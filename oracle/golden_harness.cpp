// ORACLE / TEST INFRASTRUCTURE -- not part of the product.
//
// Golden-vector generator: our driver, compiled against the UNMODIFIED
// reference sources (see Makefile, target `ref`), calling the reference's own
// functions on inputs read from a binary file and writing their outputs.
// tests/golden/make_golden.py drives it and commits the results as fixtures.
//
//   golden_harness bsdf   in out   eval / pdf_sample_bsdf / sample_bsdf
//                                  (src/material.cpp:90-119), TO_LIGHT and TO_VIEW
//   golden_harness phase  in out   HG eval / pdf / sample (src/phase_function.cpp)
//   golden_harness table  in out   TableDist1D / 2D (src/table_dist.cpp)
//   golden_harness pcg    in out   init_pcg32 / next_pcg32 / next_pcg32_real<double>
//   golden_harness light  in out   sample_light + sample_point_on_light +
//                                  pdf_point_on_light + emission on a scene with a
//                                  triangle-mesh light, a sphere light and an envmap
//   golden_harness camera in out   sample_primary (src/camera.cpp:23-47)
//   golden_harness medium in out d1.vol d3.vol a3.vol
//                                  get_sigma_a / get_sigma_s / get_majorant
//                                  (src/medium.cpp:27-37) on grid volumes the
//                                  reference's .vol loader reads (src/volume.cpp)
//
// Input/output files are flat little-endian arrays; layouts are documented per
// mode below and mirrored in make_golden.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "camera.h"
#include "light.h"
#include "material.h"
#include "medium.h"
#include "pcg.h"
#include "phase_function.h"
#include "scene.h"
#include "table_dist.h"
#include "texture.h"
#include "transform.h"

static std::vector<double> read_all(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) { perror(path); exit(1); }
    std::vector<double> v;
    double x;
    while (fread(&x, sizeof(double), 1, f) == 1) v.push_back(x);
    fclose(f);
    return v;
}
static void write_all(const char *path, const std::vector<double> &v) {
    FILE *f = fopen(path, "wb");
    if (!f) { perror(path); exit(1); }
    fwrite(v.data(), sizeof(double), v.size(), f);
    fclose(f);
}

static PathVertex local_vertex() {
    PathVertex v;
    v.geometric_normal = Vector3{0, 0, 1};
    v.shading_frame = Frame(v.geometric_normal);
    v.uv = Vector2{0, 0};
    v.uv_screen_size = 0;
    return v;
}

static ConstantTexture<Spectrum> cs(const double *p) { return ConstantTexture<Spectrum>{Vector3{p[0], p[1], p[2]}}; }
static ConstantTexture<Real> cf(double x) { return ConstantTexture<Real>{x}; }

// bsdf: record = type, params[8], dir_in[3], dir_out[3], rnd[3]   (18 doubles)
//   params: Lambertian: R(3); plastic: Kd(3) Ks(3) roughness eta... (packed as
//   in lj_gpu_bsdf_param_count order: slots then eta)
// out = eval_to_light[3], eval_to_view[3], pdf, valid, dir[3], eta, roughness  (13)
static void run_bsdf(const std::vector<double> &in, std::vector<double> &out) {
    const int rec = 18;
    TexturePool pool;
    PathVertex v = local_vertex();
    for (size_t r = 0; r + rec <= in.size(); r += rec) {
        const double *x = &in[r];
        int type = (int)x[0];
        const double *p = x + 1;
        Material m;
        if (type == 0) m = Lambertian{cs(p)};
        else if (type == 1) m = RoughPlastic{cs(p), cs(p + 3), cf(p[6]), p[7]};
        else m = RoughDielectric{cs(p), cs(p + 3), cf(p[6]), p[7]};
        Vector3 wi{x[9], x[10], x[11]}, wo{x[12], x[13], x[14]};
        Vector2 uv{x[15], x[16]};
        Real w = x[17];
        Spectrum f = eval(m, wi, wo, v, pool, TransportDirection::TO_LIGHT);
        Spectrum fv = eval(m, wi, wo, v, pool, TransportDirection::TO_VIEW);
        Real pdf = pdf_sample_bsdf(m, wi, wo, v, pool);
        std::optional<BSDFSampleRecord> s = sample_bsdf(m, wi, v, pool, uv, w);
        out.insert(out.end(), {f.x, f.y, f.z, fv.x, fv.y, fv.z, pdf});
        if (s) out.insert(out.end(), {1.0, s->dir_out.x, s->dir_out.y, s->dir_out.z, s->eta, s->roughness});
        else out.insert(out.end(), {0.0, 0.0, 0.0, 0.0, 0.0, 0.0});
    }
}

// phase: record = g, dir_in[3], dir_out[3], u[2] (9) -> eval, pdf, dir[3] (5)
static void run_phase(const std::vector<double> &in, std::vector<double> &out) {
    for (size_t r = 0; r + 9 <= in.size(); r += 9) {
        const double *x = &in[r];
        PhaseFunction pf = HenyeyGreenstein{x[0]};
        Vector3 wi{x[1], x[2], x[3]}, wo{x[4], x[5], x[6]};
        Spectrum e = eval(pf, wi, wo);
        Real pdf = pdf_sample_phase(pf, wi, wo);
        std::optional<Vector3> d = sample_phase_function(pf, wi, Vector2{x[7], x[8]});
        out.insert(out.end(), {e.x, pdf, d->x, d->y, d->z});
    }
}

// table: n1, f1[n1], m1, u1[m1], w, h, f2[w*h], m2, u2[2*m2]
//   -> idx1[m1], pmf1[m1], xy2[2*m2], pdf2[m2]
static void run_table(const std::vector<double> &in, std::vector<double> &out) {
    size_t k = 0;
    int n1 = (int)in[k++];
    std::vector<Real> f1(in.begin() + k, in.begin() + k + n1);
    k += n1;
    int m1 = (int)in[k++];
    TableDist1D t1 = make_table_dist_1d(f1);
    std::vector<double> idx, pm;
    for (int i = 0; i < m1; i++) {
        int id = sample(t1, in[k++]);
        idx.push_back(id);
        pm.push_back(pmf(t1, id));
    }
    int w = (int)in[k++], h = (int)in[k++];
    std::vector<Real> f2(in.begin() + k, in.begin() + k + (size_t)w * h);
    k += (size_t)w * h;
    int m2 = (int)in[k++];
    TableDist2D t2 = make_table_dist_2d(f2, w, h);
    std::vector<double> xy, pd;
    for (int i = 0; i < m2; i++) {
        Vector2 s = sample(t2, Vector2{in[k], in[k + 1]});
        k += 2;
        xy.push_back(s.x);
        xy.push_back(s.y);
        pd.push_back(pdf(t2, s));
    }
    out.insert(out.end(), idx.begin(), idx.end());
    out.insert(out.end(), pm.begin(), pm.end());
    out.insert(out.end(), xy.begin(), xy.end());
    out.insert(out.end(), pd.begin(), pd.end());
}

// pcg: record = stream, k -> k raw u32 outputs then k doubles of a fresh stream
static void run_pcg(const std::vector<double> &in, std::vector<double> &out) {
    for (size_t r = 0; r + 2 <= in.size(); r += 2) {
        uint64_t stream = (uint64_t)in[r];
        int k = (int)in[r + 1];
        pcg32_state s = init_pcg32(stream);
        for (int i = 0; i < k; i++) out.push_back((double)next_pcg32(s));
        pcg32_state s2 = init_pcg32(stream);
        for (int i = 0; i < k; i++) out.push_back(next_pcg32_real<double>(s2));
    }
}

// light: header = env_w, env_h, env pixels (w*h*3), then records
//   ref[3], light_w, u, v, shape_w (7)
//   -> light id, point[3], normal[3], pdf (light_pmf * pdf_point), emission[3] (11)
// Scene: shape 0 = triangle-mesh quad light (radiance 5,4,3), shape 1 = sphere
// light (radiance 2,3,4), lights 2 = envmap (scale 0.5, rotated).
static void run_light(const std::vector<double> &in, std::vector<double> &out) {
    size_t k = 0;
    int ew = (int)in[k++], eh = (int)in[k++];
    Image3 env(ew, eh);
    for (int i = 0; i < ew * eh; i++) {
        env(i) = Vector3{in[k], in[k + 1], in[k + 2]};
        k += 3;
    }
    RTCDevice dev = rtcNewDevice(nullptr);
    TexturePool pool;
    std::vector<Material> mats = {Lambertian{ConstantTexture<Spectrum>{Vector3{0.5, 0.5, 0.5}}}};
    TriangleMesh quad;
    quad.positions = {Vector3{-1.0, 2.0, -1.0}, Vector3{1.0, 2.0, -1.0}, Vector3{1.0, 2.5, 1.0}, Vector3{-1.0, 2.0, 1.5}};
    quad.indices = {Vector3i{0, 2, 1}, Vector3i{0, 3, 2}};
    quad.material_id = 0;
    quad.area_light_id = 0;
    Sphere sph;
    sph.position = Vector3{2.0, 1.0, 0.5};
    sph.radius = 0.5;
    sph.material_id = 0;
    sph.area_light_id = 1;
    std::vector<Shape> shapes = {quad, sph};
    Matrix4x4 to_world = rotate(30, Vector3{0.2, 1.0, 0.1});
    Envmap em{make_image_spectrum_texture("env", env, pool), to_world, inverse(to_world), 0.5};
    std::vector<Light> lights = {DiffuseAreaLight{0, Vector3{5.0, 4.0, 3.0}}, DiffuseAreaLight{1, Vector3{2.0, 3.0, 4.0}}, em};
    Scene scene(dev, Camera(), mats, shapes, lights, {}, 2, pool, RenderOptions{}, "");
    for (; k + 7 <= in.size(); k += 7) {
        Vector3 ref{in[k], in[k + 1], in[k + 2]};
        int lid = sample_light(scene, in[k + 3]);
        const Light &l = scene.lights[lid];
        PointAndNormal pn = sample_point_on_light(l, ref, Vector2{in[k + 4], in[k + 5]}, in[k + 6], scene);
        Real pdf = light_pmf(scene, lid) * pdf_point_on_light(l, pn, ref, scene);
        Vector3 dir = is_envmap(l) ? pn.normal : normalize(ref - pn.position);
        Spectrum e = emission(l, dir, Real(0), pn, scene);
        out.insert(out.end(), {(double)lid, pn.position.x, pn.position.y, pn.position.z, pn.normal.x,
                               pn.normal.y, pn.normal.z, pdf, e.x, e.y, e.z});
    }
}

// camera: header = cam_to_world[16], fov, w, h, filter kind, filter param,
// then records sx, sy -> org[3], dir[3]
static void run_camera(const std::vector<double> &in, std::vector<double> &out) {
    Matrix4x4 m;
    for (int i = 0; i < 16; i++) m(i / 4, i % 4) = in[i];
    double fov = in[16];
    int w = (int)in[17], h = (int)in[18], fk = (int)in[19];
    double fp = in[20];
    Filter f = fk == 0 ? Filter{Box{fp}} : (fk == 1 ? Filter{Tent{fp}} : Filter{Gaussian{fp}});
    Camera cam(m, fov, w, h, f, -1);
    for (size_t k = 21; k + 2 <= in.size(); k += 2) {
        Ray r = sample_primary(cam, Vector2{in[k], in[k + 1]});
        out.insert(out.end(), {r.org.x, r.org.y, r.org.z, r.dir.x, r.dir.y, r.dir.z});
    }
}

// medium: argv = d1.vol (1 channel), d3.vol (3 channels), a3.vol (3 channels)
//   in: header s0, s1, albedo0[3], sigma_a[3], sigma_s[3] (11), then records
//   p[3], d[3] (6)
//   out per record, for media 0, 1, 2: sigma_a[3], sigma_s[3], majorant[3] (27)
// Media (as parse_medium builds them, src/parsers/parse_scene.cpp:694-741):
//   0 heterogeneous: density = d1.vol with scale s0, constant albedo0
//   1 heterogeneous: density = d3.vol with scale s1, albedo = a3.vol
//   2 homogeneous sigma_a, sigma_s
// The majorant is taken along the ray (p, d) with tnear 0, tfar = inf.
static void run_medium(const std::vector<double> &in, std::vector<double> &out, char **vols) {
    VolumeSpectrum d1 = load_volume_from_file<Spectrum>(vols[0]);
    VolumeSpectrum d3 = load_volume_from_file<Spectrum>(vols[1]);
    VolumeSpectrum a3 = load_volume_from_file<Spectrum>(vols[2]);
    set_scale(d1, in[0]);
    set_scale(d3, in[1]);
    std::vector<Medium> media = {
        HeterogeneousMedium{{HenyeyGreenstein{0.3}}, ConstantVolume<Spectrum>{Vector3{in[2], in[3], in[4]}}, d1},
        HeterogeneousMedium{{HenyeyGreenstein{0.3}}, a3, d3},
        HomogeneousMedium{{IsotropicPhase{}}, Vector3{in[5], in[6], in[7]}, Vector3{in[8], in[9], in[10]}}};
    for (size_t k = 11; k + 6 <= in.size(); k += 6) {
        Vector3 p{in[k], in[k + 1], in[k + 2]}, d{in[k + 3], in[k + 4], in[k + 5]};
        Ray r{p, d, Real(0), std::numeric_limits<Real>::infinity()};
        for (const Medium &m : media) {
            Spectrum sa = get_sigma_a(m, p), ss = get_sigma_s(m, p), mj = get_majorant(m, r);
            out.insert(out.end(), {sa.x, sa.y, sa.z, ss.x, ss.y, ss.z, mj.x, mj.y, mj.z});
        }
    }
}

int main(int argc, char **argv) {
    if (argc < 4 || (std::string(argv[1]) == "medium" ? argc != 7 : argc != 4)) {
        fprintf(stderr, "usage: golden_harness <bsdf|phase|table|pcg|light|camera> in out\n"
                        "       golden_harness medium in out d1.vol d3.vol a3.vol\n");
        return 2;
    }
    std::string mode = argv[1];
    std::vector<double> in = read_all(argv[2]), out;
    if (mode == "bsdf") run_bsdf(in, out);
    else if (mode == "phase") run_phase(in, out);
    else if (mode == "table") run_table(in, out);
    else if (mode == "pcg") run_pcg(in, out);
    else if (mode == "light") run_light(in, out);
    else if (mode == "camera") run_camera(in, out);
    else if (mode == "medium") run_medium(in, out, argv + 4);
    else { fprintf(stderr, "unknown mode\n"); return 2; }
    write_all(argv[3], out);
    return 0;
}
