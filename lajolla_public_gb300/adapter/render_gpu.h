// render_gpu.h -- the GB300 library behind lajolla's render(const Scene&).
//
// This is the reference-side binding a lajolla maintainer adds: it compiles
// against lajolla's own headers (src/scene.h, src/image.h) and the C ABI
// (include/lj_gpu.h), and main.cpp (src/main.cpp:40) calls render_gpu
// instead of render (src/render.h:9) when the GPU is selected.  The parser,
// the Scene variants and imwrite stay as they are.
#pragma once

#include <vector>

#include "image.h"
#include "lj_gpu.h"
#include "scene.h"

// A Scene flattened into the library's descriptor.  `desc` points into the
// arrays this object owns, so keep it alive (and in place: it cannot be
// copied) while `desc` is in use.  lj_gpu_scene_create copies everything.
struct LjFlatScene {
    lj_scene_desc desc{};
    std::vector<std::vector<float>> floats;
    std::vector<std::vector<int32_t>> ints;
    std::vector<lj_shape_desc> shapes;
    std::vector<lj_material_desc> materials;
    std::vector<lj_light_desc> lights;
    std::vector<lj_medium_desc> media;
    std::vector<lj_image_desc> images;

    LjFlatScene() = default;
    LjFlatScene(const LjFlatScene &) = delete;
    LjFlatScene &operator=(const LjFlatScene &) = delete;
};

// Flattens `scene` into `out` (needs no device): shapes, materials and their
// textures (each texture image once), lights, media, camera and render
// options, in the Scene's own order, so every id keeps its meaning.
void flatten_scene(const Scene &scene, LjFlatScene &out);

// The library's FP32 HWC image (W * H * 3) as the Image3 imwrite takes
// (src/image.cpp:135-173): each value widened to double, exactly.
Image3 image_from_rgb(const float *rgb, int width, int height);

// The GPU form of Image3 render(const Scene&) (src/render.cpp:155-170):
// flattens the scene, builds it on device 0 (one lj_ctx per process, made
// on the first call), renders every sample and returns the per-pixel mean.
// Throws std::runtime_error with the library's message on failure, where
// the reference throws fl_exception.
Image3 render_gpu(const Scene &scene);
