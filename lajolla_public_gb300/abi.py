"""ctypes mirror of include/lj_gpu.h (the C ABI of the GPU hot path).

Every Structure here has the same field order, types and padding as the C
header; tests/test_abi.py checks the sizes against the compiled library.
"""
import ctypes as C

LJ_OK = 0
LJ_ERR_INVALID_ARG = -1
LJ_ERR_CUDA = -2
LJ_ERR_OUT_OF_MEMORY = -3
LJ_ERR_UNSUPPORTED = -4
LJ_ERR_DEVICE_LIMIT = -5
LJ_ERR_NO_DEVICE = -6
LJ_ERR_QUEUE_FULL = -7
LJ_ERR_NOT_FOUND = -8
LJ_ERR_TIMEOUT = -9
LJ_ERR_CANCELLED = -10
LJ_ERR_SIZE_LIMIT = -11
LJ_NOALLOC_MORTON_MAX_TRIANGLES = 65536
LJ_RENDER_COUNT_BVH = 2
LJ_UPDATE_REFIT, LJ_UPDATE_REBUILD = 0, 1
LJ_TUNE_BALANCED, LJ_TUNE_THROUGHPUT, LJ_TUNE_LATENCY = 0, 1, 2
LJ_COUNT_BVH_STRIDE = 16

LJ_TEX_CONST, LJ_TEX_IMAGE, LJ_TEX_CHECKER = 0, 1, 2
(LJ_MAT_LAMBERTIAN, LJ_MAT_ROUGHPLASTIC, LJ_MAT_ROUGHDIELECTRIC, LJ_MAT_DISNEY_DIFFUSE,
 LJ_MAT_DISNEY_METAL, LJ_MAT_DISNEY_GLASS, LJ_MAT_DISNEY_CLEARCOAT, LJ_MAT_DISNEY_SHEEN,
 LJ_MAT_DISNEY_BSDF) = range(9)
LJ_MAT_COUNT = 9
LJ_MAT_SLOTS = 12
LJ_SHAPE_MESH, LJ_SHAPE_SPHERE = 0, 1
LJ_LIGHT_AREA, LJ_LIGHT_ENVMAP = 0, 1
LJ_VOL_CONST, LJ_VOL_GRID = 0, 1
LJ_MEDIUM_HOMOGENEOUS, LJ_MEDIUM_HETEROGENEOUS = 0, 1
LJ_PHASE_ISOTROPIC, LJ_PHASE_HG = 0, 1
LJ_FILTER_BOX, LJ_FILTER_TENT, LJ_FILTER_GAUSSIAN = 0, 1, 2
(LJ_INTEGRATOR_DEPTH, LJ_INTEGRATOR_SHADING_NORMAL, LJ_INTEGRATOR_MEAN_CURVATURE,
 LJ_INTEGRATOR_RAY_DIFFERENTIAL, LJ_INTEGRATOR_MIPMAP_LEVEL, LJ_INTEGRATOR_PATH,
 LJ_INTEGRATOR_VOLPATH) = range(7)
LJ_BSDF_OP_EVAL, LJ_BSDF_OP_PDF, LJ_BSDF_OP_SAMPLE = 0, 1, 2
LJ_MAX_BOUNCES = 1024

# packed parameters per material type in the BSDF batch layout
BSDF_PARAM_COUNT = [4, 8, 8, 6, 6, 6, 2, 5, 15]
# texture slot widths per material type (3 = RGB, 1 = scalar)
SLOT_WIDTHS = [
    [3], [3, 3, 1], [3, 3, 1], [3, 1, 1], [3, 1, 1], [3, 1, 1], [1], [3, 1],
    [3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
]

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)


class lj_texture_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("image_id", C.c_int32),
                ("value0", C.c_float * 3), ("value1", C.c_float * 3),
                ("uscale", C.c_float), ("vscale", C.c_float),
                ("uoffset", C.c_float), ("voffset", C.c_float)]


class lj_material_desc(C.Structure):
    _fields_ = [("type", C.c_int32), ("eta", C.c_float),
                ("tex", lj_texture_desc * LJ_MAT_SLOTS)]


class lj_shape_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("material_id", C.c_int32),
                ("area_light_id", C.c_int32), ("interior_medium_id", C.c_int32),
                ("exterior_medium_id", C.c_int32), ("num_vertices", C.c_int32),
                ("num_triangles", C.c_int32), ("pad0", C.c_int32),
                ("positions", f32p), ("indices", i32p), ("normals", f32p), ("uvs", f32p),
                ("center", C.c_float * 3), ("radius", C.c_float)]


class lj_light_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("shape_id", C.c_int32),
                ("intensity", C.c_float * 3), ("image_id", C.c_int32),
                ("scale", C.c_float), ("pad0", C.c_int32),
                ("to_world", C.c_double * 16), ("to_local", C.c_double * 16)]


class lj_image_desc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("channels", C.c_int32),
                ("pad0", C.c_int32), ("data", f32p)]


class lj_volume_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("res", C.c_int32 * 3), ("channels", C.c_int32),
                ("value", C.c_float * 3), ("p_min", C.c_float * 3), ("p_max", C.c_float * 3),
                ("scale", C.c_float), ("data", f32p), ("channel_scale", C.c_float * 3)]


class lj_medium_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("phase_kind", C.c_int32), ("g", C.c_float),
                ("sigma_a", C.c_float * 3), ("sigma_s", C.c_float * 3),
                ("albedo", lj_volume_desc), ("density", lj_volume_desc)]


class lj_camera_desc(C.Structure):
    _fields_ = [("cam_to_world", C.c_double * 16), ("fov", C.c_double),
                ("width", C.c_int32), ("height", C.c_int32),
                ("filter_kind", C.c_int32), ("filter_param", C.c_float),
                ("medium_id", C.c_int32), ("pad0", C.c_int32)]


class lj_render_options(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("samples_per_pixel", C.c_int32),
                ("max_depth", C.c_int32), ("rr_depth", C.c_int32),
                ("vol_path_version", C.c_int32), ("max_null_collisions", C.c_int32)]


class lj_scene_desc(C.Structure):
    _fields_ = [("camera", lj_camera_desc), ("options", lj_render_options),
                ("num_shapes", C.c_int32), ("num_materials", C.c_int32),
                ("num_lights", C.c_int32), ("num_media", C.c_int32),
                ("num_images", C.c_int32), ("envmap_light_id", C.c_int32),
                ("shapes", C.POINTER(lj_shape_desc)),
                ("materials", C.POINTER(lj_material_desc)),
                ("lights", C.POINTER(lj_light_desc)),
                ("media", C.POINTER(lj_medium_desc)),
                ("images", C.POINTER(lj_image_desc))]


class lj_scene_info(C.Structure):
    _fields_ = [("bounds_lower", C.c_float * 3), ("bounds_upper", C.c_float * 3),
                ("bsphere_radius", C.c_double), ("bsphere_center", C.c_double * 3),
                ("num_triangles", C.c_int64), ("num_prims", C.c_int64),
                ("num_wide_nodes", C.c_int64), ("num_binary_nodes", C.c_int64),
                ("device_bytes", C.c_int64), ("build_ms", C.c_double)]


LJ_GPU_ABI_VERSION = 4       # the structs below mirror this version of include/lj_gpu.h
LJ_RENDER_PROFILE = 1
(LJ_KERNEL_CAMERA, LJ_KERNEL_TRACE, LJ_KERNEL_SHADE, LJ_KERNEL_SHADOW, LJ_KERNEL_OTHER, LJ_KERNEL_MEDIUM,
 LJ_KERNEL_NEE) = range(7)
LJ_KERNEL_CLASSES = 7
KERNEL_CLASS_NAMES = ["camera", "trace", "shade", "shadow", "other", "medium", "nee"]


class lj_render_params(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("spp", C.c_int32), ("sample_offset", C.c_int32),
                ("max_paths_in_flight", C.c_int32), ("flags", C.c_int32)]


class lj_stats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("samples", C.c_int64),
                ("rays_closest", C.c_int64), ("rays_shadow", C.c_int64),
                ("path_segments", C.c_int64), ("kernel_launches", C.c_int64),
                ("null_collisions", C.c_int64), ("real_collisions", C.c_int64),
                ("class_ms", C.c_double * LJ_KERNEL_CLASSES),
                ("class_launches", C.c_int64 * LJ_KERNEL_CLASSES),
                ("bvh_rays", C.c_int64 * 2), ("bvh_nodes", C.c_int64 * 2), ("bvh_prims", C.c_int64 * 2)]


class lj_ray(C.Structure):
    _fields_ = [("org", C.c_float * 3), ("tnear", C.c_float),
                ("dir", C.c_float * 3), ("tfar", C.c_float)]


class lj_hit(C.Structure):
    _fields_ = [("t", C.c_float), ("prim", C.c_int32), ("u", C.c_float), ("v", C.c_float)]


class lj_bsdf_batch(C.Structure):
    _fields_ = [("material_type", C.c_int32), ("op", C.c_int32),
                ("transport_to_view", C.c_int32), ("pad0", C.c_int32),
                ("d_params", C.c_void_p), ("d_dir_in", C.c_void_p),
                ("d_dir_out", C.c_void_p), ("d_rnd", C.c_void_p),
                ("d_out_value", C.c_void_p), ("d_out_pdf", C.c_void_p),
                ("d_out_dir", C.c_void_p), ("d_out_eta", C.c_void_p),
                ("d_out_roughness", C.c_void_p), ("d_out_valid", C.c_void_p)]


LJ_SCHED_FIFO, LJ_SCHED_SRPT = 0, 1
LJ_SERVER_PROFILE = 1
LJ_SERVER_ONE_SHADE_KERNEL = 2
LJ_JOB_QUEUED, LJ_JOB_RUNNING, LJ_JOB_DONE, LJ_JOB_FAILED, LJ_JOB_CANCELLED = range(5)


class lj_server_options(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("path_pool", C.c_int64),
                ("block_size", C.c_int32), ("max_live_jobs", C.c_int32),
                ("max_queued_jobs", C.c_int32), ("waves_per_poll", C.c_int32),
                ("policy", C.c_int32), ("use_graphs", C.c_int32), ("flags", C.c_int32),
                ("tune_objective", C.c_int32)]


class lj_job_desc(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("spp", C.c_int32), ("sample_offset", C.c_int32),
                ("width", C.c_int32), ("height", C.c_int32), ("override_depth", C.c_int32),
                ("max_depth", C.c_int32), ("rr_depth", C.c_int32), ("flags", C.c_int32)]


class lj_job_status(C.Structure):
    _fields_ = [("state", C.c_int32), ("error", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("samples_total", C.c_int64), ("samples_done", C.c_int64), ("samples_dropped", C.c_int64),
                ("submit_ms", C.c_double), ("admit_ms", C.c_double), ("finish_ms", C.c_double)]


class lj_server_stats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_int64), ("jobs_done", C.c_int64), ("jobs_failed", C.c_int64),
                ("jobs_cancelled", C.c_int64), ("waves", C.c_int64), ("graph_launches", C.c_int64),
                ("samples_done", C.c_int64), ("bytes_resident", C.c_int64), ("busy_ms", C.c_double),
                ("rays_closest", C.c_int64), ("rays_shadow", C.c_int64), ("path_segments", C.c_int64),
                ("kernel_launches", C.c_int64),
                ("class_ms", C.c_double * LJ_KERNEL_CLASSES), ("class_launches", C.c_int64 * LJ_KERNEL_CLASSES),
                ("vol_segments", C.c_int64), ("nee_requests", C.c_int64),
                ("null_collisions", C.c_int64), ("real_collisions", C.c_int64)]


STRUCT_SIZES = {
    "lj_texture_desc": C.sizeof(lj_texture_desc),
    "lj_material_desc": C.sizeof(lj_material_desc),
    "lj_shape_desc": C.sizeof(lj_shape_desc),
    "lj_light_desc": C.sizeof(lj_light_desc),
    "lj_image_desc": C.sizeof(lj_image_desc),
    "lj_volume_desc": C.sizeof(lj_volume_desc),
    "lj_medium_desc": C.sizeof(lj_medium_desc),
    "lj_camera_desc": C.sizeof(lj_camera_desc),
    "lj_render_options": C.sizeof(lj_render_options),
    "lj_scene_desc": C.sizeof(lj_scene_desc),
    "lj_scene_info": C.sizeof(lj_scene_info),
    "lj_render_params": C.sizeof(lj_render_params),
    "lj_server_options": C.sizeof(lj_server_options),
    "lj_job_desc": C.sizeof(lj_job_desc),
    "lj_job_status": C.sizeof(lj_job_status),
    "lj_server_stats": C.sizeof(lj_server_stats),
    "lj_stats": C.sizeof(lj_stats),
    "lj_ray": C.sizeof(lj_ray),
    "lj_hit": C.sizeof(lj_hit),
    "lj_bsdf_batch": C.sizeof(lj_bsdf_batch),
}
