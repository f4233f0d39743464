"""ctypes structures and signatures of the renderer part of include/lucent.h."""
import ctypes as C

P = C.POINTER
F32P, F64P, I32P, U32P, U8P, VP = P(C.c_float), P(C.c_double), P(C.c_int32), P(C.c_uint32), P(C.c_uint8), C.c_void_p


class SceneDesc(C.Structure):
    _fields_ = [("tri_count", C.c_uint32), ("positions", F32P), ("normals", F32P), ("uvs", F32P),
                ("tri_material", I32P), ("tri_light", I32P), ("tri_alpha", U8P), ("bvh_nodes", F32P),
                ("bvh_node_count", C.c_uint32), ("bvh_tri_indices", U32P), ("materials", F32P),
                ("material_count", C.c_uint32), ("spheres", F32P), ("sphere_materials", I32P),
                ("sphere_lights", I32P), ("sphere_count", C.c_uint32), ("lights", F32P), ("light_count", C.c_uint32),
                ("ground_material", C.c_int32), ("texture_count", C.c_uint32), ("texture_rgba8", P(U8P)),
                ("texture_width", U32P), ("texture_height", U32P), ("color_layers", I32P),
                ("color_layer_count", C.c_uint32), ("data_layers", I32P), ("data_layer_count", C.c_uint32)]


class LightingDesc(C.Structure):
    _fields_ = [("sun_enabled", C.c_int32), ("sun_dir", C.c_float * 3), ("sun_radiance", C.c_float * 3),
                ("sun_cos_angle", C.c_float), ("sun_pdf", C.c_float), ("env_width", C.c_uint32),
                ("env_height", C.c_uint32), ("env_rgb", F32P), ("env_rotation_cos", C.c_float),
                ("env_rotation_sin", C.c_float), ("env_intensity", C.c_float), ("env_background", C.c_int32),
                ("backdrop", C.c_float * 3)]


class CameraDesc(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3),
                ("forward", C.c_float * 3), ("tan_half_fov", C.c_float), ("aperture", C.c_float),
                ("focus_distance", C.c_float)]


class SettingsDesc(C.Structure):
    _fields_ = [("max_bounces", C.c_uint32), ("firefly_clamp", C.c_float), ("temporal", C.c_int32)]


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_uint32), ("seed", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("triangles", C.c_uint32), ("bvh_nodes", C.c_uint32), ("closest_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("last_trace_ms", C.c_double), ("phase_ms", C.c_double * 6),
                ("traversal", C.c_uint64 * 5), ("kernel_launches", C.c_uint64)]


def declare(L, sig):
    sig(L, "lucent_renderer_create", [C.c_uint32, C.c_uint32, P(VP)])
    sig(L, "lucent_renderer_destroy", [VP], None)
    sig(L, "lucent_renderer_load_scene", [VP, P(SceneDesc)])
    sig(L, "lucent_renderer_upload_lighting", [VP, P(LightingDesc)])
    sig(L, "lucent_env_sampler", [F32P, C.c_uint32, C.c_uint32, C.c_uint32, U32P, U32P, F32P, F64P])
    sig(L, "lucent_env_sampler_device", [VP, C.c_uint32, C.c_uint32, C.c_uint32, U32P, U32P, VP, F64P, VP])
    sig(L, "lucent_renderer_set_env_device", [VP, VP, C.c_uint32, C.c_uint32, VP])
    sig(L, "lucent_renderer_set_env", [VP, F32P, C.c_uint32, C.c_uint32, VP])
    sig(L, "lucent_renderer_upload_ground", [VP, C.c_int32, C.c_float])
    sig(L, "lucent_renderer_upload_camera", [VP, P(CameraDesc)])
    sig(L, "lucent_renderer_apply_settings", [VP, P(SettingsDesc)])
    sig(L, "lucent_renderer_resize", [VP, C.c_uint32, C.c_uint32])
    sig(L, "lucent_renderer_reset", [VP])
    sig(L, "lucent_renderer_set_seed", [VP, C.c_uint32])
    sig(L, "lucent_renderer_trace", [VP, C.c_uint32, VP])
    sig(L, "lucent_renderer_check", [VP, VP])
    sig(L, "lucent_renderer_read", [VP, F32P, F32P, F32P, F32P])
    sig(L, "lucent_renderer_read_color_async", [VP, F32P, VP])
    sig(L, "lucent_renderer_stats", [VP, P(RenderStats)])
    sig(L, "lucent_renderer_set_profiling", [VP, C.c_int32])
    sig(L, "lucent_renderer_trim", [VP])
    sig(L, "lucent_renderer_capture_rays", [VP, C.c_uint32, C.c_uint32])
    sig(L, "lucent_renderer_read_rays", [VP, C.c_uint32, C.c_int32, F32P, C.c_uint32, U32P])
    sig(L, "lucent_renderer_set_ray_sort", [VP, C.c_int32])
    sig(L, "lucent_renderer_set_top_levels", [VP, C.c_int32])
    sig(L, "lucent_renderer_set_wide_bvh", [VP, C.c_int32])
    sig(L, "lucent_renderer_set_pipelining", [VP, C.c_int32])
    sig(L, "lucent_renderer_create_view", [VP, C.c_uint32, C.c_uint32, C.POINTER(VP)])
    sig(L, "lucent_renderer_read_textures", [VP, U32P, U8P, U8P])
    sig(L, "lucent_renderer_set_materials", [VP, F32P, C.c_uint32])
    sig(L, "lucent_renderer_backward", [VP, C.c_uint32, C.c_uint32, F32P, F32P, F32P, VP])
    sig(L, "lucent_renderer_denoise", [VP, C.c_uint32, C.c_float, C.c_float, C.c_float, VP])
    sig(L, "lucent_renderer_display", [VP, C.c_float, C.c_int32, C.c_float, U8P, F32P, VP])
    sig(L, "lucent_renderer_display_view", [VP, C.c_uint32, C.c_uint32, C.c_float, C.c_int32, C.c_float, U8P, F32P, VP])
    sig(L, "lucent_renderer_read_denoised", [VP, F32P])
    sig(L, "lucent_bsdf_eval_tuples", [F32P, C.c_uint32, F32P])
    sig(L, "lucent_bsdf_grad_tuples", [F32P, C.c_uint32, F32P])
    sig(L, "lucent_png_unfilter", [U8P, C.c_uint32, C.c_uint32, C.c_uint32, U8P])


class BatchOptions(C.Structure):
    _fields_ = [("samples_per_wave", C.c_uint32), ("max_wave_paths", C.c_uint32), ("use_graph", C.c_int32),
                ("trace_blocks", C.c_uint32), ("shade_blocks", C.c_uint32), ("sort_rays", C.c_int32),
                ("top_levels", C.c_int32), ("wide_bvh", C.c_int32), ("scenes_per_wave", C.c_uint32),
                ("streams", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("closest_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("waves", C.c_uint32),
                ("graph_waves", C.c_uint32), ("wave_paths", C.c_uint32), ("kernel_launches", C.c_uint64)]


def declare_batch(L, sig):
    sig(L, "lucent_batch_create", [P(VP), C.c_uint32, P(VP)])
    sig(L, "lucent_batch_destroy", [VP], None)
    sig(L, "lucent_batch_set_options", [VP, P(BatchOptions)])
    sig(L, "lucent_batch_trace", [VP, C.c_uint32, VP])
    sig(L, "lucent_batch_check", [VP, VP, P(BatchStats)])
