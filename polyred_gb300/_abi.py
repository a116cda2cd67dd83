"""ctypes mirror of include/polyred_cuda.h (layouts must match the header).

Shared by the product loader (polyred_gb300.native) and by the test-side
oracle loader, so both read the same scene/frame/output descriptors.
"""
import ctypes as C

ABI_VERSION = 1

PR_OK = 0
PR_ERR_INVALID_ARG = -1
PR_ERR_OOM = -2
PR_ERR_CUDA = -3
PR_ERR_OVERFLOW = -4
PR_ERR_TIMEOUT = -5
PR_ERR_UNIMPLEMENTED = -6
PR_ERR_NO_SCENE = -7
PR_ERR_UNSUPPORTED = -8
PR_ERR_NO_DEVICE = -9
PR_ERR_SINGULAR = -10
PR_ERR_FATAL = -11

PR_MAT_FLAT_SHADING = 1
PR_MAT_AO = 2
PR_MAT_RECEIVE_SHADOW = 4
PR_MAT_MIPMAP = 8

PR_LIGHT_POINT = 0
PR_LIGHT_DIRECTIONAL = 1

PR_FRAME_PERSPECTIVE = 1
PR_FRAME_SHADOWMAP = 2
PR_FRAME_GAMMA = 4

PR_SCENE_DEVICE_PTRS = 1
PR_OUT_DEVICE_PTRS = 1

PR_TRI_NONE = 0xFFFFFFFF

PR_OBJ_TEXT_OBJ = 0
PR_OBJ_TEXT_MTL = 1
PR_OBJ_NO_INDEX = 4294967295

F16 = C.c_float * 16


class pr_object(C.Structure):
    _fields_ = [("first_tri", C.c_uint32), ("n_tris", C.c_uint32), ("mat_base", C.c_int32),
                ("reserved", C.c_uint32), ("model", F16)]


class pr_material(C.Structure):
    _fields_ = [("diffuse", C.c_uint8 * 4), ("specular", C.c_uint8 * 4), ("texture", C.c_uint8 * 4),
                ("shininess", C.c_float), ("flags", C.c_uint32), ("texture_size", C.c_int32)]


class pr_texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgba", C.c_void_p)]


PR_SCENE_DESC_SIZE_V1 = 80


class pr_scene_desc(C.Structure):
    _fields_ = [("size", C.c_uint32), ("flags", C.c_uint32), ("n_tris", C.c_uint32),
                ("n_objects", C.c_uint32), ("n_materials", C.c_uint32), ("reserved", C.c_uint32),
                ("pos", C.c_void_p), ("nor", C.c_void_p), ("uv", C.c_void_p), ("col", C.c_void_p),
                ("mat_id", C.c_void_p), ("objects", C.POINTER(pr_object)),
                ("materials", C.POINTER(pr_material)),
                ("textures", C.c_void_p)]


class pr_light(C.Structure):
    _fields_ = [("type", C.c_int32), ("cast_shadow", C.c_int32), ("pos", C.c_float * 3),
                ("dir", C.c_float * 3), ("intensity", C.c_float), ("color", C.c_uint8 * 4),
                ("shadow_view", F16), ("shadow_proj", F16)]


class pr_frame_desc(C.Structure):
    _fields_ = [("size", C.c_uint32), ("flags", C.c_uint32), ("width", C.c_int32), ("height", C.c_int32),
                ("view", F16), ("proj", F16), ("cam_pos", C.c_float * 3), ("background", C.c_uint8 * 4),
                ("n_lights", C.c_uint32), ("n_ambient", C.c_uint32), ("lights", C.POINTER(pr_light)),
                ("ambient", C.POINTER(C.c_float)), ("shadow_width", C.c_int32),
                ("shadow_height", C.c_int32), ("msaa", C.c_int32), ("reserved", C.c_int32)]


PR_FRAME_DESC_SIZE_V1 = 192


class pr_outputs(C.Structure):
    _fields_ = [("size", C.c_uint32), ("flags", C.c_uint32), ("rgba", C.c_void_p), ("tri_id", C.c_void_p),
                ("depth", C.c_void_p), ("nor", C.c_void_p), ("face_nor", C.c_void_p),
                ("world_pos", C.c_void_p), ("uvd", C.c_void_p), ("vcol", C.c_void_p),
                ("mat_id", C.c_void_p), ("shadow_maps", C.c_void_p)]


class pr_stats(C.Structure):
    _fields_ = [("size", C.c_uint32), ("n_tris_in", C.c_uint32), ("n_raster_tris", C.c_uint32),
                ("n_clipped_tris", C.c_uint32), ("n_raster_tasks", C.c_uint32), ("n_nan_fragments", C.c_uint32),
                ("n_kernel_launches", C.c_uint32), ("reserved", C.c_uint32), ("ms_shadow", C.c_float),
                ("ms_setup", C.c_float), ("ms_raster", C.c_float), ("ms_shade", C.c_float),
                ("ms_total", C.c_float), ("ms_ao", C.c_float), ("n_ao_pixels", C.c_uint32)]


PR_NOALLOC_MAX_TRIS = 65536
PR_NOALLOC_MAX_OBJECTS = 256
PR_NOALLOC_MAX_TEXELS = 1048576
PR_NOALLOC_MAX_TASKS = 262144


class pr_depth_map_desc(C.Structure):
    _fields_ = [("size", C.c_uint32), ("n_tris", C.c_uint32), ("n_objects", C.c_uint32), ("width", C.c_int32),
                ("height", C.c_int32), ("reserved", C.c_uint32), ("pos", C.c_void_p),
                ("objects", C.POINTER(pr_object)), ("view", F16), ("proj", F16), ("depth", C.c_void_p),
                ("stream", C.c_void_p)]


# Every entry point include/polyred_cuda.h declares: (name, restype, argtypes).
VP = C.c_void_p
FP = C.POINTER(C.c_float)
PR_DGB_FLOATS = 16
# differentiation G-buffer pixel flags (float 2 of a pixel)
DGB_LIT, DGB_FLAT, DGB_CONST, DGB_UNLIT = 1, 2, 4, 8
DP = C.POINTER(C.c_double)


class pr_diff_params(C.Structure):
    _fields_ = [
        ("size", C.c_uint32),
        ("n_materials", C.c_uint32),
        ("vertex_color", VP),
        ("vertex_normal", VP),
        ("kd", FP),
        ("ks", FP),
        ("shininess", FP),
    ]


class pr_diff_grads(C.Structure):
    _fields_ = [
        ("size", C.c_uint32),
        ("reserved", C.c_uint32),
        ("vertex_color", VP),
        ("vertex_normal", VP),
        ("kd", DP),
        ("ks", DP),
        ("shininess", DP),
        ("light_pos", DP),
        ("light_intensity", DP),
        ("ambient", DP),
    ]


class pr_batch_view(C.Structure):
    _fields_ = [
        ("scene", C.c_uint32),
        ("reserved", C.c_uint32),
        ("frame", C.POINTER(pr_frame_desc)),
        ("out", C.POINTER(pr_outputs)),
    ]


class pr_batch_stats(C.Structure):
    _fields_ = [
        ("size", C.c_uint32),
        ("n_views", C.c_uint32),
        ("n_passes", C.c_uint32),
        ("n_kernel_launches", C.c_uint32),
        ("graph_reused", C.c_uint32),
        ("n_fallback_views", C.c_uint32),
        ("n_retries", C.c_uint32),
        ("task_px", C.c_uint32),
        ("raster_blocks", C.c_uint32),
        ("reserved", C.c_uint32),
        ("ms_total", C.c_double),
        ("device_bytes", C.c_uint64),
    ]


class pr_obj_material(C.Structure):
    _fields_ = [("name", C.c_int32), ("map_kd", C.c_int32), ("illum", C.c_int32), ("opacity", C.c_float),
                ("refraction", C.c_float), ("shininess", C.c_float), ("ambient", C.c_uint8 * 4),
                ("diffuse", C.c_uint8 * 4), ("specular", C.c_uint8 * 4), ("emissive", C.c_uint8 * 4)]


class pr_obj_info(C.Structure):
    _fields_ = [
        ("size", C.c_uint32), ("reserved", C.c_uint32),
        ("vertices", C.POINTER(C.c_float)), ("n_vertices", C.c_int64),
        ("normals", C.POINTER(C.c_float)), ("n_normals", C.c_int64),
        ("uvs", C.POINTER(C.c_float)), ("n_uvs", C.c_int64),
        ("n_faces", C.c_int64), ("n_corners", C.c_int64),
        ("face_start", C.POINTER(C.c_int64)), ("corner_v", C.POINTER(C.c_int64)),
        ("corner_vt", C.POINTER(C.c_int64)), ("corner_vn", C.POINTER(C.c_int64)),
        ("face_object", C.POINTER(C.c_int32)), ("face_material", C.POINTER(C.c_int32)),
        ("face_smooth", C.POINTER(C.c_uint8)),
        ("n_objects", C.c_int64), ("object_name", C.POINTER(C.c_int32)),
        ("object_mat_start", C.POINTER(C.c_int64)), ("object_mat", C.POINTER(C.c_int32)),
        ("n_materials", C.c_int64), ("materials", C.POINTER(pr_obj_material)),
        ("n_warnings", C.c_int64), ("warnings", C.POINTER(C.c_int32)),
        ("strings", C.c_void_p), ("strings_len", C.c_int64),
        ("matlib", C.c_int32), ("current_material", C.c_int32), ("line", C.c_int64),
        ("error", C.c_void_p), ("error_len", C.c_int64),
    ]


ENTRY_POINTS = [
    ("pr_abi_version", C.c_int, []),
    ("pr_error_string", C.c_char_p, [C.c_int]),
    ("pr_last_error", C.c_char_p, []),
    ("pr_create", C.c_int, [C.c_int, C.POINTER(VP)]),
    ("pr_destroy", C.c_int, [VP]),
    ("pr_scene_upload", C.c_int, [VP, C.POINTER(pr_scene_desc)]),
    ("pr_shadow_reset", C.c_int, [VP]),
    ("pr_render", C.c_int, [VP, C.POINTER(pr_frame_desc), C.POINTER(pr_outputs)]),
    ("pr_render_async", C.c_int, [VP, C.POINTER(pr_frame_desc), C.POINTER(pr_outputs)]),
    ("pr_sync", C.c_int, [VP]),
    ("pr_frame_submit", C.c_int, [VP, C.POINTER(pr_scene_desc), C.POINTER(pr_frame_desc), C.POINTER(pr_outputs)]),
    ("pr_frame_stats", C.c_int, [VP, C.POINTER(pr_stats)]),
    ("pr_stream", C.c_int, [VP, C.POINTER(VP)]),
    ("pr_host_alloc", C.c_int, [C.c_size_t, C.POINTER(VP)]),
    ("pr_host_free", C.c_int, [VP]),
    ("pr_device_alloc", C.c_int, [VP, C.c_size_t, C.POINTER(VP)]),
    ("pr_device_free", C.c_int, [VP, VP]),
    ("pr_device_read", C.c_int, [VP, VP, C.c_size_t, VP]),
    ("pr_view_matrix", C.c_int, [FP, FP, FP, FP]),
    ("pr_perspective_matrix", C.c_int, [C.c_float, C.c_float, C.c_float, C.c_float, FP]),
    ("pr_orthographic_matrix", C.c_int, [C.c_float] * 6 + [FP]),
    ("pr_mat4_mul", C.c_int, [FP, FP, FP]),
    ("pr_mat4_inv", C.c_int, [FP, FP]),
    ("pr_shadow_camera", C.c_int, [FP, FP, FP, FP, FP, FP]),
    ("pr_depth_map_noalloc", C.c_int, [C.POINTER(pr_depth_map_desc)]),
    ("pr_batch_create", C.c_int, [C.c_int, C.POINTER(VP)]),
    ("pr_batch_destroy", C.c_int, [VP]),
    ("pr_batch_add_scene", C.c_int, [VP, C.POINTER(pr_scene_desc), C.POINTER(C.c_uint32)]),
    ("pr_batch_render", C.c_int, [VP, C.c_uint32, C.POINTER(pr_batch_view)]),
    ("pr_batch_tune", C.c_int, [VP, C.c_uint32, C.POINTER(pr_batch_view), C.c_char_p, C.c_size_t]),
    ("pr_batch_get_stats", C.c_int, [VP, C.POINTER(pr_batch_stats)]),
    ("pr_diff_forward", C.c_int, [VP, C.POINTER(pr_frame_desc), C.POINTER(pr_diff_params), VP, VP,
                                  C.POINTER(pr_outputs)]),
    ("pr_diff_backward", C.c_int, [VP, C.POINTER(pr_frame_desc), C.POINTER(pr_diff_params), VP, VP,
                                   C.POINTER(pr_diff_grads)]),
    ("pr_obj_create", C.c_int, [C.POINTER(VP)]),
    ("pr_obj_destroy", C.c_int, [VP]),
    ("pr_obj_parse", C.c_int, [VP, C.c_int, C.c_char_p, C.c_size_t]),
    ("pr_obj_get", C.c_int, [VP, C.POINTER(pr_obj_info)]),
    ("pr_srgb_decode_table", C.c_int, [VP]),
    ("pr_png_unfilter", C.c_int, [VP, C.c_int, C.c_size_t, C.c_int, VP]),
]


# include/polyred_cuda_testing.h: test hooks, bound by the tests only
TESTING_ENTRY_POINTS = [
    ("pr_testing_fail_alloc", C.c_int, [C.c_int64]),
    ("pr_testing_alloc_count", C.c_int64, []),
    ("pr_debug_ao_dirs", C.c_int, [C.c_int, C.c_int] + [VP] * 4),
    ("pr_debug_pow_probe", C.c_int, [VP] * 4 + [C.c_int]),
    ("pr_debug_ao_probe", C.c_int, [VP] * 7 + [C.c_int]),
    ("pr_debug_fma_probe", C.c_int, [VP] * 5 + [C.c_int]),
    ("pr_debug_texture_build", C.c_longlong, [C.c_int, C.c_int, VP, C.c_int, VP, C.c_size_t, VP]),
    ("pr_debug_texture_query", C.c_int, [C.c_int, C.c_int, VP, C.c_int, C.c_int] + [VP] * 6),
]


def bind(lib, entry_points=None):
    """Set restype/argtypes for every declared entry point on a CDLL."""
    for name, res, args in (ENTRY_POINTS if entry_points is None else entry_points):
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def bind_testing(lib):
    """Also bind the test hooks of include/polyred_cuda_testing.h."""
    return bind(lib, TESTING_ENTRY_POINTS)
