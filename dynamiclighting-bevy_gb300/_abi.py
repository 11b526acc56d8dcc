"""ctypes mirror of include/dynlight.h (the C ABI of the GPU baker).

Field order and sizes match the header exactly; `tests/test_abi.py` checks the struct sizes
against the compiled library's own `sizeof` report.
"""
import ctypes as C

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
f32p = C.POINTER(C.c_float)


class DlAlphaTexture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgba8", u8p),
                ("cutoff", C.c_float), ("reserved", C.c_uint32)]


class DlMesh(C.Structure):
    _fields_ = [("id", C.c_uint64), ("content_hash", C.c_uint64), ("vertex_count", C.c_uint32),
                ("occludes", C.c_uint32), ("index_count", C.c_uint64), ("positions", f32p),
                ("normals", f32p), ("indices", u32p), ("uv1", f32p), ("uv0", f32p),
                ("alpha", C.POINTER(DlAlphaTexture)), ("albedo", C.c_float * 3),
                ("reserved", C.c_uint32)]


class DlLight(C.Structure):
    _fields_ = [("id", C.c_uint64), ("position", C.c_float * 3), ("radius", C.c_float),
                ("illumination", C.c_uint32), ("transparency", C.c_uint32),
                ("bounce_samples", C.c_uint32), ("bounce_intensity", C.c_float),
                ("bounce_compression", C.c_int32), ("shape", C.c_uint32),
                ("rotation", C.c_float * 4), ("size", C.c_float * 2)]


class DlBakeInput(C.Structure):
    _fields_ = [("meshes", C.POINTER(DlMesh)), ("mesh_count", C.c_uint64),
                ("lights", C.POINTER(DlLight)), ("light_count", C.c_uint64)]


class DlBakeOptions(C.Structure):
    _fields_ = [("pixel_density", C.c_float), ("max_lightmap_size", C.c_uint32),
                ("bounce_compression", C.c_uint32), ("dynamic_geometry", C.c_uint32),
                ("skip_bounce", C.c_uint32), ("photon_cube_resolution", C.c_uint32),
                ("area_light_samples", C.c_uint32), ("area_light_min_samples", C.c_uint32),
                ("sun_map_resolution", C.c_uint32), ("sky_samples", C.c_uint32),
                ("sky_probe_spacing", C.c_float), ("colored_bounce", C.c_uint32),
                ("seed", C.c_uint64)]


class DlProgress(C.Structure):
    _fields_ = [("cancel", C.c_uint32), ("stage", C.c_uint32), ("done", C.c_uint64),
                ("total", C.c_uint64)]


class DlBakeConfig(C.Structure):
    _fields_ = [("form", C.c_uint32), ("device", C.c_uint32), ("block_threads", C.c_uint32),
                ("chunk_texels", C.c_uint32), ("sample_lanes", C.c_uint32),
                ("blocks_per_sm", C.c_uint32), ("count_visits", C.c_uint32),
                ("refine_epsilon", C.c_float), ("no_autotune", C.c_uint32), ("host_bvh", C.c_uint32),
                ("max_device_mib", C.c_uint32), ("min_blocks", C.c_uint32),
                ("gather_min_blocks", C.c_uint32), ("reserved", C.c_uint32 * 1)]


class DlBakeReport(C.Structure):
    _fields_ = [("ms_total", C.c_double), ("ms_upload", C.c_double), ("ms_device", C.c_double),
                ("ms_visibility", C.c_double), ("ms_download", C.c_double),
                ("shadow_rays", C.c_uint64), ("bounce_rays", C.c_uint64),
                ("burial_rays", C.c_uint64), ("photon_rays", C.c_uint64), ("pairs", C.c_uint64),
                ("work_items", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("bvh_nodes", C.c_uint64), ("occluders", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("device_bytes", C.c_uint64),
                ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64),
                ("ms_stages", C.c_double * 8), ("ms_host", C.c_double * 4),
                ("retests", C.c_uint64), ("tuned_chunk_texels", C.c_uint32),
                ("tuned_sample_lanes", C.c_uint32), ("tuned_blocks_per_sm", C.c_uint32),
                ("tuned_stack_depth", C.c_uint32), ("tuned_min_blocks", C.c_uint32),
                ("tune_trials", C.c_uint32), ("ms_tune", C.c_double),
                ("tuned_gather_lanes", C.c_uint32), ("cancel_stops", C.c_uint32),
                ("gather_node_visits", C.c_uint64), ("gather_tri_tests", C.c_uint64),
                ("ms_gather", C.c_double), ("bounce_items", C.c_uint64),
                ("tuned_gather_min_blocks", C.c_uint32), ("tuned_gather_blocks_per_sm", C.c_uint32)]


class DlLightBvhNode(C.Structure):
    _fields_ = [("aabb_min", C.c_float * 3), ("left_first", C.c_uint32),
                ("aabb_max", C.c_float * 3), ("count", C.c_uint32)]


class DlBakedLight(C.Structure):
    _fields_ = [("id", C.c_uint64), ("origin", C.c_float * 3), ("radius", C.c_float),
                ("shape", C.c_uint32), ("rotation", C.c_float * 4), ("size", C.c_float * 2),
                ("bounce_bits", C.c_uint32), ("shadow_bits_per_texel", C.c_uint32)]


class DlBakedMesh(C.Structure):
    _fields_ = [("id", C.c_uint64), ("content_hash", C.c_uint64), ("resolution", C.c_uint32),
                ("occludes", C.c_uint32), ("triangles", u32p), ("word_count", C.c_uint64)]


class DlBakeStats(C.Structure):
    _fields_ = [("meshes", C.c_uint32), ("reserved", C.c_uint32), ("triangles", C.c_uint64),
                ("texels", C.c_uint64), ("rays", C.c_uint64), ("lights_removed", C.c_uint64),
                ("bounce_rays", C.c_uint64), ("triangle_words", C.c_uint64)]


class DlBakedSettings(C.Structure):
    _fields_ = [("bounce", C.c_uint32), ("colored_bounce", C.c_uint32),
                ("dynamic_geometry", C.c_uint32), ("pixel_density", C.c_float),
                ("max_lightmap_size", C.c_uint32), ("distance_cube_resolution", C.c_uint32)]


class DlSunMap(C.Structure):
    _fields_ = [("rows", C.c_float * 12), ("resolution", C.c_uint32), ("reserved", C.c_uint32),
                ("word_count", C.c_uint64), ("texels", u32p)]


class DlSkyProbes(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("spacing", C.c_float), ("counts", C.c_uint32 * 3),
                ("reserved", C.c_uint32), ("word_count", C.c_uint64), ("words", u32p)]


class DlBakedScene(C.Structure):
    _fields_ = [("settings", DlBakedSettings), ("light_count", C.c_uint64),
                ("lights", C.POINTER(DlBakedLight)), ("light_bvh_count", C.c_uint64),
                ("light_bvh", C.POINTER(DlLightBvhNode)), ("mesh_count", C.c_uint64),
                ("meshes", C.POINTER(DlBakedMesh)), ("distance_cube_words", C.c_uint64),
                ("distance_cubes", u32p), ("sun_map_count", C.c_uint64),
                ("sun_maps", C.POINTER(DlSunMap)), ("sky_probes", C.POINTER(DlSkyProbes)),
                ("stats", DlBakeStats)]


STRUCTS = {
    "dl_alpha_texture": DlAlphaTexture, "dl_mesh": DlMesh, "dl_light": DlLight,
    "dl_sun_map": DlSunMap, "dl_sky_probes": DlSkyProbes,
    "dl_bake_input": DlBakeInput, "dl_bake_options": DlBakeOptions, "dl_progress": DlProgress,
    "dl_bake_config": DlBakeConfig, "dl_bake_report": DlBakeReport,
    "dl_light_bvh_node": DlLightBvhNode, "dl_baked_light": DlBakedLight,
    "dl_baked_mesh": DlBakedMesh, "dl_bake_stats": DlBakeStats,
    "dl_baked_settings": DlBakedSettings, "dl_baked_scene": DlBakedScene,
}

# Every extern "C" symbol include/dynlight.h declares.
EXPORTS = [
    "dl_abi_version", "dl_status_string", "dl_last_error", "dl_bake", "dl_bake_ex",
    "dl_baked_scene_free", "dl_default_options", "dl_session_create", "dl_session_run",
    "dl_session_result", "dl_session_report", "dl_session_destroy", "dl_encode_payload",
    "dl_free", "dl_filter_bounce_window_noalloc", "dl_session_bounce_map", "dl_session_encode_payload",
    "dl_session_occluder_bvh", "dl_release_memory", "dl_probe_read_bandwidth",
]

STATUS = {0: "ok", 1: "cancelled", 2: "duplicate id", 3: "invalid mesh", 4: "invalid light",
          5: "invalid options", 16: "cuda error", 17: "out of memory", 18: "queue timeout",
          19: "busy", 20: "unsupported", 21: "invalid argument"}
