/*
 * dynlight GB300 baker: the C ABI.
 *
 * One blocking call bakes a scene on one GPU and returns what the reference's
 *
 *     pub fn bake(input: &BakeInput, options: &BakeOptions, progress: &BakeProgress)
 *         -> Result<BakedScene, BakeError>                      (src/bake/baker.rs:27-31)
 *
 * returns: per mesh the `dynamic_triangles` words (src/bake/triangle_words.rs:1-13), the lights
 * in light-BVH slot order (src/bake/baker.rs:41-50), the light BVH nodes
 * (src/bake/light_bvh.rs:16-22), the distance cubes, sun maps and sky probes for moving meshes
 * (src/bake/baker.rs:114-152) and the bake statistics (src/bake/format/types.rs:205-222).
 * Every struct is plain data with explicit sizes so a Rust `#[repr(C)]` mirror binds it
 * directly; no C++ or CUDA type crosses the boundary, and no exception leaves it.
 *
 * Ownership: the caller owns every input array, which is read during the call only. Results
 * live in a library allocation freed with dl_baked_scene_free(); the library keeps up to 2 GiB
 * of freed results' word buffers to reuse for later results. Device memory is owned by the
 * library. One dl_bake / dl_bake_ex runs at a time per process (a second concurrent call returns
 * DL_BUSY); a dl_session is used by one thread at a time.
 */
#ifndef DYNLIGHT_GB300_H
#define DYNLIGHT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DL_ABI_VERSION 2u

/* Status codes. The first five mirror BakeError (src/bake/input.rs:198-209). */
typedef enum dl_status {
    DL_OK = 0,
    DL_CANCELLED = 1,       /* BakeError::Cancelled, through dl_progress.cancel */
    DL_DUPLICATE_ID = 2,    /* BakeError::DuplicateId (src/bake/baker.rs:205-233) */
    DL_INVALID_MESH = 3,    /* BakeError::InvalidMesh (src/bake/input.rs:233-287) */
    DL_INVALID_LIGHT = 4,   /* BakeError::InvalidLight (src/bake/input.rs:290-323) */
    DL_INVALID_OPTIONS = 5, /* BakeError::InvalidOptions (src/bake/input.rs:336-373) */
    DL_CUDA_ERROR = 16,     /* a CUDA call failed; dl_last_error() names it */
    DL_OUT_OF_MEMORY = 17,  /* device or host allocation failed */
    DL_QUEUE_TIMEOUT = 18,  /* reserved, never returned: the work queue is claimed with atomic
                               counters and no kernel of this library waits on another thread,
                               so there is no device wait to bound */
    DL_BUSY = 19,           /* another bake is running in this process */
    DL_UNSUPPORTED = 20,    /* a scene this library cannot bake (a map side above 65535 texels,
                               an occluder BVH deeper than the traversal stack) */
    DL_INVALID_ARGUMENT = 21
} dl_status;

/* Light shape codes, as the .dynlight lights section stores them (src/bake/format/lights.rs:27-54). */
typedef enum dl_light_shape {
    DL_SHAPE_POINT = 0,
    DL_SHAPE_RECTANGLE = 1,
    DL_SHAPE_TUBE = 2,
    DL_SHAPE_SUN = 3,
    DL_SHAPE_SKY = 4
} dl_light_shape;

/* Illumination (src/light/kinds.rs:97-103). */
enum { DL_ILLUMINATION_DIRECT = 0, DL_ILLUMINATION_SINGLE_BOUNCE = 1 };
/* Transparency (src/light/kinds.rs:108-118): anything but Disabled alpha-tests shadow rays. */
enum { DL_TRANSPARENCY_DISABLED = 0, DL_TRANSPARENCY_ENABLED = 1, DL_TRANSPARENCY_ENABLED_MAX = 2 };
/* DynamicGeometryMode (src/shared/settings.rs:229-237). */
enum { DL_GEOMETRY_LIGHTING_ONLY = 0, DL_GEOMETRY_DISTANCE_CUBES = 1, DL_GEOMETRY_ANGULAR = 2 };

/* AlphaTexture (src/bake/input.rs:62-97): RGBA8 rows top to bottom. */
typedef struct dl_alpha_texture {
    uint32_t width;
    uint32_t height;
    const uint8_t *rgba8; /* width * height * 4 bytes */
    float cutoff;
    uint32_t reserved;
} dl_alpha_texture;

/* BakeMesh (src/bake/input.rs:24-45), world space. */
typedef struct dl_mesh {
    uint64_t id;               /* BakeId */
    uint64_t content_hash;
    uint32_t vertex_count;
    uint32_t occludes;         /* 0 or 1 */
    uint64_t index_count;      /* multiple of 3 */
    const float *positions;    /* vertex_count * 3 */
    const float *normals;      /* vertex_count * 3, or NULL for flat (face) normals */
    const uint32_t *indices;   /* index_count */
    const float *uv1;          /* vertex_count * 2: shadow map coordinates */
    const float *uv0;          /* vertex_count * 2, or NULL */
    const dl_alpha_texture *alpha; /* NULL: opaque; needs uv0 */
    float albedo[3];           /* mean linear reflected color; colored bounce reads it */
    uint32_t reserved;
} dl_mesh;

/* BakeLight (src/bake/input.rs:101-122) with its LightShape (src/light/shape.rs:19-30). */
typedef struct dl_light {
    uint64_t id;
    float position[3];
    float radius;
    uint32_t illumination;       /* DL_ILLUMINATION_* */
    uint32_t transparency;       /* DL_TRANSPARENCY_* */
    uint32_t bounce_samples;     /* BakeBounce.samples (at least 2 are taken) */
    float bounce_intensity;      /* BakeBounce.intensity */
    int32_t bounce_compression;  /* bits per bounce pixel 8/6/5/4, or -1 for the options' */
    uint32_t shape;              /* dl_light_shape */
    float rotation[4];           /* quaternion x, y, z, w (rectangle, tube, sun) */
    float size[2];               /* rectangle: width, height; tube: length, 0;
                                    sun: angular diameter in degrees, 0 */
} dl_light;

typedef struct dl_bake_input {
    const dl_mesh *meshes;
    uint64_t mesh_count;
    const dl_light *lights;
    uint64_t light_count;
} dl_bake_input;

/* BakeOptions (src/bake/input.rs:136-164). */
typedef struct dl_bake_options {
    float pixel_density;
    uint32_t max_lightmap_size;
    uint32_t bounce_compression;     /* bits per pixel: 8, 6, 5 or 4 */
    uint32_t dynamic_geometry;       /* DL_GEOMETRY_* */
    uint32_t skip_bounce;
    uint32_t photon_cube_resolution;
    uint32_t area_light_samples;
    uint32_t area_light_min_samples;
    uint32_t sun_map_resolution;
    uint32_t sky_samples;
    float sky_probe_spacing;
    uint32_t colored_bounce;
    uint64_t seed;
} dl_bake_options;

/* BakeProgress (src/bake/progress.rs:41-110). The caller may set `cancel` from any thread;
 * the library polls it between stages and the device work queue stops at its next item. It is
 * first read after validation, as in the reference (src/bake/baker.rs:32-55): invalid input
 * reports its own error even when the flag was set before the call. */
typedef struct dl_progress {
    volatile uint32_t cancel;
    volatile uint32_t stage; /* BakeStage order (src/bake/progress.rs:8-16) */
    volatile uint64_t done;
    volatile uint64_t total;
} dl_progress;

/* How the bake runs. BATCHED and PLAIN give identical bytes, bit-exact with the reference's
   binary32 arithmetic. REFINED is the batched form with three precision changes: ray/triangle
   tests whose binary32 barycentrics, determinant or hit distance fall within `refine_epsilon` of
   a boundary are re-tested in binary64; closest hits are chosen by the candidates' binary64
   distances (with their barycentrics); soft-visibility weights and bounce gathers are summed
   with compensated (Kahan) sums. Its bytes may differ from the other forms where those change a
   level. */
enum {
    DL_FORM_BATCHED = 0, /* every (triangle, light) pair through one persistent kernel fed by a
                            device work queue, launched from a CUDA graph */
    DL_FORM_PLAIN = 1,   /* one launch per mesh, a warp per triangle looping over its lights and
                            texels: the reference's loop order on the GPU */
    DL_FORM_REFINED = 2, /* the batched form with binary64 edge re-tests and compensated sums */
    DL_FORM_BOUNCE_REFINED = 3 /* the batched form's bit-exact visibility and burial (its masks
                            are the BATCHED form's, bit for bit) with the REFINED form's photon
                            cubes, bounce gathers and compensated bounce sums (its bounce follows
                            an FP64 bake) */
};

/* Launch configuration of one bake; zero-initialise for the defaults. */
typedef struct dl_bake_config {
    uint32_t form;             /* DL_FORM_* */
    uint32_t device;           /* CUDA device ordinal */
    uint32_t block_threads;    /* 0: tuned default */
    uint32_t chunk_texels;     /* (pair, texel) items a warp claims from the queue at once, 0: tuned */
    uint32_t sample_lanes;     /* lanes sharing one texel's sky samples and bounce-gather samples
                                  (1, 2, 4, 8, 16 or 32), 0: tuned */
    uint32_t blocks_per_sm;    /* upper bound of persistent blocks per SM, 0: as many as fit */
    uint32_t count_visits;     /* 1: run the instrumented visibility kernel that counts BVH node
                                  visits and triangle tests (for roofline accounting; slower) */
    float refine_epsilon;      /* DL_FORM_REFINED: re-test margin (barycentric units; times
                                  max(1, ray length) for distances), 0: 1e-4 */
    uint32_t no_autotune;      /* 1: never time candidate launch shapes; unset knobs take defaults.
                                  0: knobs left 0 are picked by timing trials on the first run of a
                                  scene shape (cached per process) */
    uint32_t host_bvh;         /* 1: build the occluder BVH on the host's cores and upload it;
                                  0: build it on the device (the same tree, in milliseconds) */
    uint32_t max_device_mib;   /* cap on the device memory one bake (session) may hold, in MiB:
                                  scene, BVH and its build scratch, every stage's buffers. An
                                  allocation past it fails the call with DL_OUT_OF_MEMORY and
                                  frees what the bake held. 0: no cap */
    uint32_t min_blocks;       /* register budget of the bit-exact visibility kernel, as the
                                  blocks of 128 threads per SM it is compiled to fit: 7, 8, 9, 10
                                  or 12 (72, 64, 56, 48 or 40 registers per thread), 0: tuned.
                                  The refined and counting kernels have one budget (7) */
    uint32_t gather_min_blocks; /* the same for the bit-exact bounce gather: 6, 8, 9 or 10 (80,
                                  64, 56 or 48 registers), 0: tuned; the refined gather has one (8) */
    uint32_t reserved[1];
} dl_bake_config;

/* Timings (device events, milliseconds) and counters of the last bake. */
typedef struct dl_bake_report {
    double ms_total;          /* host wall clock of the whole call */
    double ms_upload;         /* host -> device copies and BVH build */
    double ms_device;         /* device time of the bake pipeline, events on its stream */
    double ms_visibility;     /* device time of the visibility stage alone */
    double ms_download;       /* device -> host copies and serialization */
    uint64_t shadow_rays;     /* BakeStats.rays */
    uint64_t bounce_rays;     /* BakeStats.bounce_rays */
    uint64_t burial_rays;     /* closest-hit rays of the burial test */
    uint64_t photon_rays;     /* closest-hit rays of the photon cubes */
    uint64_t pairs;           /* (triangle, light) pairs traced */
    uint64_t work_items;      /* items of the device work queue */
    uint64_t kernel_launches; /* kernels this library launched for the bake */
    uint64_t bvh_nodes;
    uint64_t occluders;
    uint64_t h2d_bytes;
    uint64_t d2h_bytes;
    uint64_t device_bytes;    /* peak device memory held by the bake */
    uint64_t node_visits;     /* BVH nodes visited by the visibility stage (counting config only) */
    uint64_t tri_tests;       /* triangle tests of the visibility stage (counting config only) */
    double ms_stages[8];      /* device time per stage: setup+association, texels, burial,
                                 visibility (with its queue), bounce, optimize+seams,
                                 serialization+crop+packing, unused */
    double ms_host[4];        /* host time of session creation: validation + sorting + lights,
                                 occluder BVH build, flattening + uploads, unused */
    uint64_t retests;         /* DL_FORM_REFINED: ray/triangle tests re-run in binary64 (tests
                                 near a boundary, and every closest-hit candidate) */
    /* launch shape of the batched visibility kernel (picked by the autotuner or the config) */
    uint32_t tuned_chunk_texels, tuned_sample_lanes, tuned_blocks_per_sm, tuned_stack_depth;
    uint32_t tuned_min_blocks;  /* launch bound: blocks per SM the registers were sized for */
    uint32_t tune_trials;       /* candidate shapes timed in this run (0: defaults or cached) */
    double ms_tune;             /* host time of those trials */
    uint32_t tuned_gather_lanes; /* lanes sharing one texel's samples in the bounce gather */
    uint32_t cancel_stops;       /* warps of the device work queues that saw the cancel flag and
                                    stopped claiming work (a cancelled run; 0 otherwise) */
    uint64_t gather_node_visits; /* BVH nodes visited by the bounce gather (counting config only) */
    uint64_t gather_tri_tests;   /* triangle tests of the bounce gather (counting config only) */
    double ms_gather;            /* device time of the bounce gather kernel alone (0: no gather) */
    uint64_t bounce_items;       /* (bounce pair, texel) items of the gather queue */
    uint32_t tuned_gather_min_blocks;   /* gather launch bound: blocks per SM its registers fit */
    uint32_t tuned_gather_blocks_per_sm; /* gather blocks resident per SM in the launch */
} dl_bake_report;

/* LightBvhNode (src/bake/light_bvh.rs:16-22), 32 bytes. */
typedef struct dl_light_bvh_node {
    float aabb_min[3];
    uint32_t left_first;
    float aabb_max[3];
    uint32_t count;
} dl_light_bvh_node;

/* BakedLight (src/bake/format/types.rs:161-175). */
typedef struct dl_baked_light {
    uint64_t id;
    float origin[3];
    float radius;
    uint32_t shape;                 /* dl_light_shape */
    float rotation[4];
    float size[2];
    uint32_t bounce_bits;           /* 0: no baked bounce */
    uint32_t shadow_bits_per_texel; /* 1, 4 or 8 */
} dl_baked_light;

/* BakedMesh (src/bake/format/types.rs:178-190). */
typedef struct dl_baked_mesh {
    uint64_t id;
    uint64_t content_hash;
    uint32_t resolution;
    uint32_t occludes;
    const uint32_t *triangles; /* the mesh's dynamic_triangles words */
    uint64_t word_count;
} dl_baked_mesh;

/* BakeStats (src/bake/format/types.rs:205-222). */
typedef struct dl_bake_stats {
    uint32_t meshes;
    uint32_t reserved;
    uint64_t triangles;
    uint64_t texels;
    uint64_t rays;
    uint64_t lights_removed;
    uint64_t bounce_rays;
    uint64_t triangle_words;
} dl_bake_stats;

/* BakedSettings (src/bake/format/types.rs:128-145). */
typedef struct dl_baked_settings {
    uint32_t bounce;
    uint32_t colored_bounce;
    uint32_t dynamic_geometry;
    float pixel_density;
    uint32_t max_lightmap_size;
    uint32_t distance_cube_resolution;
} dl_baked_settings;

/* SunMap (src/bake/format/types.rs:115-128): map space coordinate i of world point p is
 * rows[4i..4i+2] . p + rows[4i+3]; `resolution`^2 unorm16 depths, two per word (texel 2k low). */
typedef struct dl_sun_map {
    float rows[12];
    uint32_t resolution;
    uint32_t reserved;
    uint64_t word_count;
    const uint32_t *texels;
} dl_sun_map;

/* SkyProbes (src/bake/format/types.rs:72-113): probe (x, y, z) at origin + spacing * (x, y, z),
 * two words per probe (x fastest), the openness of +X, -X, +Y, -Y, +Z, -Z as unorm8. */
typedef struct dl_sky_probes {
    float origin[3];
    float spacing;
    uint32_t counts[3];
    uint32_t reserved;
    uint64_t word_count;
    const uint32_t *words;
} dl_sky_probes;

/* BakedScene (src/bake/format/types.rs:13-37). With DL_GEOMETRY_LIGHTING_ONLY the distance
 * cubes, sun maps and sky probes are empty, as in the reference (src/bake/baker.rs:114-152). */
typedef struct dl_baked_scene {
    dl_baked_settings settings;
    uint64_t light_count;
    const dl_baked_light *lights;
    uint64_t light_bvh_count;
    const dl_light_bvh_node *light_bvh;
    uint64_t mesh_count;
    const dl_baked_mesh *meshes;
    uint64_t distance_cube_words;   /* 6 x 64^2 f16 distances per local light, two per word */
    const uint32_t *distance_cubes;
    uint64_t sun_map_count;         /* one per sun in light order, or none */
    const dl_sun_map *sun_maps;
    const dl_sky_probes *sky_probes; /* NULL: none */
    dl_bake_stats stats;
} dl_baked_scene;

/* Library version, DL_ABI_VERSION. */
uint32_t dl_abi_version(void);

/* Human-readable name of a status. */
const char *dl_status_string(dl_status status);

/* Detail of the last failure on the calling thread (validation reason, CUDA error). */
const char *dl_last_error(void);

/* Replaces bake() (src/bake/baker.rs:27-203) with the batched form and default tuning.
 * `progress` may be NULL. On DL_OK `*out` holds the result. */
dl_status dl_bake(const dl_bake_input *input, const dl_bake_options *options,
                  dl_progress *progress, dl_baked_scene **out);

/* dl_bake with an explicit form and tuning; `report` (may be NULL) receives timings. */
dl_status dl_bake_ex(const dl_bake_input *input, const dl_bake_options *options,
                     const dl_bake_config *config, dl_progress *progress,
                     dl_baked_scene **out, dl_bake_report *report);

void dl_baked_scene_free(dl_baked_scene *scene);

/* The reference's option defaults (BakeOptions::default, src/bake/input.rs:166-194 with
 * BakeSettings::default, src/bake/settings.rs:67-81). */
void dl_default_options(dl_bake_options *options);

/* ---- Device-resident sessions: the same bake split at its host<->device boundaries, so a
 * caller can repeat the device part on resident inputs (the benchmark's kernel-only number). */
typedef struct dl_session dl_session;

/* Validates and sorts the input, builds the light and occluder BVHs and uploads the scene. */
dl_status dl_session_create(const dl_bake_input *input, const dl_bake_options *options,
                            const dl_bake_config *config, dl_session **out);
/* Runs every device stage of the bake on the resident scene; results stay on the device. */
dl_status dl_session_run(dl_session *session, dl_progress *progress);
/* Downloads the last run's results and serializes them. */
dl_status dl_session_result(dl_session *session, dl_baked_scene **out);
dl_status dl_session_report(const dl_session *session, dl_bake_report *report);
/* encode's payload (src/bake/format/mod.rs:101-119,170-213) of the session's last run, assembled
 * on the device next to the resident words, with its CRC-32 computed there: the same bytes as
 * dl_encode_payload on dl_session_result's scene. `*bytes` is freed with dl_free; the gzip
 * layer stays with the caller. */
dl_status dl_session_encode_payload(dl_session *session, uint8_t **bytes, uint64_t *length, uint32_t *crc);
/* No counterpart in the reference (whose occluder BVH is internal to Occluders,
   src/bake/occluder.rs:63-114): a copy of the session's occluder BVH as the traversal reads it —
   up to `node_cap` 64-byte nodes (child boxes c0, c1, c2 as 12 floats, then the two child
   references as int32: >= 0 an inner node, < 0 a leaf ~(first << 3 | count), ~0 empty, then two
   zero words) and up to `tri_cap` triangles in leaf order (12 floats: v0 with the occluder index's
   bits in the fourth, e1 and e2 with a zero fourth). `*node_count` and `*depth` (the deepest
   level, the root being 1) are set either way. For tests and tools. */
dl_status dl_session_occluder_bvh(dl_session *session, void *nodes, uint64_t node_cap, float *triangles,
                                  uint64_t tri_cap, uint32_t *node_count, uint32_t *depth);
/* No counterpart in the reference (whose BounceMap is internal to bake_mesh_bounce,
   src/bake/bounce.rs:155-217): the last run's filtered bounce map of (mesh id, light slot) —
   its window (min_x, min_y, max_x, max_y) and up to `cap` RGB texels row-major over the window,
   before quantization. `*texels` gets the window's texel count, 0 when the pair has no map.
   For precision reports of bounce irradiance. */
dl_status dl_session_bounce_map(dl_session *session, uint64_t mesh_id, uint32_t slot, uint32_t rect[4],
                                float *rgb, uint32_t cap, uint32_t *texels);
void dl_session_destroy(dl_session *session);
/* No counterpart in the reference: device memory that finished sessions freed stays in the
   device's stream-ordered pool, and downloaded results' pinned host buffers stay cached, for the
   next bake; this hands both back (to the driver and the host). Call it between bakes. */
void dl_release_memory(void);

/* ---- .dynlight payload (src/bake/format/mod.rs:101-213): the uncompressed payload bytes and
 * its CRC-32 (IEEE). The file's gzip layer is left to the caller's deflate library. */
dl_status dl_encode_payload(const dl_baked_scene *scene, uint8_t **bytes, uint64_t *length,
                            uint32_t *crc32);
void dl_free(void *pointer);

/* ---- Non-allocating bounce filter. No counterpart in the reference: its BounceMap filter
 * (src/bake/bounce_map.rs:67-112) runs only inside bake(). For callers that cannot allocate
 * device memory (a fixed engine memory budget, code running while a stream is captured, a frame
 * thread), this applies the same dilation and 7-tap separable blur to one window of a bounce map
 * held in caller-owned device buffers and allocates nothing.
 *
 * in_rgb / out_rgb: device buffers of width * height RGB float triples, row-major, whose byte
 * ranges do not overlap (else DL_INVALID_ARGUMENT); the window covers map texels
 * [x0, x0 + width) x [y0, y0 + height) of a map_size^2 map (the blur clamps to the map and reads
 * 0 outside the window, as the bake does). At most DL_NOALLOC_MAX_TEXELS texels, else
 * DL_INVALID_ARGUMENT; both checks come before any launch. Runs on the calling thread's current
 * device (devices 0 to 63, else DL_UNSUPPORTED), enqueued on `stream` (a cudaStream_t, NULL for
 * the legacy default stream).
 *
 * The blur's intermediate lives in one fixed device array of DL_NOALLOC_MAX_TEXELS * 12 bytes
 * (3 MiB) that every device loading the library holds until the process exits. The first call on
 * a device looks up that array's address (cudaGetSymbolAddress) and keeps it; make that call
 * before any stream capture. A process that calls cudaDeviceReset on a device must not call this
 * entry point on that device afterwards: the kept address belongs to the context the reset ended.
 * All calls share the array: calls whose work overlaps on the GPU (concurrent streams, threads)
 * race on it, so serialize them. */
#define DL_NOALLOC_MAX_TEXELS (512u * 512u)
dl_status dl_filter_bounce_window_noalloc(const float *in_rgb, float *out_rgb, uint32_t width, uint32_t height,
                                          uint32_t x0, uint32_t y0, uint32_t map_size, void *stream);

/* ---- Cache read bandwidth. No counterpart in the reference: a measurement helper for the
 * roofline of the traversal kernels, whose node and triangle reads are served by the L1 and L2
 * caches. Reads a zeroed buffer of `bytes` on `device` `passes` times per launch and stores the
 * best of five timed launches (after one warm-up) in *gbs, in 1e9 bytes per second. level 2:
 * every block streams the whole buffer with L1-bypassing loads (for a buffer that fits in L2,
 * the L2 read bandwidth); level 1: each block re-reads its own 32 KiB slice with cached loads
 * (the L1 read bandwidth). Allocates and frees its buffer; `bytes` from 1 MiB to 4 GiB. */
dl_status dl_probe_read_bandwidth(int device, uint32_t level, uint64_t bytes, uint32_t passes, double *gbs);

#ifdef __cplusplus
}
#endif

#endif /* DYNLIGHT_GB300_H */
