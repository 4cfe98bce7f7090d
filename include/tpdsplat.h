/*
 * tpdsplat.h — C ABI of the GB300 Gaussian-splatting pipeline (libtpdsplat.so).
 *
 * Drop-in boundary for the reference renderer's Gaussian engine. Each entry
 * point names the reference interface it replaces (paths relative to the
 * reference project root, torpedo/):
 *
 *   tpd_create / tpd_destroy      Context<R>::bindEngine<GaussianEngine>()  rendering/include/torpedo/rendering/Context.h:192-239
 *                                 GaussianEngine::~GaussianEngine / destroy  volumetric/include/torpedo/volumetric/GaussianEngine.h:29
 *   tpd_settings                  GaussianEngine::Settings                  volumetric/include/torpedo/volumetric/GaussianEngine.h:17-21
 *   tpd_compile                   GaussianEngine::compile(scene, settings)  volumetric/src/GaussianEngine.cpp:359-399
 *   tpd_set_transform             TransformHost::transform(entity, mat4)    rendering/src/TransformHost.cpp:3-12
 *   tpd_set_camera                GaussianEngine::updateCameraBuffer        volumetric/src/GaussianEngine.cpp:764-775
 *   tpd_raster_frame              GaussianEngine::rasterFrame(camera)       volumetric/src/GaussianEngine.cpp:621-712
 *   tpd_read_image                GaussianEngine::draw(swapImage)           volumetric/src/GaussianEngine.cpp:714-762, 865-875
 *
 * Conventions: extern "C", plain pointers and sizes, int status codes (no
 * exceptions cross the ABI), one engine per host thread. Matrices are 16
 * floats, row-major, exactly as the reference's tpd::mat4 stores them.
 * Records are the reference's 240-byte GaussianPoint
 * (volumetric/include/torpedo/volumetric/GaussianGeometry.h:10-18):
 *   float position[3]; float opacity; float quaternion[4] (x,y,z,w);
 *   float scale[4] (x,y,z, w = modifier); float sh[48]
 * with opacity / scale already activated (sigmoid / exp), as fromModel() and
 * random() produce them.
 */
#ifndef TPDSPLAT_H
#define TPDSPLAT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TPD_ABI_VERSION 1

#if defined(__GNUC__)
#define TPD_API __attribute__((visibility("default")))
#else
#define TPD_API
#endif

typedef enum tpd_status {
    TPD_OK = 0,
    TPD_ERR_ARG = 1,       /* invalid argument (reference: std::runtime_error / early return) */
    TPD_ERR_OOM = 2,       /* device allocation failed */
    TPD_ERR_TIMEOUT = 3,   /* a bounded device wait or the host frame wait ran out */
    TPD_ERR_DEVICE = 4,    /* CUDA runtime error; see tpd_last_error */
    TPD_ERR_STATE = 5,     /* call out of order (e.g. render before compile) */
    TPD_ERR_CAPACITY = 6,  /* key capacity exceeded and could not grow */
    TPD_ERR_IO = 7         /* file could not be read or parsed */
} tpd_status;

/* Device status bits: tpd_frame_stats.status, and the status word that the
 * stage entry points leave in their scratch (see tpd_sort_pairs). 0 = clean. */
#define TPD_DEVSTAT_KEY_OVERFLOW 0x1u      /* more keys than the key buffers hold (the frame is rendered again) */
#define TPD_DEVSTAT_LOOKBACK_TIMEOUT 0x2u  /* a decoupled look-back wait ran out: prefixes and offsets are invalid */
#define TPD_DEVSTAT_BAD_INPUT 0x8u         /* an input outside its documented range */
#define TPD_DEVSTAT_BAD_INDEX 0x10u        /* an index failed its bounds check; the access was skipped */

typedef struct tpd_engine tpd_engine;

typedef struct tpd_settings {
    uint32_t sh_degree;            /* GaussianEngine::Settings::sphericalHarmonicsDegree, clamped to 3 */
    uint32_t band3_compat;         /* 1 (default): SH band-3 term exactly as splat/common.slang:69 writes it */
    int32_t device;                /* CUDA device ordinal (default 0) */
    void* stream;                  /* cudaStream_t to run on; NULL: the engine creates one */
    uint32_t use_graph;            /* 1 (default): frames replay a captured CUDA graph */
    uint32_t spin_limit;           /* look-back spin iterations before TPD_ERR_TIMEOUT (0: default) */
    uint64_t initial_key_capacity; /* 0: sized on the first frame */
    double timeout_s;              /* host wait limit per frame in seconds (0: 60) */
    uint32_t test_never_publish;   /* test hook: scan partition 0 never publishes (exercises the bounded spin) */
    uint32_t stage_timing;         /* 1: frames run without a graph and record CUDA events between stages */
    uint32_t sort_ctas_per_sm;     /* residency of the 256 x 16-key radix pass kernels: 2 (0 = default, no register spills) or 3;
                                      for the counted key sort 3 (0 = default) or 2 */
    uint32_t depth_sort_items;     /* keys per thread of the depth sort's 256-thread radix passes: 16 (0 = default), 8 or 4 */
    uint32_t sort_threads;         /* CTA size of the key sort's onesweep passes (key_sort_lookback = 1): 512 x 8 keys
                                      (0 = default) or 256 x 16; the counted passes run 256 x 16 */
    uint32_t depth_sort_threads;   /* CTA size of the depth sort's radix passes: 256 (0 = default) or 512 (8 keys each,
                                      whatever depth_sort_items says) */
    uint32_t blend_round;          /* list entries the blend stages per round: 128 (0 = default), 64 or 256 */
    uint32_t blend_backward_round; /* list entries the blend adjoint stages per round: 64 (0 = default), 32 or 128 */
    uint32_t blend_persistent;     /* 1: the blend and its adjoint run persistent CTAs taking (view, tile) items from a
                                      queue (the adjoint's longest lists first); 0 (default): one CTA per tile */
    uint32_t key_sort_lookback;    /* 0 (default): the key sort's radix passes count every partition's digits first and
                                      scatter without waiting (counted passes, 3 CTAs per SM, or 2 with
                                      sort_ctas_per_sm = 2); 1: onesweep passes with a decoupled look-back */
    uint32_t keep_backward_state;  /* whether frames keep the adjoint's inputs (per-pixel final transmittance and last
                                      contributor; tracking them costs the blend about 5%): 0 (default) once
                                      tpd_backward has been called on this engine; 1 always; 2 never. tpd_step_async
                                      always keeps them; tpd_backward and a read of TPD_BUF_FINAL_T /
                                      TPD_BUF_N_CONTRIB render the last frame again (its own views) when it kept none */
    uint32_t reserved[1];
} tpd_settings;

/* Stages of a frame (and of a training step), for tpd_stage_times. */
enum {
    TPD_STAGE_PREPROCESS = 0, /* camera upload, entity matrices, preprocess (splats + depth keys) */
    TPD_STAGE_DEPTH_SORT = 1, /* radix sort of the (view | depth) keys */
    TPD_STAGE_KEYGEN = 2,     /* tile-count scan and key duplication in depth order (one kernel) */
    TPD_STAGE_KEY_SORT = 3,   /* radix sort of the (tile | depth) keys on their tile-id bits */
    TPD_STAGE_RANGES = 4,     /* empty: the key sort's last pass writes the tile ranges */
    TPD_STAGE_BLEND = 5,      /* alpha blend */
    TPD_STAGE_BACKWARD_SETUP = 6,      /* tpd_step_async: gradient clear and the adjoint's tile order (0 in frames) */
    TPD_STAGE_BLEND_BACKWARD = 7,      /* tpd_step_async: blend adjoint (0 in frames) */
    TPD_STAGE_PREPROCESS_BACKWARD = 8, /* tpd_step_async: preprocess adjoint (0 in frames) */
    TPD_STAGE_COUNT = 9
};

typedef struct tpd_frame_stats {
    uint64_t keys;          /* duplicated (tile, Gaussian) keys, the reference's tilesRendered */
    uint64_t key_capacity;  /* current key buffer capacity */
    uint32_t visible;       /* (view, Gaussian) pairs with a non-empty tile rect */
    uint32_t tiles;         /* 16x16 tiles over all views */
    uint32_t key_bits;      /* low key bits sorted: getHigherMSB(tiles) + 32 */
    uint32_t sort_passes;   /* 8-bit radix passes */
    uint32_t status;        /* device status bits (0 = clean) */
    uint32_t retries;       /* frames re-run after growing the key buffers */
    uint32_t views;         /* views rendered */
    uint32_t reserved[5];
} tpd_frame_stats;

/* One camera for the batched form: view and projection as Camera /
 * PerspectiveCamera hold them (rendering/include/torpedo/rendering/Camera.h:42-47). */
typedef struct tpd_view {
    float view[16];
    float proj[16];
    uint32_t width, height;
} tpd_view;

enum {
    TPD_IMAGE_RGB32F = 0, /* H x W x 3 floats, no background (blend.slang:104 stores (C, 1)) */
    TPD_IMAGE_RGBA8 = 1   /* H x W RGBA8 UNORM, alpha 255: the reference's target format (GaussianEngine.cpp:318) */
};

enum {
    TPD_BUF_RECORDS = 0,   /* n x 240 B */
    TPD_BUF_SPLATS = 1,    /* views x n x 48 B (splat.slang:33-39) */
    TPD_BUF_OFFSETS = 2,   /* views x n u32: exclusive scan of tile counts */
    TPD_BUF_KEYS = 3,      /* keys u64 (tile << 32 | depth bits), sorted after a frame; rebuilt from the
                              sorted tile ids and values when asked for (waits for the stream) */
    TPD_BUF_VALUES = 4,    /* Gaussian index u32, in sorted order after a frame */
    TPD_BUF_RANGES = 5,    /* tiles x 2 u32 */
    TPD_BUF_IMAGE = 6,     /* pixels x 3 floats, views packed */
    TPD_BUF_FINAL_T = 7,   /* pixels floats */
    TPD_BUF_N_CONTRIB = 8, /* pixels u32 */
    TPD_BUF_G2D = 9        /* views x n x 12 floats after tpd_backward: px, py, conic xyz, opacity, rgb, 3 pad */
};

TPD_API const char* tpd_version(void);
TPD_API const char* tpd_status_string(int status);
TPD_API void tpd_settings_init(tpd_settings* s);

TPD_API int tpd_create(const tpd_settings* s, tpd_engine** out);
TPD_API void tpd_destroy(tpd_engine* e);
TPD_API const char* tpd_last_error(const tpd_engine* e);

/* Uploads n records (host memory). entity_index (nullable): per-record entity,
 * < n_entities; NULL = all entity 0. Model matrices start as identity.
 * Replaces compile(); the caller's buffers can be freed afterwards. n == 0 is
 * accepted and renders an empty image (the reference warns and returns). */
TPD_API int tpd_compile(tpd_engine* e, const void* records, uint32_t n, const uint32_t* entity_index, uint32_t n_entities);

/* Training form: builds the records on the device from raw device parameters
 * (means n x 3, log_scales n x 3, quats n x 4 used as given, opacity_logits n,
 * sh n x 48): opacity = sigmoid(logit), scale = exp(log_scale), modifier 1. */
TPD_API int tpd_compile_params_device(tpd_engine* e, const float* means, const float* log_scales, const float* quats,
                              const float* opacity_logits, const float* sh, uint32_t n);

TPD_API int tpd_set_transform(tpd_engine* e, uint32_t entity, const float model[16]);

/* view: world->view; proj: the camera's projection (PerspectiveCamera). The
 * engine uploads view, proj*view and (proj[0], proj[5]) like updateCameraBuffer. */
TPD_API int tpd_set_camera(tpd_engine* e, const float view[16], const float proj[16], uint32_t width, uint32_t height);

/* Batched form: up to 256 views of any sizes rendered in one frame. */
TPD_API int tpd_set_views(tpd_engine* e, const tpd_view* views, uint32_t n_views);

/* Renders the current view(s). Synchronous with the host, like rasterFrame. */
TPD_API int tpd_raster_frame(tpd_engine* e, tpd_frame_stats* stats);

/* Enqueues count frames of the current view(s) back to back without waiting
 * (a frame must have been rendered by tpd_raster_frame since the last change,
 * so the key capacity is known). tpd_sync waits for them and reports the last
 * frame's stats; TPD_ERR_CAPACITY means the keys outgrew the buffers and the
 * frames must be re-rendered with tpd_raster_frame. */
TPD_API int tpd_raster_frames_async(tpd_engine* e, uint32_t count);
TPD_API int tpd_sync(tpd_engine* e, tpd_frame_stats* stats);

/* Pipelined rendering, no counterpart in the reference (its rasterFrame waits):
 * tpd_render_async renders the current view(s) and copies the image (format
 * TPD_IMAGE_*) to dst without waiting; the copy runs on a second stream beside
 * the next frame. The camera constants and transforms are taken when the call
 * is made, so tpd_set_camera may be called again at once. At most two renders
 * may be outstanding; tpd_wait_render waits for the oldest, fills its stats and
 * returns its status (TPD_ERR_CAPACITY: keys outgrew the buffers, render with
 * tpd_raster_frame). dst must stay valid and unread until then. Needs a frame
 * rendered with tpd_raster_frame after any change. */
TPD_API int tpd_render_async(tpd_engine* e, void* dst, uint32_t format, int dst_is_device);
TPD_API int tpd_wait_render(tpd_engine* e, tpd_frame_stats* stats);

/* Accumulated per-stage GPU time (ms, TPD_STAGE_COUNT entries) and frame count
 * since the last reset, when the engine was created with stage_timing = 1. */
TPD_API int tpd_stage_times(tpd_engine* e, double* ms, uint64_t* frames, int reset);

/* Copies the rendered image(s) of all views, packed view after view. */
TPD_API int tpd_read_image(tpd_engine* e, void* dst, uint32_t format, int dst_is_device);

/* Gradients of sum(dL_dimage * image) of the last frame (device pointers,
 * same packing as the image) w.r.t. raw parameters (device, shapes as in
 * tpd_compile_params_device). g2d (nullable) receives nothing; read it with
 * tpd_get_buffer(TPD_BUF_G2D). Any output pointer may be NULL. */
TPD_API int tpd_backward(tpd_engine* e, const float* dL_dimage, float* g_means, float* g_log_scales, float* g_quats,
                 float* g_logits, float* g_sh);

/* Training step, no counterpart in the reference (it has no backward): count
 * times forward frame + backward on the current views, enqueued without host
 * waits; with use_graph both are one captured CUDA graph per step (captured
 * again when the pointers change). Gradients are overwritten each step.
 * Needs a frame rendered with tpd_raster_frame after any change (it sizes the
 * key buffers); tpd_sync then reports TPD_ERR_CAPACITY if the keys outgrew
 * them. */
TPD_API int tpd_step_async(tpd_engine* e, const float* dL_dimage, float* g_means, float* g_log_scales, float* g_quats,
                   float* g_logits, float* g_sh, uint32_t count);

TPD_API int tpd_get_buffer(const tpd_engine* e, uint32_t which, void** device_ptr, uint64_t* bytes);
/* Copies bytes [offset, offset + bytes) of an internal buffer (TPD_BUF_*) to dst. */
TPD_API int tpd_read_buffer(tpd_engine* e, uint32_t which, void* dst, uint64_t offset, uint64_t bytes,
                            int dst_is_device);
TPD_API void* tpd_get_stream(const tpd_engine* e);

/* ---- stage entry points on caller device memory (stream may be NULL) ---- */

/* Number of low key bits the reference sorts for a tile count:
 * getHigherMSB(tiles) + 32 (GaussianEngine.h:234-245, GaussianEngine.cpp:351-357). */
TPD_API uint32_t tpd_key_bits_for_tiles(uint32_t tiles);

/* Radix sort (radix-shuffle / prefixA / prefixB / mapping .slang): stable
 * sort of n (key, value) pairs on the low key_bits bits. Result in keys/vals
 * if *result_in_alt == 0, else in keys_alt/vals_alt. workspace: at least
 * tpd_sort_workspace_size(n) bytes of device memory, 16-byte aligned.
 * The call enqueues its work on the stream and returns; once that work is
 * done, the uint32 at byte offset TPD_WORKSPACE_STATUS_OFFSET of the
 * workspace holds the device status (TPD_DEVSTAT_* bits): anything but 0
 * means the result is invalid. */
#define TPD_WORKSPACE_STATUS_OFFSET 0
TPD_API size_t tpd_sort_workspace_size(uint32_t n);
TPD_API int tpd_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                   uint32_t key_bits, void* workspace, size_t workspace_bytes, void* stream, int* result_in_alt);

/* prefix.slang: exclusive scan of the tiles word of n 48-byte splats into
 * offsets (u32), total into *total (device u32). workspace: at least
 * tpd_scan_workspace_size(n) bytes of device memory, 16-byte aligned; its
 * status word (TPD_WORKSPACE_STATUS_OFFSET) as for tpd_sort_pairs. */
TPD_API size_t tpd_scan_workspace_size(uint32_t n);
TPD_API int tpd_scan_tiles(const void* splats, uint32_t n, uint32_t* offsets, uint32_t* total, void* workspace,
                   size_t workspace_bytes, void* stream);

/* No counterpart in the reference: tpd_scan_tiles without a workspace. The
 * scratch is a fixed array in this library's device memory, so the call
 * allocates nothing; it is for callers that cannot hand out device memory
 * when they scan (all of it held by their own arena or caching allocator) or
 * must not call cudaMalloc/cudaFree in a per-frame loop, since either can
 * wait for the whole device. n above TPD_SCAN_STATIC_MAX_SPLATS returns
 * TPD_ERR_CAPACITY. The first call on each device (that device current) sets
 * up the scratch's address and should come before any stream capture. One
 * scratch per device: calls whose work overlaps on one device race, so order
 * them on one stream. Each call clears its scratch first; nothing has to
 * start at zero. The scratch address is looked up once per device in the
 * device's primary context (the runtime's default): do not call it from
 * another driver context, nor after cudaDeviceReset in the same process.
 * status (nullable, device u32) receives the scan's device status
 * (TPD_DEVSTAT_* bits) on the stream: anything but 0 means offsets and total
 * are invalid. */
#define TPD_SCAN_STATIC_MAX_SPLATS (1u << 24)
TPD_API int tpd_scan_tiles_static(const void* splats, uint32_t n, uint32_t* offsets, uint32_t* total,
                                  uint32_t* status, void* stream);

/* Test hook: nonzero makes partition 0 of every later tpd_scan_tiles /
 * tpd_scan_tiles_static call never publish its look-back descriptor, so the
 * bounded wait of partition 1 runs out and the call's status reports it. */
TPD_API void tpd_test_set_never_publish(uint32_t on);

/* ---- host utilities (no device) ---- */

/* Camera::lookAt (rendering/src/Camera.cpp:3-16) with the reference's
 * compensated dot / difference-of-products arithmetic. */
TPD_API void tpd_look_at(const float eye[3], const float center[3], const float up[3], float view_out[16]);
/* PerspectiveCamera projection (extension/src/PerspectiveCamera.cpp:9-23):
 * fy = 1 / tan(fov_y/2) (fov_y_degrees <= 0: fy = sqrt(3)), fx = fy / aspect,
 * reversed-Z [near, far] -> [1, 0]. */
TPD_API void tpd_perspective(uint32_t width, uint32_t height, float fov_y_degrees, float near_plane, float far_plane,
                     float proj_out[16]);
/* math::mul(proj, view) with the reference's compensated dot (mat4.h:256-264). */
TPD_API void tpd_mat4_mul(const float a[16], const float b[16], float out[16]);

/* Seeded synthetic scene (mt19937_64, seed as given; normals drawn in double):
 * means ~ N(0,1)^3 (mean_box <= 0) or U[-mean_box, mean_box]^3; log-scales ~
 * N(-4, 0.5); quaternion = normalize(N(0,1)^4) as (x,y,z,w); opacity logit ~
 * N(0,1); sh ~ N(0, 0.2). Writes raw parameters (any pointer may be NULL) and
 * the activated 240-byte records (nullable). */
TPD_API void tpd_synthetic_scene(uint64_t seed, uint32_t n, float mean_box, float* means, float* log_scales, float* quats,
                         float* opacity_logits, float* sh, void* records);

/* GaussianPoint::random (volumetric/src/GaussianGeometry.cpp:8-32), seeded. */
TPD_API void tpd_random_points(uint64_t seed, uint32_t n, float radius, const float center[3], float min_scale,
                       float max_scale, float min_opacity, float max_opacity, void* records);

/* GaussianPoint::fromModel (volumetric/src/GaussianGeometry.cpp:59-127): reads
 * a 3DGS PLY (binary little-endian or ASCII). Call with records == NULL to get
 * the count in *n_out, then again with room for *n_out records. */
TPD_API int tpd_load_ply(const char* path, void* records, uint32_t* n_out);

#ifdef __cplusplus
}
#endif

#endif /* TPDSPLAT_H */
