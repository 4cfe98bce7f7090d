/*
 * tpd_oracle.h — CPU oracle for the Gaussian-splatting hot path.
 *
 * TEST INFRASTRUCTURE ONLY. The product (libtpdsplat) never links, loads or
 * calls anything here; only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs use it, as the checker or as the timed
 * CPU baseline.
 *
 * What it restates (paths relative to the reference project root):
 *   - project.slang + splat/common.slang + splat/volume.slang  -> orc_preprocess_{f32,f64}
 *   - prefix.slang                                             -> orc_scan_tiles
 *   - keygen.slang                                             -> orc_keygen
 *   - radix-shuffle/prefixA/prefixB/mapping.slang              -> orc_radix4_sort
 *   - range.slang                                              -> orc_tile_ranges
 *   - blend.slang                                              -> orc_blend_{f32,f64}
 *   - (no reference)                                           -> orc_backward_f64
 *
 * Two arithmetic forms:
 *   f32: a transcription with the shaders' operation order: expressions are
 *        evaluated left to right as written, matrix products accumulate
 *        k = 0..n-1, no fused multiply-add (built with -ffp-contract=off).
 *   f64: the same maths in double, used for image / gradient error.
 *
 * Parity status: the reference's shader path (Slang -> SPIR-V -> Vulkan) cannot
 * be compiled or run on these machines, and the reference has no tests or
 * golden vectors. Shader maths is therefore "parity unpinned": it is pinned
 * only by hand-built known-answer cases and properties. The host-side inputs
 * (camera matrices, pass count) are pinned against the reference's own C++
 * compiled here (oracle/_ref, fixtures in tests/golden/).
 */
#pragma once
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 240-byte record, 60 floats: pos[0..2] opacity[3] quat[4..7]=(x,y,z,w)
 * scale[8..11]=(x,y,z,modifier) sh[12..59] (DC rgb, then channel-major rest).
 * GaussianGeometry.h:10-18, splat.slang:24-31. */
#define ORC_REC_FLOATS 60
/* 48-byte splat, 12 words: color[0..2] tiles[3](u32) px py viewZ radius conic[8..10] opacity[11].
 * splat.slang:33-39. */
#define ORC_SPLAT_WORDS 12

typedef struct orc_camera {
    float view[16];     /* row-major world->view */
    float projview[16]; /* row-major proj*view */
    float focal[2];     /* (P00, P11) */
    uint32_t width, height;
} orc_camera;

/* Preprocess, FP32 transcription. out: n*12 words. transforms: n_ent*16 floats
 * row-major; ent_idx may be NULL (all entity 0, identity if transforms NULL). */
void orc_preprocess_f32(const float* recs, uint32_t n, const uint32_t* ent_idx,
                        const float* transforms, const orc_camera* cam,
                        uint32_t sh_degree, int band3_compat, uint32_t* out);

/* Preprocess in FP64. out_splat: n*12 doubles (tiles as a double count).
 * out_rect: n*4 u32 (rmin.x rmin.y rmax.x rmax.y). fragile: n bytes, 1 when a
 * tile-rect / culling / radius decision lies within a small window of its
 * threshold (the "one ulp of a tile edge" set). */
void orc_preprocess_f64(const float* recs, uint32_t n, const uint32_t* ent_idx,
                        const float* transforms, const orc_camera* cam,
                        uint32_t sh_degree, int band3_compat, double* out_splat,
                        uint32_t* out_rect, uint8_t* fragile);

/* Exclusive scan of the tiles word of each splat into offsets[n]; returns the total. */
uint64_t orc_scan_tiles(const uint32_t* splats, uint32_t n, uint32_t* offsets);

/* Key duplication (keygen.slang:23-53). offsets from orc_scan_tiles. */
void orc_keygen(const uint32_t* splats, const uint32_t* offsets, uint32_t n,
                uint32_t width, uint32_t height, uint64_t* keys, uint32_t* vals);

/* Stable sort of (key, val) by the full 64-bit key (std::stable_sort). */
void orc_stable_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t k);

/* The reference's 4-way LSD radix sort on the low 2*passes bits, restated:
 * per pass a stable block-local split of 256-key blocks, a scan of per-block
 * digit counts and a digit-major scatter. threads<=0 -> OpenMP default. */
void orc_radix4_sort(uint64_t* keys, uint32_t* vals, uint64_t k, uint32_t passes, int threads);

/* getHigherMSB + updateRadixPassCount (GaussianEngine.h:234-245, GaussianEngine.cpp:351-357). */
uint32_t orc_higher_msb(uint32_t n);
uint32_t orc_radix_pass_count(uint32_t width, uint32_t height);

/* Tile ranges (range.slang:18-35), ranges zero-filled first. ranges: tiles*2 u32. */
void orc_tile_ranges(const uint64_t* keys, uint64_t k, uint32_t n_tiles, uint32_t* ranges);

/* Blend, FP32 transcription (blend.slang:24-105). image: h*w*3 floats.
 * final_T / n_contrib (may be NULL): per pixel transmittance and the number of
 * list entries processed up to and including the last contributor. */
void orc_blend_f32(const uint32_t* splats, const uint32_t* vals, const uint32_t* ranges,
                   uint32_t width, uint32_t height, float* image, float* final_T,
                   uint32_t* n_contrib, int threads);

/* The work measure of the blend: (pixel, list entry) pairs evaluated until
 * each pixel terminates, by the FP32 blend's rules (blend.slang:24-105: the
 * entry that would bring T below 1e-4 is evaluated and ends the pixel), and
 * the pairs that contribute colour. */
void orc_blend_pair_count(const uint32_t* splats, const uint32_t* vals, const uint32_t* ranges,
                          uint32_t width, uint32_t height, uint64_t* evaluated, uint64_t* contributing,
                          int threads);

/* Blend in FP64 over the same lists. splat64: n*12 doubles (orc_preprocess_f64).
 * fragile (may be NULL): 1 for pixels where an alpha / skip / termination
 * decision lies within a small window of its threshold. */
void orc_blend_f64(const double* splat64, const uint32_t* vals, const uint32_t* ranges,
                   uint32_t width, uint32_t height, double* image, double* final_T,
                   uint32_t* n_contrib, uint8_t* fragile);

/* Whole-frame FP32 transcription (preprocess -> scan -> keygen -> 4-way radix
 * sort -> ranges -> blend), the timed CPU baseline. Returns K (keys).
 * tile_rows_limit: render only the first tile rows of the image (0 = all). */
uint64_t orc_frame_f32(const float* recs, uint32_t n, const orc_camera* cam,
                       uint32_t sh_degree, float* image, int threads, uint32_t tile_rows_limit);

/* ---- inputs (tpd_oracle_host.cpp): seeded scenes and camera matrices ----
 * The camera maths of the reference (Camera::lookAt, PerspectiveCamera,
 * math::mul) with its accurate dot / cross arithmetic; the seeded synthetic
 * scene of the five workloads as 240-byte records. */
void orc_look_at(const float eye[3], const float center[3], const float up[3], float view[16]);
void orc_perspective(uint32_t width, uint32_t height, float fov_y_degrees, float near_plane, float far_plane,
                     float proj[16]);
void orc_mat4_mul(const float a[16], const float b[16], float out[16]);
void orc_synthetic_scene(uint64_t seed, uint32_t n, float mean_box, float* records);

/* ---- FP64 differentiable forward / backward over raw parameters ----
 * Raw parameters (double): means[n*3], log_scales[n*3], quats[n*4] (x,y,z,w,
 * used as stored, not normalised), opacity_logits[n], sh[n*48]; the scale
 * modifier is 1. Lists (vals/ranges) are fixed: the caller passes the GPU's. */
typedef struct orc_params64 {
    const double* means; const double* log_scales; const double* quats;
    const double* opacity_logits; const double* sh;
} orc_params64;

/* Forward in FP64 from raw parameters with fixed lists; image h*w*3. */
void orc_render_params_f64(const orc_params64* p, uint32_t n, const orc_camera* cam,
                           uint32_t sh_degree, int band3_compat, const uint32_t* vals,
                           const uint32_t* ranges, double* image);

/* Analytic FP64 gradient of sum(dL_dimage * image) w.r.t. the raw parameters.
 * grads: same shapes as orc_params64 (means, log_scales, quats, logits, sh).
 * g2d (may be NULL): n*9 doubles, dL/d(px, py, conic.x, conic.y, conic.z, opacity, r, g, b). */
void orc_backward_f64(const orc_params64* p, uint32_t n, const orc_camera* cam,
                      uint32_t sh_degree, int band3_compat, const uint32_t* vals,
                      const uint32_t* ranges, const double* dL_dimage,
                      double* g_means, double* g_log_scales, double* g_quats,
                      double* g_logits, double* g_sh, double* g2d);

#ifdef __cplusplus
}
#endif
