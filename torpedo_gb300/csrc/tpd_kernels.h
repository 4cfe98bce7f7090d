// tpd_kernels.h — host-side launch interface of the splatting kernels.
// Plain C++ (no CUDA syntax) so the engine and the C ABI can include it.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace tpd {

struct ViewConst;
struct Splat;

// Per-engine control block in device memory.
struct FrameCtl {
    uint32_t status;         // kStatus* bits, sticky until the host clears them
    uint32_t tag;            // launch tag, advanced once per frame / call
    uint32_t total_keys;     // K, written by the tile-count scan
    uint32_t visible;        // Gaussians with a non-empty tile rect
    uint32_t ticket[16];     // partition tickets, cleared at frame start
    uint32_t sort_hist[8][256];  // per-pass digit counts of the radix sort
    uint32_t debug[4];       // checked builds: site, index, bound of the first failed check
    uint32_t pad[8];
};

// Entity matrices: rows 0..2 of view*model and rows 0..3 of projview*model.
constexpr int kEntityMatFloats = 28;

// Ticket slots.
constexpr int kTicketPreprocess = 0;
constexpr int kTicketScan = 1;
constexpr int kTicketSortBase = 4;  // + pass (<= 8 passes)

struct PreprocessArgs {
    const float* recs;        // n x 60 floats (240-byte records)
    uint32_t n;
    const uint32_t* ent_idx;  // per-Gaussian entity index or nullptr (entity 0)
    const float* ent_mats;    // n_views x n_ent x kEntityMatFloats
    uint32_t n_ent;
    const ViewConst* views;   // device, n_views
    uint32_t n_views;         // <= kMaxViews
    uint32_t sh_degree;
    uint32_t band3_compat;
    Splat* splats;            // n_views x n (view-major)
    uint32_t* offsets;        // n_views x n, key offsets (fused scan); nullptr: no scan
    uint64_t* desc;           // look-back descriptors, ceil(n/128) entries
    FrameCtl* ctl;
    uint32_t spin_limit;
    uint32_t never_publish;   // test hook: partition 0 never publishes
};

constexpr uint32_t kMaxViews = 256;

// Clears tickets and sort histograms of ctl and advances its tag; computes
// entity matrices for n_views x n_ent (transforms nullptr -> identity).
void launch_frame_begin(FrameCtl* ctl, const float* transforms, uint32_t n_ent, const ViewConst* views,
                        uint32_t n_views, float* ent_mats, cudaStream_t s);
void launch_preprocess(const PreprocessArgs& a, cudaStream_t s);

// Standalone exclusive scan of Splat.tiles (prefix.slang); total -> ctl->total_keys.
void launch_scan_tiles(const Splat* splats, uint32_t n, uint32_t* offsets, uint64_t* desc, FrameCtl* ctl,
                       uint32_t spin_limit, uint32_t never_publish, cudaStream_t s);

// keygen.slang: keys = (tile_base + tile) << 32 | bits(viewZ), vals = Gaussian index,
// for n_views x n (view, Gaussian) items. K is read from ctl->total_keys; keys
// beyond capacity are dropped and flagged. Also accumulates the radix sort's
// digit histograms for key_bits into ctl->sort_hist (cleared at frame start).
void launch_keygen(const Splat* splats, const uint32_t* offsets, uint32_t n, const ViewConst* views,
                   uint32_t n_views, uint64_t* keys, uint32_t* vals, uint32_t capacity, uint32_t key_bits,
                   FrameCtl* ctl, int num_sms, cudaStream_t s);

// Onesweep LSD radix sort of (key, val) pairs on the low key_bits bits.
// K = min(ctl->total_keys, capacity). Result in (keys, vals) if the pass count
// is even, else in (keys_alt, vals_alt); returns true when it is in *_alt.
// desc: sort_desc_entries(capacity) descriptors.
size_t sort_desc_entries(uint32_t capacity);
uint32_t sort_pass_count(uint32_t key_bits);
// hist_ready: ctl->sort_hist already holds the digit histograms (keygen built
// them), so the histogram kernel is skipped. after_hist (nullable): event
// recorded between the histogram and the first pass.
bool launch_sort(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, uint32_t capacity,
                 uint32_t key_bits, uint64_t* desc, FrameCtl* ctl, uint32_t spin_limit, int num_sms,
                 cudaStream_t s, cudaEvent_t after_hist = nullptr, bool hist_ready = false, int ctas_per_sm = 2);
// Clears status, sort histograms and tickets, sets total_keys and advances the
// tag (standalone stage calls).
void launch_sort_begin(FrameCtl* ctl, uint32_t total, cudaStream_t s);

// range.slang: ranges[tile] = [start, end) over sorted keys, zero elsewhere.
void launch_tile_ranges(const uint64_t* keys, uint32_t n_tiles, uint32_t* ranges, FrameCtl* ctl, uint32_t capacity,
                        int num_sms, cudaStream_t s);

struct BlendArgs {
    const Splat* splats;      // n_views x n (view-major)
    uint32_t n;               // Gaussians per view
    FrameCtl* ctl;            // K = min(ctl->total_keys, capacity); frames with a fatal status are skipped
    uint32_t capacity;
    const uint32_t* vals;
    const uint32_t* ranges;   // 2 x n_tiles (global tile ids)
    const ViewConst* views;   // device, n_views entries
    const uint32_t* tile_view;  // per global tile: view index (nullptr: single view 0)
    uint32_t n_tiles;
    float* image;             // HWC float3 per view, packed per view at image_offset[view]
    const uint64_t* image_offset;  // per view pixel offset (nullptr: 0)
    float* final_T;           // per pixel (nullable)
    uint32_t* n_contrib;      // per pixel (nullable)
};
void launch_blend(const BlendArgs& a, cudaStream_t s);

// RGBA8 UNORM pack of an HWC float3 image (alpha 1), the reference's target format.
void launch_pack_rgba8(const float* rgb, uint32_t* rgba, size_t pixels, cudaStream_t s);

// ---- backward
struct BlendBackwardArgs {
    const Splat* splats;      // n_views x n (view-major)
    uint32_t n;               // Gaussians per view
    FrameCtl* ctl;
    uint32_t capacity;
    const uint32_t* vals;
    const uint32_t* ranges;
    const ViewConst* views;
    const uint32_t* tile_view;
    uint32_t n_tiles;
    const uint64_t* image_offset;
    const float* final_T;
    const uint32_t* n_contrib;
    const float* dL_dimage;   // HWC float3
    float* g2d;               // n x 9 (px, py, conic.xyz, opacity, rgb), accumulated
    uint32_t g2d_stride;      // floats between consecutive Gaussians' g2d (9) ...
    uint64_t g2d_view_stride; // ... and between views (batched: n*9; single: 0)
};
void launch_blend_backward(const BlendBackwardArgs& a, cudaStream_t s);

struct PreprocessBackwardArgs {
    const float* recs;
    uint32_t n;
    const uint32_t* ent_idx;
    const float* ent_mats;    // per view: n_ent x 28, view-major
    uint32_t n_ent;
    const ViewConst* views;   // device
    uint32_t n_views;
    uint32_t sh_degree;
    uint32_t band3_compat;
    const Splat* splats;      // per view n splats, view-major
    const float* g2d;         // per view n x 9, view-major
    float* g_means;           // n x 3
    float* g_log_scales;      // n x 3
    float* g_quats;           // n x 4
    float* g_logits;          // n
    float* g_sh;              // n x 48
};
void launch_preprocess_backward(const PreprocessBackwardArgs& a, cudaStream_t s);

// Raw parameters -> 240-byte records: opacity = sigmoid(logit), scale = exp(log_scale)
// with modifier 1, quaternion and SH copied as given.
void launch_pack_records(const float* means, const float* log_scales, const float* quats, const float* logits,
                         const float* sh, uint32_t n, float* recs, cudaStream_t s);

}  // namespace tpd
