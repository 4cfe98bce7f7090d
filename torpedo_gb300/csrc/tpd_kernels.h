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
    uint32_t status;         // kStatus* bits, cleared at frame start
    uint32_t tag;            // launch tag, advanced once per frame / call
    uint32_t total_keys;     // K, written by the tile-count scan
    uint32_t visible;        // (view, Gaussian) pairs with a non-empty tile rect
    uint32_t ticket[32];     // partition tickets, cleared at frame start
    uint32_t sort_hist[8][256];   // digit counts of the key sort, by 8-bit digit position
    uint32_t depth_hist[8][256];  // digit counts of the depth sort, by 8-bit digit position
    uint32_t debug[4];       // site, index, bound of the first failed index guard
    uint32_t depth_count;    // (view, Gaussian) items with a non-empty tile rect: those the depth sort keeps
    // depth-sort passes skipped because their digit was the same for every
    // key (the order stays in the pass's input buffer): when odd, the later
    // passes swap their buffers and the sorted items are in the other one
    uint32_t depth_skips;
    uint32_t pad[2];
};

// Entity matrices: rows 0..2 of view*model and rows 0..3 of projview*model.
constexpr int kEntityMatFloats = 28;

// Ticket slots and look-back tag slots (tag = ctl->tag * 32 + slot).
constexpr int kTicketPreprocess = 0;
constexpr int kTicketScan = 1;
constexpr int kTicketBlend = 2;           // tile queue of a persistent blend launch
constexpr int kTicketBlendBackward = 3;   // tile queue of a persistent adjoint launch (reset by tile order)
constexpr int kTicketKeySortBase = 8;     // + 8-bit digit position
constexpr int kTicketDepthSortBase = 16;  // + 8-bit digit position
constexpr uint32_t kTagScan = 0;
constexpr uint32_t kTagKeySort = 1;       // + digit position
constexpr uint32_t kTagDepthSort = 16;    // + digit position

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
    // depth-sort input (nullptr: not written): item = v * n + i,
    // key = (v << 32) | bits(viewZ), or (v << 32) | 0xFFFFFFFF when culled
    uint64_t* depth_keys;
    uint32_t* depth_items;
    uint32_t depth_key_bits;  // 32 + bits of (n_views - 1); its digit histograms go to ctl->depth_hist
    // > 0: the 8-bit digit counts of the frame's tile ids (all keys the
    // visible items will emit, tile ids below 2^tile_bits) go to ctl->sort_hist[0..]
    uint32_t tile_bits;
    FrameCtl* ctl;
    // words set to zero after the kernel's dependency wait (nullptr: none):
    // the key sort's precounted rows, for keygen's counts
    uint32_t* zero_words;
    uint64_t zero_count;
};

constexpr uint32_t kMaxViews = 256;

// Kernel set-up that must happen once per device (a shared-memory opt-in, an
// occupancy query): calls init() the first time it is asked for on the
// current device and returns that result on every later call there.
// Thread-safe; keyed by (device, init).
int device_once(int (*init)());

// The test hook of the standalone scans (tpd_test_set_never_publish).
uint32_t test_never_publish_standalone();

// Clears tickets, histograms and status of ctl and advances its tag; computes
// entity matrices for n_views x n_ent (transforms nullptr -> identity).
void launch_frame_begin(FrameCtl* ctl, const float* transforms, uint32_t n_ent, const ViewConst* views,
                        uint32_t n_views, float* ent_mats, cudaStream_t s);
void launch_preprocess(const PreprocessArgs& a, int num_sms, cudaStream_t s);

// Standalone exclusive scan of Splat.tiles (prefix.slang); total -> ctl->total_keys.
void launch_scan_tiles(const Splat* splats, uint32_t n, uint32_t* offsets, uint64_t* desc, FrameCtl* ctl,
                       uint32_t spin_limit, uint32_t never_publish, cudaStream_t s);

// Items (view, Gaussian) in depth order per partition of the fused scan and
// key duplication: its look-back descriptors number n_items / kKeygenPart + 2.
constexpr uint32_t kKeygenPart = 512;

// The tile counts of the ctl->depth_count (view, Gaussian) items in depth
// order (items[r] = v * n + i < n_items) scanned into exclusive key offsets
// offsets[r] (prefix.slang), fused with keygen.slang's key duplication: keys
// (tile_base + tile) << 32 | bits(viewZ) with vals = Gaussian index. The
// items come in depth order, so only the tile id of each key is written
// (tiles[], u32): the depth half of a key is the depth of its value's splat
// (launch_materialize_keys). K goes to ctl->total_keys and the non-empty
// count to ctl->visible; keys beyond capacity are dropped and flag the frame
// (kStatusKeyOverflow). Also presets ranges (2 x n_tiles u32) to
// (0xFFFFFFFF, 0) for the key sort's last pass. The digit counts of the tile
// ids come from the preprocess (tile_bits).
// items: where the depth sort leaves the order with no pass skipped;
// items_other: the other buffer, which holds it when ctl->depth_skips is odd.
// desc: look-back descriptors (tag ctl->tag * 32 + kTagScan), never cleared.
// count_rows (or nullptr): the key sort's first counted pass's partition
// rows, zero on entry (PreprocessArgs.zero_words): each written key adds one
// to count_rows[256 * (slot / 4096) + (tile & 255)] (SortPlan.precounted).
void launch_keygen_scan(const Splat* splats, const uint32_t* items, const uint32_t* items_other, uint32_t n_items,
                        uint32_t n, const ViewConst* views, uint32_t* offsets, uint32_t* tiles, uint32_t* vals,
                        uint32_t capacity, uint32_t* ranges, uint32_t n_tiles, uint64_t* desc, uint32_t* count_rows,
                        FrameCtl* ctl, uint32_t spin_limit, uint32_t never_publish, int num_sms, cudaStream_t s);

// keys[i] = tiles[i] << 32 | bits(viewZ of splat vals[i] in the tile's view),
// i < min(ctl->total_keys, capacity): the 64-bit (tile | depth) keys of a
// frame, from its sorted tile ids and values (read-back only).
void launch_materialize_keys(const uint32_t* tiles, const uint32_t* vals, const Splat* splats, uint32_t n,
                             const uint32_t* tile_view, uint32_t n_tiles, uint32_t capacity, const FrameCtl* ctl,
                             uint64_t* keys, cudaStream_t s);

// Onesweep LSD radix sort of (key, val) pairs on key bits [first_bit, key_bits),
// first_bit a multiple of 8. K = min(ctl->total_keys, capacity). hist: the
// [8][256] digit counts by digit position (hist_ready: already filled, else a
// histogram kernel builds them); tickets ctl->ticket[ticket_base + position];
// look-back tags ctl->tag * 32 + tag_base + position. Result in (keys, vals)
// for an even pass count, else in (keys_alt, vals_alt); returns true for *_alt.
// desc: sort_desc_entries(capacity, items) descriptors (tagged, never cleared).
size_t sort_desc_entries(uint32_t capacity, uint32_t items = 16);
uint32_t sort_pass_count(uint32_t key_bits);
struct SortPlan {
    uint32_t first_bit = 0;
    uint32_t key_bits = 64;
    uint32_t (*hist)[256] = nullptr;
    bool hist_ready = false;
    uint32_t ticket_base = kTicketKeySortBase;
    uint32_t tag_base = kTagKeySort;
    int ctas_per_sm = 2;
    uint32_t items = 16;               // keys per thread: 16 (4096-key partitions), 8 or 4
    uint32_t threads = 256;            // 512: 4096-key partitions as 512 threads x 8 keys (items unused)
    uint32_t* ranges = nullptr;        // key sort: the last pass also writes the tile ranges (preset by keygen)
    uint32_t n_tiles = 0;
    uint32_t fixed_count = 0;          // nonzero: sort this many pairs, else min(ctl->total_keys, capacity)
    // a frame whose keys overflowed the capacity (its histograms count keys
    // that were not written) sorts nothing; it is rendered again
    bool skip_on_overflow = false;
    // depth sort: the first pass drops the keys whose low 32 bits are
    // 0xFFFFFFFF (culled items) and keeps ctl->depth_count, which the later
    // passes sort; a later pass whose digit is the same for every key copies
    bool compact_culled = false;
    cudaEvent_t after_hist = nullptr;  // recorded between the histogram and the first pass
    // non-null, 32-bit keys: counted passes (every partition's digit offsets
    // counted and scanned beforehand, no look-back; plain pass kinds only) using this work
    // area of sort_counted_work_words(capacity) u32, zero at rest (every
    // launch leaves it so)
    uint32_t* counted_work = nullptr;
    // counted passes: the first pass's partition rows (the first
    // 256 x ceil(capacity / 4096) words of counted_work) already hold every
    // 4096-key partition's digit counts, added by the kernel that wrote the
    // keys onto rows that were zero (launch_keygen_scan with count_rows); the
    // pass only scans them
    bool precounted = false;
};
size_t sort_counted_work_words(uint32_t capacity);
bool launch_sort(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, uint32_t capacity,
                 const SortPlan& plan, uint64_t* desc, FrameCtl* ctl, uint32_t spin_limit, int num_sms,
                 cudaStream_t s);
// The same for 32-bit keys (the frame's tile ids).
bool launch_sort(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t capacity,
                 const SortPlan& plan, uint64_t* desc, FrameCtl* ctl, uint32_t spin_limit, int num_sms,
                 cudaStream_t s);
// Clears status, histograms and tickets, sets total_keys and advances the tag
// (standalone stage calls).
void launch_sort_begin(FrameCtl* ctl, uint32_t total, cudaStream_t s);


struct BlendArgs {
    const Splat* splats;      // n_views x n (view-major)
    uint32_t n;               // Gaussians per view
    FrameCtl* ctl;            // K = min(ctl->total_keys, capacity); frames with a fatal status are skipped
    uint32_t capacity;
    const uint32_t* vals;
    uint32_t* ranges;         // 2 x n_tiles (global tile ids); an empty tile's (0xFFFFFFFF, 0) is rewritten to (0, 0)
    const ViewConst* views;   // device, n_views entries
    const uint32_t* tile_view;  // per global tile: view index (nullptr: single view 0)
    uint32_t n_tiles;
    float* image;             // HWC float3 per view, packed per view at image_offset[view]
    const uint64_t* image_offset;  // per view pixel offset (nullptr: 0)
    // per pixel: final transmittance and list entries up to the last
    // contributor (the adjoint's inputs); both null: not tracked
    float* final_T;
    uint32_t* n_contrib;
    // nullable: the image also as RGBA8 UNORM (alpha 255), packed like image
    // (launch_pack_rgba8's conversion), written with it
    uint32_t* rgba;
};
// Launch settings of the blend and its adjoint: list entries per staged
// round (forward 64 / 128 / 256, adjoint 32 / 64 / 128) and the form of the
// launch: one CTA per tile, or persistent CTAs (SMs x resident CTAs) taking
// (view, tile) items from a queue in FrameCtl. None of them changes a result.
struct BlendLaunch {
    uint32_t round = 128;
    uint32_t backward_round = 64;
    bool persistent = false;
    int num_sms = 148;
};
void launch_blend(const BlendArgs& a, const BlendLaunch& l, cudaStream_t s);

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
    float* g2d;               // n x kG2DStride (px, py, conic.xyz, opacity, rgb, 3 pad), accumulated
    uint64_t g2d_view_stride; // floats between views' g2d (n * kG2DStride)
    const uint32_t* tile_order;  // nullable: CTA b differentiates tile tile_order[b] (launch_tile_order)
};
void launch_blend_backward(const BlendBackwardArgs& a, const BlendLaunch& l, cudaStream_t s);

// order[0 .. n_tiles): the tiles by decreasing list length (in classes of
// equal floor(log2(length + 1)); any order within a class), so the longest
// lists start first and no SM is left with one at the end. ranges as the
// blend leaves them (empty tiles (0, 0)); lengths are clipped at
// min(ctl->total_keys, capacity). Also resets the adjoint's tile queue.
void launch_tile_order(const uint32_t* ranges, uint32_t n_tiles, FrameCtl* ctl, uint32_t capacity,
                       uint32_t* order, cudaStream_t s);

// Per-splat gradient record of the blend adjoint: 9 used floats padded to 12
// (48 B), so it is accumulated with three 16-byte vector atomics.
constexpr uint32_t kG2DStride = 12;

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
    const float* g2d;         // per view n x kG2DStride, view-major
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
