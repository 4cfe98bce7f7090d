// engine.cu — the C ABI (include/tpdsplat.h): engine state, buffers and the
// per-frame schedule.
//
// Reference: GaussianEngine (volumetric/src/GaussianEngine.cpp). Differences
// by design:
//  - The reference reads tilesRendered back to the host in the middle of every
//    frame (GaussianEngine.cpp:665-674) to size its key buffers. Here every
//    kernel after the scan reads K from device memory and the key buffers have
//    a capacity: keygen drops keys past it and raises a status bit, the key
//    sort and the blend then do nothing, and the host grows the buffers and
//    re-runs the frame. A frame therefore has no host round trip and is
//    replayed as one CUDA graph.
//  - One stream, no queue-ownership transfers; images stay in device memory
//    until tpd_read_image (the reference copies into a swapchain image).
//  - Host waits poll an event with a time limit (the reference waits on
//    fences with UINT64_MAX, GaussianEngine.cpp:634, 665).
//  - V >= 1 views per frame; V = 1 reproduces the reference's keys exactly
//    (tile ids without offset).
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/tpdsplat.h"
#include "tpd_common.cuh"
#include "tpd_kernels.h"

using namespace tpd;

namespace tpd {

int device_once(int (*init)()) {
    static std::mutex m;
    static std::map<std::pair<int, uintptr_t>, int> done;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_pair(dev, reinterpret_cast<uintptr_t>(init));
    std::lock_guard<std::mutex> lock(m);
    const auto it = done.find(key);
    if (it != done.end()) return it->second;
    const int v = init();
    done.emplace(key, v);
    return v;
}

namespace {
std::atomic<uint32_t> g_never_publish_standalone{0};
}
uint32_t test_never_publish_standalone() { return g_never_publish_standalone.load(); }

}  // namespace tpd

namespace {

constexpr uint32_t kDefaultSpin = 1u << 20;
// Look-back descriptors keep 30 bits of (frame tag * 32 + slot), so a tag
// value comes round again after 2^25 frames; the engine clears its
// descriptors whenever the frame tag reaches a multiple of this, and a stale
// descriptor can then never carry the current frame's tag.
constexpr uint64_t kTagWindow = 1ull << 25;
constexpr uint32_t kScanTileStandalone = 1024;

struct StatsHead {
    uint32_t status, tag, total_keys, visible;
};

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

}  // namespace

struct tpd_engine {
    tpd_settings settings{};
    int device = 0;
    int num_sms = 148;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string last_error;
    cudaEvent_t done_event = nullptr;

    // scene
    uint32_t n = 0;
    uint32_t n_ent = 1;
    bool compiled = false;
    float* d_recs = nullptr;
    uint32_t* d_ent_idx = nullptr;
    float* h_transforms = nullptr;  // pinned, n_ent x 16
    float* d_transforms = nullptr;
    bool identity_transforms = true;

    // views
    uint32_t n_views = 0;
    ViewConst* h_views = nullptr;  // pinned, kMaxViews
    ViewConst* d_views = nullptr;
    std::vector<uint32_t> vw, vh;
    uint32_t total_tiles = 0;
    uint64_t total_pixels = 0;
    uint32_t* d_tile_view = nullptr;
    uint32_t* d_tile_order = nullptr;  // tiles by decreasing list length, for the blend adjoint
    uint64_t* d_image_offset = nullptr;

    // frame buffers
    uint64_t splat_cap = 0;  // entries of splats / offsets / depth keys (views x n)
    Splat* d_splats = nullptr;
    uint32_t* d_offsets = nullptr;  // key offsets of the items in depth order
    uint64_t* d_dkeys[2] = {nullptr, nullptr};
    uint32_t* d_ditems[2] = {nullptr, nullptr};
    uint64_t* d_desc_depth = nullptr;
    uint32_t depth_key_bits = 32;
    bool depth_in_alt = false;
    uint64_t* d_desc_pre = nullptr;
    uint64_t desc_pre_cap = 0;
    float* d_ent_mats = nullptr;
    uint64_t ent_mats_cap = 0;
    uint64_t capacity = 0;
    uint32_t* d_tiles[2] = {nullptr, nullptr};  // the frame's keys as tile ids (depth order fixed by the presort)
    uint64_t* d_keys64 = nullptr;               // (tile | depth) keys rebuilt for read-back, on demand
    uint64_t keys64_cap = 0;
    uint32_t* d_vals[2] = {nullptr, nullptr};
    uint64_t* d_desc_sort = nullptr;
    uint32_t* d_sort_work = nullptr;  // counted key-sort passes: partition counts and offsets (zero at rest)
    uint32_t* d_ranges = nullptr;
    uint64_t pixel_cap = 0, tile_cap = 0;
    float* d_image = nullptr;
    float* d_final_T = nullptr;
    uint32_t* d_n_contrib = nullptr;
    uint32_t* d_rgba = nullptr;
    float* d_g2d = nullptr;
    uint64_t g2d_cap = 0;
    float* d_gscratch = nullptr;
    uint64_t gscratch_cap = 0;
    FrameCtl* d_ctl = nullptr;
    StatsHead* h_stats = nullptr;  // pinned

    uint32_t key_bits = 0, passes = 0;
    bool sorted_in_alt = false;
    bool frame_valid = false;

    // stage timing: a ring of event sets, harvested at synchronisation points
    static constexpr int kTimingSlots = 64;
    static constexpr int kTimingEvents = TPD_STAGE_COUNT + 1;
    cudaEvent_t tev[kTimingSlots][kTimingEvents] = {};
    bool tev_pending[kTimingSlots] = {};
    int tslot = 0;
    int cur_tslot = -1;  // the slot of the last enqueued frame (its backward stages are recorded there)
    double stage_ms[TPD_STAGE_COUNT] = {};
    uint64_t timed_frames = 0;

    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    bool graph_state = false;      // the frame graph keeps the adjoint's inputs
    bool state_kept = false;       // the last frame kept them (final T, last contributor)
    bool backward_seen = false;    // tpd_backward has been called on this engine
    bool needs_eager = true;  // the first frame after any change runs without a graph
    uint64_t frames = 0;
    uint64_t tags = 0;  // frame tags issued so far (FrameCtl.tag of the last enqueued frame)

    // forward + backward step graph (tpd_step_async), keyed by the caller's pointers
    cudaGraphExec_t step_graph = nullptr;
    const void* step_key[6] = {};

    // pipelined renders (tpd_render_async / tpd_wait_render): a ring of slots,
    // each with its own pinned copy of the frame's constants and stats, a
    // device staging image and completion events; the image copy to the
    // caller runs on copy_stream, so the next frame computes meanwhile
    static constexpr int kRing = 2;
    // per slot and image format (RGBA8, RGB32F): the slot's upload of the
    // view constants (and transforms), the frame, its image into the slot's
    // staging buffer (the blend writes RGBA8 itself) and the stats copy
    cudaGraphExec_t slot_graph[kRing][2] = {};
    bool slot_graph_state[kRing][2] = {};  // captured keeping the adjoint's inputs
    bool slot_graph_ident[kRing][2] = {};  // captured without transforms
    cudaStream_t copy_stream = nullptr;
    ViewConst* ring_views[kRing] = {};
    float* ring_transforms[kRing] = {};
    uint32_t ring_transforms_cap = 0;
    StatsHead* ring_stats[kRing] = {};
    unsigned char* ring_image[kRing] = {};
    uint64_t ring_image_cap = 0;
    cudaEvent_t ring_ready[kRing] = {};  // main stream: frame, staging image and stats done
    cudaEvent_t ring_done[kRing] = {};   // copy stream: the caller's image written
    bool ring_busy[kRing] = {};
    uint64_t ring_next = 0, ring_oldest = 0;
};

namespace {

int fail(tpd_engine* e, int code, const std::string& msg) {
    if (e) e->last_error = msg;
    return code;
}

#define TPD_CUDA(e, call)                                                                                  \
    do {                                                                                                   \
        cudaError_t _err = (call);                                                                         \
        if (_err != cudaSuccess) {                                                                         \
            return fail((e), _err == cudaErrorMemoryAllocation ? TPD_ERR_OOM : TPD_ERR_DEVICE,             \
                        std::string(#call) + ": " + cudaGetErrorString(_err));                             \
        }                                                                                                  \
    } while (0)

template <typename T>
cudaError_t dalloc(T*& p, uint64_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
}

void invalidate_step_graph(tpd_engine* e) {
    if (e->step_graph) cudaGraphExecDestroy(e->step_graph);
    e->step_graph = nullptr;
    for (auto& k : e->step_key) k = nullptr;
}

void invalidate_slot_graphs(tpd_engine* e) {
    for (auto& row : e->slot_graph)
        for (auto& g : row) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

void invalidate_graph(tpd_engine* e) {
    if (e->graph) cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
    e->graph_valid = false;
    e->needs_eager = true;
    invalidate_step_graph(e);
    invalidate_slot_graphs(e);
}

// Views x n sized buffers.
int ensure_splat_buffers(tpd_engine* e) {
    const uint64_t need = uint64_t(e->n) * e->n_views;
    if (need > e->splat_cap) {
        invalidate_graph(e);
        TPD_CUDA(e, dalloc(e->d_splats, need));
        TPD_CUDA(e, dalloc(e->d_offsets, need));
        for (int b = 0; b < 2; ++b) {
            TPD_CUDA(e, dalloc(e->d_dkeys[b], need));
            TPD_CUDA(e, dalloc(e->d_ditems[b], need));
        }
        const size_t de = sort_desc_entries(uint32_t(need), 4);  // room for the smallest partitions
        TPD_CUDA(e, dalloc(e->d_desc_depth, de));
        TPD_CUDA(e, cudaMemset(e->d_desc_depth, 0, de * 8));
        e->splat_cap = need;
    }
    const uint64_t parts = need / std::min(kScanTileStandalone, kKeygenPart) + 2;  // the frame's scan partitions
    if (parts > e->desc_pre_cap) {
        invalidate_graph(e);
        TPD_CUDA(e, dalloc(e->d_desc_pre, parts));
        TPD_CUDA(e, cudaMemset(e->d_desc_pre, 0, parts * 8));
        e->desc_pre_cap = parts;
    }
    const uint64_t em = uint64_t(e->n_ent) * e->n_views * kEntityMatFloats;
    if (em > e->ent_mats_cap) {
        invalidate_graph(e);
        TPD_CUDA(e, dalloc(e->d_ent_mats, em));
        e->ent_mats_cap = em;
    }
    return TPD_OK;
}

int ensure_key_capacity(tpd_engine* e, uint64_t want) {
    if (want <= e->capacity) return TPD_OK;
    if (want > 0x7FFFFFFFull) return fail(e, TPD_ERR_CAPACITY, "key count exceeds 2^31-1");
    invalidate_graph(e);
    for (int b = 0; b < 2; ++b) {
        TPD_CUDA(e, dalloc(e->d_tiles[b], want));
        TPD_CUDA(e, dalloc(e->d_vals[b], want));
    }
    const size_t entries = sort_desc_entries(uint32_t(want));
    TPD_CUDA(e, dalloc(e->d_desc_sort, entries));
    TPD_CUDA(e, cudaMemset(e->d_desc_sort, 0, entries * 8));
    const size_t words = sort_counted_work_words(uint32_t(want));
    TPD_CUDA(e, dalloc(e->d_sort_work, words));
    TPD_CUDA(e, cudaMemset(e->d_sort_work, 0, words * 4));
    e->capacity = want;
    return TPD_OK;
}

int wait_event(tpd_engine* e, cudaEvent_t ev);

int wait_stream(tpd_engine* e) {
    TPD_CUDA(e, cudaEventRecord(e->done_event, e->stream));
    return wait_event(e, e->done_event);
}

// Polls ev with the engine's host wait limit.
int wait_event(tpd_engine* e, cudaEvent_t ev) {
    const double limit = e->settings.timeout_s > 0 ? e->settings.timeout_s : 60.0;
    const auto t0 = std::chrono::steady_clock::now();
    while (true) {
        const cudaError_t q = cudaEventQuery(ev);
        if (q == cudaSuccess) return TPD_OK;
        if (q != cudaErrorNotReady)
            return fail(e, TPD_ERR_DEVICE, std::string("frame: ") + cudaGetErrorString(q) +
                                               (e->last_error.rfind("stage", 0) == 0 ? " (" + e->last_error + ")" : ""));
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (dt > limit) return fail(e, TPD_ERR_TIMEOUT, "frame did not finish within the host wait limit");
        // frames take about a millisecond: poll without sleeping at first (a
        // sleep of a few microseconds lasts tens on Linux), then back off
        if (dt < 0.005)
            std::this_thread::yield();
        else
            std::this_thread::sleep_for(std::chrono::microseconds(dt < 0.05 ? 50 : 500));
    }
}

void harvest_slot(tpd_engine* e, int slot) {
    if (!e->tev_pending[slot]) return;
    cudaEventSynchronize(e->tev[slot][tpd_engine::kTimingEvents - 1]);
    for (int k = 0; k < TPD_STAGE_COUNT; ++k) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e->tev[slot][k], e->tev[slot][k + 1]) == cudaSuccess) e->stage_ms[k] += ms;
    }
    e->timed_frames++;
    e->tev_pending[slot] = false;
}

void harvest_all(tpd_engine* e) {
    for (int i = 0; i < tpd_engine::kTimingSlots; ++i) harvest_slot(e, i);
}

// The blend's launch settings (tpd_settings: round sizes and the persistent form).
BlendLaunch blend_launch(const tpd_engine* e) {
    BlendLaunch l;
    l.round = e->settings.blend_round == 64 || e->settings.blend_round == 256 ? e->settings.blend_round : 128;
    l.backward_round = e->settings.blend_backward_round == 32 || e->settings.blend_backward_round == 128
                           ? e->settings.blend_backward_round
                           : 64;
    l.persistent = e->settings.blend_persistent != 0;
    l.num_sms = e->num_sms;
    return l;
}

// Enqueues one frame on the stream (no host synchronisation).
// io = false leaves out the uploads of the view constants and transforms and
// the stats copy (the pipelined renders enqueue those per slot).
// state: the blend also keeps the adjoint's inputs (final T, last contributor);
// rgba: non-null, the blend also writes the image there as RGBA8.
void enqueue_frame(tpd_engine* e, bool io = true, bool state = true, uint32_t* rgba = nullptr) {
    cudaStream_t s = e->stream;
    cudaEvent_t* ev = nullptr;
    if (e->settings.stage_timing) {
        const int slot = e->tslot;
        e->tslot = (e->tslot + 1) % tpd_engine::kTimingSlots;
        harvest_slot(e, slot);
        if (!e->tev[slot][0])
            for (int k = 0; k < tpd_engine::kTimingEvents; ++k) cudaEventCreate(&e->tev[slot][k]);
        ev = e->tev[slot];
        e->tev_pending[slot] = true;
        e->cur_tslot = slot;
    }
    // TPD_DEBUG_SYNC=1 (eager frames only): synchronise after each stage and
    // name the first stage whose kernels report an error.
    static const bool debug_sync = [] {
        const char* v = std::getenv("TPD_DEBUG_SYNC");
        return v && v[0] == '1';
    }();
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap_status);
    static const char* kStageNames[] = {"begin", "preprocess", "depth sort", "keygen", "key sort", "ranges", "blend",
                                        "backward set-up", "blend adjoint", "preprocess adjoint"};
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], s);
        if (debug_sync && cap_status == cudaStreamCaptureStatusNone) {
            const cudaError_t err = cudaStreamSynchronize(s);
            if (err != cudaSuccess && e->last_error.rfind("stage", 0) != 0)
                e->last_error = std::string("stage ") + kStageNames[k] + ": " + cudaGetErrorString(err);
        }
    };
    mark(0);
    if (io) {
        cudaMemcpyAsync(e->d_views, e->h_views, sizeof(ViewConst) * e->n_views, cudaMemcpyHostToDevice, s);
        if (!e->identity_transforms)
            cudaMemcpyAsync(e->d_transforms, e->h_transforms, sizeof(float) * 16 * e->n_ent, cudaMemcpyHostToDevice,
                            s);
    }
    launch_frame_begin(e->d_ctl, e->identity_transforms ? nullptr : e->d_transforms, e->n_ent, e->d_views,
                       e->n_views, e->d_ent_mats, s);
    PreprocessArgs pa{};
    pa.recs = e->d_recs;
    pa.n = e->n;
    pa.ent_idx = e->d_ent_idx;
    pa.ent_mats = e->d_ent_mats;
    pa.n_ent = e->n_ent;
    pa.views = e->d_views;
    pa.n_views = e->n_views;
    pa.sh_degree = e->settings.sh_degree;
    pa.band3_compat = e->settings.band3_compat;
    pa.splats = e->d_splats;
    pa.depth_keys = e->d_dkeys[0];
    pa.depth_items = e->d_ditems[0];
    pa.depth_key_bits = e->depth_key_bits;
    pa.tile_bits = e->key_bits - 32;  // the key sort's digit counts
    pa.ctl = e->d_ctl;
    // counted key-sort passes (default): keygen counts the first pass's
    // partition rows, which the preprocess clears
    const bool counted = e->settings.key_sort_lookback == 0;
    const uint32_t key_parts = std::max(1u, uint32_t((e->capacity + 4095u) / 4096u));
    pa.zero_words = counted ? e->d_sort_work : nullptr;
    pa.zero_count = counted ? uint64_t(key_parts) * 256u : 0u;
    launch_preprocess(pa, e->num_sms, s);
    mark(1);
    const uint32_t spin = e->settings.spin_limit ? e->settings.spin_limit : kDefaultSpin;
    const uint32_t items = e->n * e->n_views;
    SortPlan dp;
    dp.first_bit = 0;
    dp.key_bits = e->depth_key_bits;
    dp.hist = e->d_ctl->depth_hist;
    dp.hist_ready = true;
    dp.ticket_base = kTicketDepthSortBase;
    dp.tag_base = kTagDepthSort;
    dp.ctas_per_sm = int(e->settings.sort_ctas_per_sm);
    dp.items = e->settings.depth_sort_items == 4 || e->settings.depth_sort_items == 8 ? e->settings.depth_sort_items : 16;
    dp.threads = e->settings.depth_sort_threads == 512 ? 512 : 256;
    dp.fixed_count = items;
    dp.compact_culled = true;  // culled items leave in the first pass; the rest sort ctl->depth_count
    e->depth_in_alt = launch_sort(e->d_dkeys[0], e->d_ditems[0], e->d_dkeys[1], e->d_ditems[1], items, dp,
                                  e->d_desc_depth, e->d_ctl, spin, e->num_sms, s);
    // the order is in the other buffer when a pass skipped (ctl->depth_skips odd)
    const uint32_t* order = e->d_ditems[e->depth_in_alt ? 1 : 0];
    const uint32_t* order_other = e->d_ditems[e->depth_in_alt ? 0 : 1];
    mark(2);
    const uint32_t cap = uint32_t(e->capacity);
    launch_keygen_scan(e->d_splats, order, order_other, items, e->n, e->d_views, e->d_offsets, e->d_tiles[0],
                       e->d_vals[0], cap, e->d_ranges, e->total_tiles, e->d_desc_pre,
                       counted ? e->d_sort_work : nullptr, e->d_ctl, spin, e->settings.test_never_publish, e->num_sms,
                       s);
    mark(3);
    SortPlan kp;
    kp.first_bit = 0;  // tile ids; the depth half of the keys is already in order
    kp.skip_on_overflow = true;
    kp.key_bits = e->key_bits - 32;
    kp.hist = e->d_ctl->sort_hist;
    kp.hist_ready = true;
    kp.ticket_base = kTicketKeySortBase;
    kp.tag_base = kTagKeySort;
    kp.ctas_per_sm = int(e->settings.sort_ctas_per_sm);
    kp.threads = e->settings.sort_threads == 256 ? 256 : 512;
    kp.ranges = e->d_ranges;  // the last pass writes the tile ranges
    kp.n_tiles = e->total_tiles;
    // counted passes (default), or onesweep passes with a look-back
    if (counted) {
        kp.counted_work = e->d_sort_work;
        kp.precounted = true;  // keygen counted the first pass's rows
        kp.ctas_per_sm = e->settings.sort_ctas_per_sm == 2 ? 2 : 3;
    }
    e->sorted_in_alt = launch_sort(e->d_tiles[0], e->d_vals[0], e->d_tiles[1], e->d_vals[1], cap, kp, e->d_desc_sort,
                                   e->d_ctl, spin, e->num_sms, s);
    mark(4);
    const int b = e->sorted_in_alt ? 1 : 0;
    mark(5);  // (tile ranges come out of the key sort's last pass)
    BlendArgs ba{};
    ba.splats = e->d_splats;
    ba.n = e->n;
    ba.ctl = e->d_ctl;
    ba.capacity = cap;
    ba.vals = e->d_vals[b];
    ba.ranges = e->d_ranges;
    ba.views = e->d_views;
    ba.tile_view = e->n_views > 1 ? e->d_tile_view : nullptr;
    ba.n_tiles = e->total_tiles;
    ba.image = e->d_image;
    ba.image_offset = e->n_views > 1 ? e->d_image_offset : nullptr;
    ba.final_T = state ? e->d_final_T : nullptr;
    ba.n_contrib = state ? e->d_n_contrib : nullptr;
    ba.rgba = rgba;
    launch_blend(ba, blend_launch(e), s);
    mark(6);
    // the backward stages of a frame without backward take no time; a
    // training step records them again after its adjoint kernels
    if (ev)
        for (int k = TPD_STAGE_BACKWARD_SETUP + 1; k <= TPD_STAGE_PREPROCESS_BACKWARD + 1; ++k) cudaEventRecord(ev[k], s);
    if (io) cudaMemcpyAsync(e->h_stats, e->d_ctl, sizeof(StatsHead), cudaMemcpyDeviceToHost, s);
}

// Clears the look-back descriptors (stream-ordered) before the frame whose
// tag reaches a multiple of kTagWindow; call once per frame launched, right
// before it is enqueued or its graph launched.
void before_frame(tpd_engine* e) {
    if (++e->tags % kTagWindow != 0) return;
    cudaMemsetAsync(e->d_desc_depth, 0, sort_desc_entries(uint32_t(e->splat_cap), 4) * 8, e->stream);
    cudaMemsetAsync(e->d_desc_pre, 0, e->desc_pre_cap * 8, e->stream);
    cudaMemsetAsync(e->d_desc_sort, 0, sort_desc_entries(uint32_t(e->capacity)) * 8, e->stream);
}

// Whether frames rendered now keep the adjoint's inputs (keep_backward_state).
bool frame_state(const tpd_engine* e) {
    return e->settings.keep_backward_state == 1 || (e->settings.keep_backward_state == 0 && e->backward_seen);
}

// The frame graph, captured again when it was captured with the other state choice.
int ensure_frame_graph(tpd_engine* e, bool state) {
    if (e->graph_valid && e->graph_state == state) return TPD_OK;
    if (e->graph) cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
    e->graph_valid = false;
    cudaGraph_t g = nullptr;
    TPD_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_frame(e, true, state);
    TPD_CUDA(e, cudaStreamEndCapture(e->stream, &g));
    cudaGraphExec_t ge = nullptr;
    const cudaError_t err = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    TPD_CUDA(e, err);
    e->graph = ge;
    e->graph_valid = true;
    e->graph_state = state;
    return TPD_OK;
}

int run_frame_once(tpd_engine* e, bool use_graph) {
    const bool state = frame_state(e);
    if (use_graph) {
        const int rc = ensure_frame_graph(e, state);
        if (rc != TPD_OK) return rc;
        before_frame(e);
        TPD_CUDA(e, cudaGraphLaunch(e->graph, e->stream));
    } else {
        before_frame(e);
        enqueue_frame(e, true, state);
        TPD_CUDA(e, cudaGetLastError());
    }
    e->state_kept = state;
    return wait_stream(e);
}

// Renders the last frame again, keeping the adjoint's inputs: from the device
// copies of its view constants and transforms, so a camera set since then
// does not enter. Enqueued only.
void rerender_with_state(tpd_engine* e) {
    before_frame(e);
    enqueue_frame(e, false, true);
    e->state_kept = true;
}

int set_views_internal(tpd_engine* e, const tpd_view* views, uint32_t nv) {
    if (nv == 0 || nv > kMaxViews) return fail(e, TPD_ERR_ARG, "view count must be in [1, 256]");
    bool shape_changed = nv != e->n_views;
    for (uint32_t v = 0; v < nv && !shape_changed; ++v)
        shape_changed = views[v].width != e->vw[v] || views[v].height != e->vh[v];
    for (uint32_t v = 0; v < nv; ++v)
        if (views[v].width == 0 || views[v].height == 0 || views[v].width > 65536 || views[v].height > 65536)
            return fail(e, TPD_ERR_ARG, "image size must be in [1, 65536]");
    uint32_t tiles = 0;
    uint64_t pixels = 0;
    std::vector<uint32_t> tile_view;
    std::vector<uint64_t> img_off(nv);
    for (uint32_t v = 0; v < nv; ++v) {
        ViewConst& c = e->h_views[v];
        std::memcpy(c.view, views[v].view, sizeof(c.view));
        tpd_mat4_mul(views[v].proj, views[v].view, c.projview);
        c.focal[0] = views[v].proj[0];
        c.focal[1] = views[v].proj[5];
        c.width = views[v].width;
        c.height = views[v].height;
        c.tile_base = tiles;
        const uint32_t t = grid_x(c.width) * grid_y(c.height);
        if (shape_changed) {
            tile_view.insert(tile_view.end(), t, v);
            img_off[v] = pixels;
        }
        tiles += t;
        pixels += uint64_t(c.width) * c.height;
    }
    if (!shape_changed) return TPD_OK;
    invalidate_graph(e);
    e->frame_valid = false;
    e->n_views = nv;
    e->vw.assign(nv, 0);
    e->vh.assign(nv, 0);
    for (uint32_t v = 0; v < nv; ++v) {
        e->vw[v] = views[v].width;
        e->vh[v] = views[v].height;
    }
    e->total_tiles = tiles;
    e->total_pixels = pixels;
    e->key_bits = tpd_key_bits_for_tiles(tiles);
    e->passes = sort_pass_count(e->key_bits) - 4;  // tile-id passes of the key sort
    {
        uint32_t vb = 0;
        while ((1u << vb) < nv) ++vb;
        e->depth_key_bits = 32 + vb;
    }
    if (pixels > e->pixel_cap) {
        TPD_CUDA(e, dalloc(e->d_image, pixels * 3));
        TPD_CUDA(e, dalloc(e->d_final_T, pixels));
        TPD_CUDA(e, dalloc(e->d_n_contrib, pixels));
        TPD_CUDA(e, dalloc(e->d_rgba, pixels));
        e->pixel_cap = pixels;
    }
    if (tiles > e->tile_cap) {
        TPD_CUDA(e, dalloc(e->d_ranges, uint64_t(tiles) * 2));
        TPD_CUDA(e, dalloc(e->d_tile_view, tiles));
        TPD_CUDA(e, dalloc(e->d_tile_order, tiles));
        e->tile_cap = tiles;
    }
    if (!e->d_image_offset) TPD_CUDA(e, dalloc(e->d_image_offset, kMaxViews));
    TPD_CUDA(e, cudaMemcpy(e->d_tile_view, tile_view.data(), tiles * 4ull, cudaMemcpyHostToDevice));
    TPD_CUDA(e, cudaMemcpy(e->d_image_offset, img_off.data(), nv * 8ull, cudaMemcpyHostToDevice));
    return ensure_splat_buffers(e);
}

int alloc_scene(tpd_engine* e, uint32_t n, uint32_t n_ent) {
    invalidate_graph(e);
    e->frame_valid = false;
    e->n = n;
    e->n_ent = n_ent ? n_ent : 1;
    TPD_CUDA(e, dalloc(e->d_recs, uint64_t(n) * kRecordFloats));
    if (e->h_transforms) cudaFreeHost(e->h_transforms);
    e->h_transforms = nullptr;
    TPD_CUDA(e, cudaMallocHost(reinterpret_cast<void**>(&e->h_transforms), sizeof(float) * 16 * e->n_ent));
    for (uint32_t k = 0; k < e->n_ent; ++k)
        for (int j = 0; j < 16; ++j) e->h_transforms[k * 16 + j] = (j % 5) == 0 ? 1.f : 0.f;
    e->identity_transforms = true;
    TPD_CUDA(e, dalloc(e->d_transforms, uint64_t(e->n_ent) * 16));
    if (e->n_views) return ensure_splat_buffers(e);
    return TPD_OK;
}

void fill_stats_from(tpd_engine* e, const StatsHead& h, tpd_frame_stats* stats, uint32_t retries) {
    if (!stats) return;
    std::memset(stats, 0, sizeof(*stats));
    stats->keys = h.total_keys;
    stats->key_capacity = e->capacity;
    stats->visible = h.visible;
    stats->tiles = e->total_tiles;
    stats->key_bits = e->key_bits;
    stats->sort_passes = e->passes;
    stats->status = h.status;
    stats->retries = retries;
    stats->views = e->n_views;
}

void fill_stats(tpd_engine* e, tpd_frame_stats* stats, uint32_t retries) {
    fill_stats_from(e, *e->h_stats, stats, retries);
}

// Pinned ring slots and staging images of the pipelined renders, sized for
// the current views and transforms (before any render is outstanding).
int ensure_ring(tpd_engine* e) {
    if (!e->copy_stream) {
        TPD_CUDA(e, cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < tpd_engine::kRing; ++i) {
            TPD_CUDA(e, cudaMallocHost(reinterpret_cast<void**>(&e->ring_views[i]), sizeof(ViewConst) * kMaxViews));
            TPD_CUDA(e, cudaMallocHost(reinterpret_cast<void**>(&e->ring_stats[i]), sizeof(StatsHead)));
            TPD_CUDA(e, cudaEventCreateWithFlags(&e->ring_ready[i], cudaEventDisableTiming));
            TPD_CUDA(e, cudaEventCreateWithFlags(&e->ring_done[i], cudaEventDisableTiming));
        }
    }
    if (!e->identity_transforms && e->n_ent > e->ring_transforms_cap) {
        invalidate_slot_graphs(e);  // they read the old buffers
        for (int i = 0; i < tpd_engine::kRing; ++i) {
            if (e->ring_transforms[i]) cudaFreeHost(e->ring_transforms[i]);
            e->ring_transforms[i] = nullptr;
            TPD_CUDA(e, cudaMallocHost(reinterpret_cast<void**>(&e->ring_transforms[i]), sizeof(float) * 16 * e->n_ent));
        }
        e->ring_transforms_cap = e->n_ent;
    }
    const uint64_t bytes = e->total_pixels * 12;  // room for RGB32F
    if (bytes > e->ring_image_cap) {
        invalidate_slot_graphs(e);
        for (int i = 0; i < tpd_engine::kRing; ++i) TPD_CUDA(e, dalloc(e->ring_image[i], bytes));
        e->ring_image_cap = bytes;
    }
    return TPD_OK;
}

// Status of a finished frame, as tpd_raster_frame reports it.
int frame_status(tpd_engine* e, const StatsHead& h) {
    if (h.status & kStatusKeyOverflow) {
        e->frame_valid = false;
        return fail(e, TPD_ERR_CAPACITY, "keys outgrew the key buffers; render with tpd_raster_frame");
    }
    if (h.status & kStatusBadIndex) {
        uint32_t dbg[4] = {0, 0, 0, 0};
        cudaMemcpy(dbg, e->d_ctl->debug, sizeof(dbg), cudaMemcpyDeviceToHost);
        return fail(e, TPD_ERR_DEVICE, "bounds check failed: site " + std::to_string(dbg[0]) + " index " +
                                           std::to_string((uint64_t(dbg[3]) << 32) | dbg[1]) + " bound " +
                                           std::to_string(dbg[2]));
    }
    if (h.status & kStatusFatal) return fail(e, TPD_ERR_TIMEOUT, "a bounded device wait ran out");
    return TPD_OK;
}

}  // namespace

extern "C" {

const char* tpd_version(void) { return "tpdsplat 0.1 (sm_103a)"; }

const char* tpd_status_string(int s) {
    switch (s) {
        case TPD_OK: return "ok";
        case TPD_ERR_ARG: return "invalid argument";
        case TPD_ERR_OOM: return "out of device memory";
        case TPD_ERR_TIMEOUT: return "timeout";
        case TPD_ERR_DEVICE: return "device error";
        case TPD_ERR_STATE: return "invalid state";
        case TPD_ERR_CAPACITY: return "capacity exceeded";
        case TPD_ERR_IO: return "i/o error";
        default: return "unknown";
    }
}

void tpd_settings_init(tpd_settings* s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    s->sh_degree = 3;
    s->band3_compat = 1;
    s->device = 0;
    s->use_graph = 1;
    s->timeout_s = 60.0;
}

int tpd_create(const tpd_settings* s, tpd_engine** out) {
    if (!out) return TPD_ERR_ARG;
    *out = nullptr;
    tpd_engine* e = new tpd_engine();
    if (s) e->settings = *s;
    else tpd_settings_init(&e->settings);
    if (e->settings.sh_degree > 3) e->settings.sh_degree = 3;  // GaussianEngine.cpp:366-370
    e->device = e->settings.device;
    auto bail = [&](int code) {
        tpd_destroy(e);
        return code;
    };
    if (cudaSetDevice(e->device) != cudaSuccess) return bail(TPD_ERR_DEVICE);
    cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->device);
    if (e->settings.stream) {
        e->stream = static_cast<cudaStream_t>(e->settings.stream);
    } else {
        if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(TPD_ERR_DEVICE);
        e->own_stream = true;
    }
    if (cudaEventCreateWithFlags(&e->done_event, cudaEventDisableTiming) != cudaSuccess) return bail(TPD_ERR_DEVICE);
    if (cudaMalloc(&e->d_ctl, sizeof(FrameCtl)) != cudaSuccess) return bail(TPD_ERR_OOM);
    if (cudaMemset(e->d_ctl, 0, sizeof(FrameCtl)) != cudaSuccess) return bail(TPD_ERR_DEVICE);
    if (cudaMallocHost(reinterpret_cast<void**>(&e->h_stats), sizeof(StatsHead)) != cudaSuccess) return bail(TPD_ERR_OOM);
    if (cudaMallocHost(reinterpret_cast<void**>(&e->h_views), sizeof(ViewConst) * kMaxViews) != cudaSuccess)
        return bail(TPD_ERR_OOM);
    std::memset(e->h_views, 0, sizeof(ViewConst) * kMaxViews);
    if (cudaMalloc(&e->d_views, sizeof(ViewConst) * kMaxViews) != cudaSuccess) return bail(TPD_ERR_OOM);
    if (e->settings.initial_key_capacity) {
        if (ensure_key_capacity(e, e->settings.initial_key_capacity) != TPD_OK) return bail(TPD_ERR_OOM);
    }
    *out = e;
    return TPD_OK;
}

void tpd_destroy(tpd_engine* e) {
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    invalidate_graph(e);
    dfree(e->d_recs);
    dfree(e->d_ent_idx);
    dfree(e->d_transforms);
    dfree(e->d_views);
    dfree(e->d_tile_view);
    dfree(e->d_tile_order);
    dfree(e->d_image_offset);
    dfree(e->d_splats);
    dfree(e->d_offsets);
    for (int b = 0; b < 2; ++b) {
        dfree(e->d_dkeys[b]);
        dfree(e->d_ditems[b]);
    }
    dfree(e->d_desc_depth);
    dfree(e->d_desc_pre);
    dfree(e->d_ent_mats);
    for (int b = 0; b < 2; ++b) {
        dfree(e->d_tiles[b]);
        dfree(e->d_vals[b]);
    }
    dfree(e->d_desc_sort);
    dfree(e->d_sort_work);
    dfree(e->d_keys64);
    dfree(e->d_ranges);
    dfree(e->d_image);
    dfree(e->d_final_T);
    dfree(e->d_n_contrib);
    dfree(e->d_rgba);
    dfree(e->d_g2d);
    dfree(e->d_gscratch);
    dfree(e->d_ctl);
    if (e->h_stats) cudaFreeHost(e->h_stats);
    if (e->h_views) cudaFreeHost(e->h_views);
    if (e->h_transforms) cudaFreeHost(e->h_transforms);
    if (e->copy_stream) cudaStreamSynchronize(e->copy_stream);
    for (int i = 0; i < tpd_engine::kRing; ++i) {
        if (e->ring_views[i]) cudaFreeHost(e->ring_views[i]);
        if (e->ring_transforms[i]) cudaFreeHost(e->ring_transforms[i]);
        if (e->ring_stats[i]) cudaFreeHost(e->ring_stats[i]);
        dfree(e->ring_image[i]);
        if (e->ring_ready[i]) cudaEventDestroy(e->ring_ready[i]);
        if (e->ring_done[i]) cudaEventDestroy(e->ring_done[i]);
    }
    if (e->copy_stream) cudaStreamDestroy(e->copy_stream);
    if (e->done_event) cudaEventDestroy(e->done_event);
    for (int i = 0; i < tpd_engine::kTimingSlots; ++i)
        for (int k = 0; k < tpd_engine::kTimingEvents; ++k)
            if (e->tev[i][k]) cudaEventDestroy(e->tev[i][k]);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

const char* tpd_last_error(const tpd_engine* e) { return e ? e->last_error.c_str() : "no engine"; }

int tpd_compile(tpd_engine* e, const void* records, uint32_t n, const uint32_t* entity_index, uint32_t n_entities) {
    if (!e) return TPD_ERR_ARG;
    if (n > 0 && !records) return fail(e, TPD_ERR_ARG, "records is NULL");
    if (n_entities == 0) n_entities = 1;
    if (entity_index) {
        for (uint32_t i = 0; i < n; ++i)
            if (entity_index[i] >= n_entities) return fail(e, TPD_ERR_ARG, "entity index out of range");
    }
    cudaSetDevice(e->device);
    int rc = alloc_scene(e, n, n_entities);
    if (rc != TPD_OK) return rc;
    if (n) TPD_CUDA(e, cudaMemcpy(e->d_recs, records, uint64_t(n) * kRecordBytes, cudaMemcpyHostToDevice));
    if (entity_index && n) {
        TPD_CUDA(e, dalloc(e->d_ent_idx, n));
        TPD_CUDA(e, cudaMemcpy(e->d_ent_idx, entity_index, n * 4ull, cudaMemcpyHostToDevice));
    } else {
        dfree(e->d_ent_idx);
    }
    e->compiled = true;
    return TPD_OK;
}

int tpd_compile_params_device(tpd_engine* e, const float* means, const float* log_scales, const float* quats,
                              const float* opacity_logits, const float* sh, uint32_t n) {
    if (!e) return TPD_ERR_ARG;
    if (n > 0 && (!means || !log_scales || !quats || !opacity_logits || !sh))
        return fail(e, TPD_ERR_ARG, "parameter pointer is NULL");
    cudaSetDevice(e->device);
    int rc = alloc_scene(e, n, 1);
    if (rc != TPD_OK) return rc;
    dfree(e->d_ent_idx);
    launch_pack_records(means, log_scales, quats, opacity_logits, sh, n, e->d_recs, e->stream);
    TPD_CUDA(e, cudaGetLastError());
    TPD_CUDA(e, cudaStreamSynchronize(e->stream));
    e->compiled = true;
    return TPD_OK;
}

int tpd_set_transform(tpd_engine* e, uint32_t entity, const float model[16]) {
    if (!e || !model) return TPD_ERR_ARG;
    if (!e->compiled) return fail(e, TPD_ERR_STATE, "set_transform before compile");
    if (entity >= e->n_ent) return TPD_OK;  // unknown entities are ignored (TransformHost.cpp:4-6)
    std::memcpy(e->h_transforms + entity * 16, model, 64);
    if (e->identity_transforms) invalidate_graph(e);  // the frame gains a transform upload
    e->identity_transforms = false;
    return TPD_OK;
}

int tpd_set_camera(tpd_engine* e, const float view[16], const float proj[16], uint32_t width, uint32_t height) {
    if (!e || !view || !proj) return TPD_ERR_ARG;
    tpd_view v;
    std::memcpy(v.view, view, 64);
    std::memcpy(v.proj, proj, 64);
    v.width = width;
    v.height = height;
    cudaSetDevice(e->device);
    return set_views_internal(e, &v, 1);
}

int tpd_set_views(tpd_engine* e, const tpd_view* views, uint32_t n_views) {
    if (!e || !views) return TPD_ERR_ARG;
    cudaSetDevice(e->device);
    return set_views_internal(e, views, n_views);
}

int tpd_raster_frame(tpd_engine* e, tpd_frame_stats* stats) {
    if (!e) return TPD_ERR_ARG;
    if (!e->compiled) return fail(e, TPD_ERR_STATE, "raster_frame before compile");
    if (!e->n_views) return fail(e, TPD_ERR_STATE, "raster_frame before set_camera");
    cudaSetDevice(e->device);
    int rc = ensure_splat_buffers(e);
    if (rc != TPD_OK) return rc;
    if (e->capacity == 0) {
        rc = ensure_key_capacity(e, std::max<uint64_t>(uint64_t(e->n) * e->n_views * 4, 1u << 20));
        if (rc != TPD_OK) return rc;
    }
    uint32_t retries = 0;
    e->frame_valid = false;
    while (true) {
        // the first frame after any reallocation runs eagerly; later ones replay the graph
        const bool graph = e->settings.use_graph && !e->settings.stage_timing && !e->needs_eager && retries == 0;
        rc = run_frame_once(e, graph);
        if (rc != TPD_OK) return rc;
        if (!graph) e->needs_eager = false;
        const StatsHead h = *e->h_stats;
        if (h.status & kStatusKeyOverflow) {
            if (retries >= 3) return fail(e, TPD_ERR_CAPACITY, "key buffers kept overflowing");
            rc = ensure_key_capacity(e, uint64_t(h.total_keys) + uint64_t(h.total_keys) / 4 + 1024);
            if (rc != TPD_OK) return rc;
            ++retries;
            continue;
        }
        if (h.status & kStatusBadIndex) {
            uint32_t dbg[4] = {0, 0, 0, 0};
            cudaMemcpy(dbg, e->d_ctl->debug, sizeof(dbg), cudaMemcpyDeviceToHost);
            return fail(e, TPD_ERR_DEVICE, "bounds check failed: site " + std::to_string(dbg[0]) + " index " +
                                               std::to_string((uint64_t(dbg[3]) << 32) | dbg[1]) + " bound " +
                                               std::to_string(dbg[2]));
        }
        if (h.status & (kStatusLookbackTimeout | kStatusMbarTimeout)) {
            e->frames++;
            return fail(e, TPD_ERR_TIMEOUT, "a bounded device wait ran out (status " + std::to_string(h.status) + ")");
        }
        break;
    }
    e->frames++;
    e->frame_valid = true;
    if (e->settings.stage_timing) harvest_all(e);
    fill_stats(e, stats, retries);
    return TPD_OK;
}

int tpd_raster_frames_async(tpd_engine* e, uint32_t count) {
    if (!e) return TPD_ERR_ARG;
    if (!e->frame_valid || e->needs_eager)
        return fail(e, TPD_ERR_STATE, "render one frame with tpd_raster_frame after any change first");
    cudaSetDevice(e->device);
    const bool graph = e->settings.use_graph && !e->settings.stage_timing;
    const bool state = frame_state(e);
    if (graph) {
        const int rc = ensure_frame_graph(e, state);
        if (rc != TPD_OK) return rc;
    }
    for (uint32_t i = 0; i < count; ++i) {
        before_frame(e);
        if (graph) TPD_CUDA(e, cudaGraphLaunch(e->graph, e->stream));
        else enqueue_frame(e, true, state);
    }
    TPD_CUDA(e, cudaGetLastError());
    if (count) e->state_kept = state;
    e->frames += count;
    return TPD_OK;
}

int tpd_sync(tpd_engine* e, tpd_frame_stats* stats) {
    if (!e) return TPD_ERR_ARG;
    cudaSetDevice(e->device);
    int rc = wait_stream(e);
    if (rc != TPD_OK) return rc;
    if (e->settings.stage_timing) harvest_all(e);
    const StatsHead h = *e->h_stats;
    fill_stats(e, stats, 0);
    if (h.status & kStatusKeyOverflow) {
        e->frame_valid = false;
        return fail(e, TPD_ERR_CAPACITY, "keys outgrew the key buffers; render with tpd_raster_frame");
    }
    if (h.status & kStatusFatal) return fail(e, TPD_ERR_TIMEOUT, "a bounded device wait ran out");
    return TPD_OK;
}

int tpd_render_async(tpd_engine* e, void* dst, uint32_t format, int dst_is_device) {
    if (!e || !dst) return TPD_ERR_ARG;
    if (format != TPD_IMAGE_RGB32F && format != TPD_IMAGE_RGBA8) return fail(e, TPD_ERR_ARG, "unknown image format");
    if (!e->frame_valid || e->needs_eager)
        return fail(e, TPD_ERR_STATE, "render one frame with tpd_raster_frame after any change first");
    cudaSetDevice(e->device);
    const int slot = int(e->ring_next % tpd_engine::kRing);
    if (e->ring_busy[slot]) return fail(e, TPD_ERR_STATE, "two renders outstanding: call tpd_wait_render first");
    if (e->ring_oldest == e->ring_next) {  // nothing outstanding: buffers may be resized
        const int rc = ensure_ring(e);
        if (rc != TPD_OK) return rc;
    } else if (e->total_pixels * 12 > e->ring_image_cap ||
               (!e->identity_transforms && e->n_ent > e->ring_transforms_cap)) {
        return fail(e, TPD_ERR_STATE, "the views grew while renders are outstanding: call tpd_wait_render first");
    }
    cudaStream_t s = e->stream;
    // the frame's constants, snapshotted into the slot (its last render has
    // been waited for); the slot's upload reads them when it runs
    std::memcpy(e->ring_views[slot], e->h_views, sizeof(ViewConst) * e->n_views);
    if (!e->identity_transforms)
        std::memcpy(e->ring_transforms[slot], e->h_transforms, sizeof(float) * 16 * e->n_ent);
    const int f = format == TPD_IMAGE_RGBA8 ? 0 : 1;
    const uint64_t bytes = format == TPD_IMAGE_RGBA8 ? e->total_pixels * 4 : e->total_pixels * 12;
    const bool state = frame_state(e);
    auto enqueue_slot = [&]() {
        cudaMemcpyAsync(e->d_views, e->ring_views[slot], sizeof(ViewConst) * e->n_views, cudaMemcpyHostToDevice, s);
        if (!e->identity_transforms)
            cudaMemcpyAsync(e->d_transforms, e->ring_transforms[slot], sizeof(float) * 16 * e->n_ent,
                            cudaMemcpyHostToDevice, s);
        enqueue_frame(e, false, state, f == 0 ? reinterpret_cast<uint32_t*>(e->ring_image[slot]) : nullptr);
        if (f == 1) cudaMemcpyAsync(e->ring_image[slot], e->d_image, bytes, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(e->ring_stats[slot], e->d_ctl, sizeof(StatsHead), cudaMemcpyDeviceToHost, s);
    };
    const bool graph = e->settings.use_graph && !e->settings.stage_timing;
    if (graph) {
        cudaGraphExec_t& G = e->slot_graph[slot][f];
        if (G && (e->slot_graph_state[slot][f] != state || e->slot_graph_ident[slot][f] != e->identity_transforms)) {
            cudaGraphExecDestroy(G);
            G = nullptr;
        }
        if (!G) {
            cudaGraph_t g = nullptr;
            TPD_CUDA(e, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            enqueue_slot();
            TPD_CUDA(e, cudaStreamEndCapture(s, &g));
            cudaGraphExec_t ge = nullptr;
            const cudaError_t err = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            TPD_CUDA(e, err);
            G = ge;
            e->slot_graph_state[slot][f] = state;
            e->slot_graph_ident[slot][f] = e->identity_transforms;
        }
        before_frame(e);
        TPD_CUDA(e, cudaGraphLaunch(G, s));
    } else {
        before_frame(e);
        enqueue_slot();
    }
    e->state_kept = state;
    TPD_CUDA(e, cudaEventRecord(e->ring_ready[slot], s));
    // the caller's copy runs beside the next frame
    TPD_CUDA(e, cudaStreamWaitEvent(e->copy_stream, e->ring_ready[slot], 0));
    TPD_CUDA(e, cudaMemcpyAsync(dst, e->ring_image[slot], bytes,
                                dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, e->copy_stream));
    TPD_CUDA(e, cudaEventRecord(e->ring_done[slot], e->copy_stream));
    TPD_CUDA(e, cudaGetLastError());
    e->ring_busy[slot] = true;
    ++e->ring_next;
    ++e->frames;
    return TPD_OK;
}

int tpd_wait_render(tpd_engine* e, tpd_frame_stats* stats) {
    if (!e) return TPD_ERR_ARG;
    if (e->ring_oldest == e->ring_next) return fail(e, TPD_ERR_STATE, "no render outstanding");
    cudaSetDevice(e->device);
    const int slot = int(e->ring_oldest % tpd_engine::kRing);
    const int rc = wait_event(e, e->ring_done[slot]);
    if (rc != TPD_OK) return rc;
    e->ring_busy[slot] = false;
    ++e->ring_oldest;
    const StatsHead h = *e->ring_stats[slot];
    fill_stats_from(e, h, stats, 0);
    return frame_status(e, h);
}

int tpd_stage_times(tpd_engine* e, double* ms, uint64_t* frames, int reset) {
    if (!e) return TPD_ERR_ARG;
    cudaSetDevice(e->device);
    harvest_all(e);
    if (ms) for (int k = 0; k < TPD_STAGE_COUNT; ++k) ms[k] = e->stage_ms[k];
    if (frames) *frames = e->timed_frames;
    if (reset) {
        for (int k = 0; k < TPD_STAGE_COUNT; ++k) e->stage_ms[k] = 0.0;
        e->timed_frames = 0;
    }
    return TPD_OK;
}

int tpd_read_image(tpd_engine* e, void* dst, uint32_t format, int dst_is_device) {
    if (!e || !dst) return TPD_ERR_ARG;
    if (!e->frame_valid) return fail(e, TPD_ERR_STATE, "no rendered frame");
    cudaSetDevice(e->device);
    const cudaMemcpyKind kind = dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (format == TPD_IMAGE_RGB32F) {
        TPD_CUDA(e, cudaMemcpyAsync(dst, e->d_image, e->total_pixels * 12, kind, e->stream));
    } else if (format == TPD_IMAGE_RGBA8) {
        launch_pack_rgba8(e->d_image, e->d_rgba, e->total_pixels, e->stream);
        TPD_CUDA(e, cudaGetLastError());
        TPD_CUDA(e, cudaMemcpyAsync(dst, e->d_rgba, e->total_pixels * 4, kind, e->stream));
    } else {
        return fail(e, TPD_ERR_ARG, "unknown image format");
    }
    return wait_stream(e);
}

}  // extern "C"

namespace {

struct BackwardOut {
    float *means, *log_scales, *quats, *logits, *sh;
};

// Sizes the backward's buffers (before any capture: this may allocate) and
// points absent gradient outputs at engine scratch.
int prepare_backward(tpd_engine* e, BackwardOut& o) {
    const uint64_t g2d = uint64_t(e->n) * e->n_views * kG2DStride;
    if (g2d > e->g2d_cap) {
        invalidate_step_graph(e);
        TPD_CUDA(e, dalloc(e->d_g2d, g2d));
        e->g2d_cap = g2d;
    }
    const uint64_t gs = uint64_t(e->n) * (3 + 3 + 4 + 1 + 48);
    if ((!o.means || !o.log_scales || !o.quats || !o.logits || !o.sh) && gs > e->gscratch_cap) {
        invalidate_step_graph(e);
        TPD_CUDA(e, dalloc(e->d_gscratch, gs));
        e->gscratch_cap = gs;
    }
    // scratch sections: quaternions and SH first, so both start 16-byte aligned
    float* sc = e->d_gscratch;
    const uint64_t n = e->n;
    if (!o.quats) o.quats = sc;
    if (!o.sh) o.sh = sc + n * 4;
    if (!o.means) o.means = sc + n * 52;
    if (!o.log_scales) o.log_scales = sc + n * 55;
    if (!o.logits) o.logits = sc + n * 58;
    return TPD_OK;
}

// Blend adjoint (per-splat gradients, zeroed first) then preprocess adjoint.
void enqueue_backward(tpd_engine* e, const float* dL_dimage, const BackwardOut& o) {
    // stage timing: the events of the frame this backward follows, while
    // that frame's slot has not been harvested (tpd_step_async)
    cudaEvent_t* ev = nullptr;
    if (e->settings.stage_timing && e->cur_tslot >= 0 && e->tev_pending[e->cur_tslot]) ev = e->tev[e->cur_tslot];
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], e->stream);
    };
    cudaMemsetAsync(e->d_g2d, 0, uint64_t(e->n) * e->n_views * kG2DStride * 4, e->stream);
    const int b = e->sorted_in_alt ? 1 : 0;
    BlendBackwardArgs bb{};
    bb.splats = e->d_splats;
    bb.n = e->n;
    bb.ctl = e->d_ctl;
    bb.capacity = uint32_t(e->capacity);
    bb.vals = e->d_vals[b];
    bb.ranges = e->d_ranges;
    bb.views = e->d_views;
    bb.tile_view = e->n_views > 1 ? e->d_tile_view : nullptr;
    bb.n_tiles = e->total_tiles;
    bb.image_offset = e->n_views > 1 ? e->d_image_offset : nullptr;
    bb.final_T = e->d_final_T;
    bb.n_contrib = e->d_n_contrib;
    bb.dL_dimage = dL_dimage;
    bb.g2d = e->d_g2d;
    bb.g2d_view_stride = uint64_t(e->n) * kG2DStride;
    // longest tile lists first: the adjoint's cost per tile varies more than the forward's
    launch_tile_order(e->d_ranges, e->total_tiles, e->d_ctl, uint32_t(e->capacity), e->d_tile_order, e->stream);
    bb.tile_order = e->d_tile_order;
    mark(TPD_STAGE_BACKWARD_SETUP + 1);
    launch_blend_backward(bb, blend_launch(e), e->stream);
    mark(TPD_STAGE_BLEND_BACKWARD + 1);
    PreprocessBackwardArgs pb{};
    pb.recs = e->d_recs;
    pb.n = e->n;
    pb.ent_idx = e->d_ent_idx;
    pb.ent_mats = e->d_ent_mats;
    pb.n_ent = e->n_ent;
    pb.views = e->d_views;
    pb.n_views = e->n_views;
    pb.sh_degree = e->settings.sh_degree;
    pb.band3_compat = e->settings.band3_compat;
    pb.splats = e->d_splats;
    pb.g2d = e->d_g2d;
    pb.g_means = o.means;
    pb.g_log_scales = o.log_scales;
    pb.g_quats = o.quats;
    pb.g_logits = o.logits;
    pb.g_sh = o.sh;
    launch_preprocess_backward(pb, e->stream);
    mark(TPD_STAGE_PREPROCESS_BACKWARD + 1);
}

}  // namespace

extern "C" {

int tpd_backward(tpd_engine* e, const float* dL_dimage, float* g_means, float* g_log_scales, float* g_quats,
                 float* g_logits, float* g_sh) {
    if (!e || !dL_dimage) return TPD_ERR_ARG;
    if (!e->frame_valid) return fail(e, TPD_ERR_STATE, "backward before a rendered frame");
    cudaSetDevice(e->device);
    e->backward_seen = true;  // with keep_backward_state 0, later frames keep the adjoint's inputs
    BackwardOut o{g_means, g_log_scales, g_quats, g_logits, g_sh};
    const int rc = prepare_backward(e, o);
    if (rc != TPD_OK) return rc;
    if (!e->state_kept) rerender_with_state(e);
    enqueue_backward(e, dL_dimage, o);
    TPD_CUDA(e, cudaGetLastError());
    return wait_stream(e);
}

int tpd_step_async(tpd_engine* e, const float* dL_dimage, float* g_means, float* g_log_scales, float* g_quats,
                   float* g_logits, float* g_sh, uint32_t count) {
    if (!e || !dL_dimage) return TPD_ERR_ARG;
    if (!e->frame_valid || e->needs_eager)
        return fail(e, TPD_ERR_STATE, "render one frame with tpd_raster_frame after any change first");
    cudaSetDevice(e->device);
    BackwardOut o{g_means, g_log_scales, g_quats, g_logits, g_sh};
    const int rc = prepare_backward(e, o);
    if (rc != TPD_OK) return rc;
    const bool graph = e->settings.use_graph && !e->settings.stage_timing;
    const void* key[6] = {dL_dimage, o.means, o.log_scales, o.quats, o.logits, o.sh};
    if (graph && (!e->step_graph || std::memcmp(key, e->step_key, sizeof(key)) != 0)) {
        invalidate_step_graph(e);
        cudaGraph_t g = nullptr;
        TPD_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_frame(e);
        enqueue_backward(e, dL_dimage, o);
        TPD_CUDA(e, cudaStreamEndCapture(e->stream, &g));
        cudaGraphExec_t ge = nullptr;
        const cudaError_t err = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        TPD_CUDA(e, err);
        e->step_graph = ge;
        std::memcpy(e->step_key, key, sizeof(key));
    }
    for (uint32_t i = 0; i < count; ++i) {
        before_frame(e);
        if (graph) {
            TPD_CUDA(e, cudaGraphLaunch(e->step_graph, e->stream));
        } else {
            enqueue_frame(e);
            enqueue_backward(e, dL_dimage, o);
        }
    }
    TPD_CUDA(e, cudaGetLastError());
    if (count) e->state_kept = true;  // a training step's frame keeps the adjoint's inputs
    e->frames += count;
    return TPD_OK;
}

namespace {

// The sorted (tile | depth) keys of the last frame, for read-back: the frame
// itself sorts tile ids only (their depth order comes from the presort), and
// a key's depth is that of its value's splat, so the keys are rebuilt here
// into a buffer of their own, allocated on first use. Waits for the stream.
int rebuild_keys(tpd_engine* e) {
    cudaSetDevice(e->device);
    if (e->keys64_cap < e->capacity) {
        dfree(e->d_keys64);
        e->keys64_cap = 0;
        TPD_CUDA(e, dalloc(e->d_keys64, e->capacity));
        e->keys64_cap = e->capacity;
    }
    const int b = e->sorted_in_alt ? 1 : 0;
    launch_materialize_keys(e->d_tiles[b], e->d_vals[b], e->d_splats, e->n, e->n_views > 1 ? e->d_tile_view : nullptr,
                            e->total_tiles, uint32_t(e->capacity), e->d_ctl, e->d_keys64, e->stream);
    TPD_CUDA(e, cudaGetLastError());
    return wait_stream(e);
}

}  // namespace

int tpd_get_buffer(const tpd_engine* e, uint32_t which, void** ptr, uint64_t* bytes) {
    if (!e || !ptr) return TPD_ERR_ARG;
    if (which == TPD_BUF_KEYS && e->capacity > 0) {
        const int rc = rebuild_keys(const_cast<tpd_engine*>(e));  // a read-back cache, not engine state
        if (rc != TPD_OK) return rc;
    }
    if ((which == TPD_BUF_FINAL_T || which == TPD_BUF_N_CONTRIB) && e->frame_valid && !e->state_kept) {
        tpd_engine* m = const_cast<tpd_engine*>(e);  // the same frame, with the buffers asked for
        cudaSetDevice(m->device);
        rerender_with_state(m);
        TPD_CUDA(m, cudaGetLastError());
        const int rc = wait_stream(m);
        if (rc != TPD_OK) return rc;
    }
    const int b = e->sorted_in_alt ? 1 : 0;
    void* p = nullptr;
    uint64_t sz = 0;
    const uint64_t vn = uint64_t(e->n) * e->n_views;
    switch (which) {
        case TPD_BUF_RECORDS: p = e->d_recs; sz = uint64_t(e->n) * kRecordBytes; break;
        case TPD_BUF_SPLATS: p = e->d_splats; sz = vn * sizeof(Splat); break;
        case TPD_BUF_OFFSETS: p = e->d_offsets; sz = vn * 4; break;
        case TPD_BUF_KEYS: p = e->d_keys64; sz = e->keys64_cap * 8; break;
        case TPD_BUF_VALUES: p = e->d_vals[b]; sz = e->capacity * 4; break;
        case TPD_BUF_RANGES: p = e->d_ranges; sz = uint64_t(e->total_tiles) * 8; break;
        case TPD_BUF_IMAGE: p = e->d_image; sz = e->total_pixels * 12; break;
        case TPD_BUF_FINAL_T: p = e->d_final_T; sz = e->total_pixels * 4; break;
        case TPD_BUF_N_CONTRIB: p = e->d_n_contrib; sz = e->total_pixels * 4; break;
        case TPD_BUF_G2D: p = e->d_g2d; sz = vn * kG2DStride * 4; break;
        default: return TPD_ERR_ARG;
    }
    *ptr = p;
    if (bytes) *bytes = sz;
    return TPD_OK;
}

int tpd_read_buffer(tpd_engine* e, uint32_t which, void* dst, uint64_t offset, uint64_t bytes, int dst_is_device) {
    if (!e || !dst) return TPD_ERR_ARG;
    void* p = nullptr;
    uint64_t sz = 0;
    int rc = tpd_get_buffer(e, which, &p, &sz);
    if (rc != TPD_OK) return rc;
    if (offset + bytes > sz || !p) return fail(e, TPD_ERR_ARG, "read past the end of the buffer");
    cudaSetDevice(e->device);
    TPD_CUDA(e, cudaMemcpyAsync(dst, static_cast<char*>(p) + offset, bytes,
                                dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, e->stream));
    return wait_stream(e);
}

void* tpd_get_stream(const tpd_engine* e) { return e ? static_cast<void*>(e->stream) : nullptr; }

// ---- stage entry points

size_t tpd_sort_workspace_size(uint32_t n) {
    return 256 * ((sizeof(FrameCtl) + 255) / 256) + sort_desc_entries(n) * 8;
}

int tpd_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                   uint32_t key_bits, void* workspace, size_t workspace_bytes, void* stream, int* result_in_alt) {
    if (!result_in_alt) return TPD_ERR_ARG;
    *result_in_alt = 0;
    if (n == 0) return TPD_OK;
    if (!keys || !vals || !keys_alt || !vals_alt || !workspace) return TPD_ERR_ARG;
    if (key_bits == 0 || key_bits > 64 || n > 0x7FFFFFFFu) return TPD_ERR_ARG;
    if (workspace_bytes < tpd_sort_workspace_size(n)) return TPD_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    FrameCtl* ctl = static_cast<FrameCtl*>(workspace);
    uint64_t* desc = reinterpret_cast<uint64_t*>(static_cast<char*>(workspace) + 256 * ((sizeof(FrameCtl) + 255) / 256));
    int sms = 148, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaMemsetAsync(desc, 0, sort_desc_entries(n) * 8, s) != cudaSuccess) return TPD_ERR_DEVICE;
    launch_sort_begin(ctl, n, s);
    SortPlan plan;
    plan.first_bit = 0;
    plan.key_bits = key_bits;
    plan.hist = ctl->sort_hist;
    plan.hist_ready = false;
    // onesweep passes of 256 threads x 16 keys (ballot ranking, 2 CTAs per SM)
    // with a look-back: on 64-bit keys faster than 512 x 8 keys with match
    // ranking (0.845 against 0.910 ms for 9M random keys of 45 bits, the
    // histogram kernel included) and than the counted passes that serve the
    // frame's 32-bit key sort
    plan.threads = 256;
    plan.ctas_per_sm = 2;
    const bool alt = launch_sort(keys, vals, keys_alt, vals_alt, n, plan, desc, ctl, kDefaultSpin, sms, s);
    *result_in_alt = alt ? 1 : 0;
    return cudaGetLastError() == cudaSuccess ? TPD_OK : TPD_ERR_DEVICE;
}

size_t tpd_scan_workspace_size(uint32_t n) {
    return 256 * ((sizeof(FrameCtl) + 255) / 256) + (size_t(n) / kScanTileStandalone + 2) * 8;
}

int tpd_scan_tiles(const void* splats, uint32_t n, uint32_t* offsets, uint32_t* total, void* workspace,
                   size_t workspace_bytes, void* stream) {
    if (!total || !workspace) return TPD_ERR_ARG;
    if (n > 0 && (!splats || !offsets)) return TPD_ERR_ARG;
    if (workspace_bytes < tpd_scan_workspace_size(n)) return TPD_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    FrameCtl* ctl = static_cast<FrameCtl*>(workspace);
    uint64_t* desc = reinterpret_cast<uint64_t*>(static_cast<char*>(workspace) + 256 * ((sizeof(FrameCtl) + 255) / 256));
    const size_t entries = size_t(n) / kScanTileStandalone + 2;
    if (cudaMemsetAsync(desc, 0, entries * 8, s) != cudaSuccess) return TPD_ERR_DEVICE;
    launch_sort_begin(ctl, 0, s);
    launch_scan_tiles(static_cast<const Splat*>(splats), n, offsets, desc, ctl, kDefaultSpin,
                      test_never_publish_standalone(), s);
    if (cudaMemcpyAsync(total, &ctl->total_keys, 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return TPD_ERR_DEVICE;
    return cudaGetLastError() == cudaSuccess ? TPD_OK : TPD_ERR_DEVICE;
}

void tpd_test_set_never_publish(uint32_t on) { g_never_publish_standalone.store(on ? 1u : 0u); }

}  // extern "C"
