// keygen.cu — kernel (b): the tile-count scan and key duplication, as one
// kernel over the Gaussians in depth order.
//
// Reference: prefix.slang:40-158 (the scan of the per-Gaussian tile counts)
// and keygen.slang:23-53 (one thread per Gaussian looping over its tile
// rect). It also presets the tile ranges (fillBuffer, GaussianEngine.cpp:843-848)
// that the key sort's last pass fills in (range.slang:18-35, in sort.cu), and
// counts the key sort's first-pass digits per 4096-key partition.
//
// GB300 form of keygen: Gaussians are visited in depth order (a prior sort of
// the (view | depth) keys), so the emitted keys only need a stable sort on
// their tile-id bits afterwards: per tile the order is (depth, index), exactly
// the reference's stable sort of (tile | depth) keys emitted in index order.
// A warp owns 32 consecutive Gaussians and writes their (contiguous) keys
// one output slot per lane, finding each slot's Gaussian through a small
// owner map in shared memory, so stores are coalesced and one large Gaussian
// does not serialise its warp. Keys and values are bit-identical to the
// reference's.
#include <algorithm>

#include "tpd_common.cuh"
#include "tpd_kernels.h"
#include "tpd_scan.cuh"

namespace tpd {
namespace {

constexpr uint32_t kKeygenThreads = 256;
constexpr uint32_t kKeygenChunks = kKeygenPart / kKeygenThreads;  // 32-item chunks per warp and partition
static_assert(kKeygenChunks * kKeygenThreads == kKeygenPart, "a partition is whole chunks of every warp");
static_assert(kKeygenThreads == 256, "a thread per low tile-id digit flushes the partition counts");

// A warp writes the keys of 32 consecutive items (one per lane), whose keys
// are contiguous, in windows of kKeyWindow output slots:
//  1. each lane with keys marks its first slot in the window's owner map,
//     a prefix-max over the map gives every slot its owning lane;
//  2. lane l fills slots l, l + 32, ...: owner's rectangle from a per-warp
//     table, (row, column) of the slot's index inside the rectangle, the key,
//     one coalesced store of key and value.
constexpr uint32_t kKeyWindow = 256;
constexpr uint32_t kKeygenWarps = kKeygenThreads / 32;

struct KeygenSmem {
    uint32_t owner[kKeygenWarps][kKeyWindow];  // owning lane of each slot of the window
    uint32_t t0[kKeygenWarps][32];             // first tile of the lane's rectangle
    uint32_t wgx[kKeygenWarps][32];            // rectangle width | view grid width << 16
    uint32_t excl[kKeygenWarps][32];           // first slot of the lane's keys (warp-relative)
    uint32_t gi[kKeygenWarps][32];             // Gaussian index
};

// Per item of a warp's 32 (one per lane): the first tile of its rectangle (t0,
// row-major in its view), the rectangle's width and the view's grid width
// (wgx = w | gx << 16), its key count (w h) and Gaussian index.
struct ItemRect {
    uint32_t t0, wgx, cnt, gi;
};

__device__ __forceinline__ ItemRect item_rect(uint32_t item, bool valid, float4 texel, uint32_t n_items, uint32_t n,
                                              const ViewConst* __restrict__ views, FrameCtl* ctl) {
    uint32_t w = 1, h = 0, gx = 1, gi = 0, t0 = 0;
    if (valid && TPD_INBOUNDS(ctl, 21, item, n_items)) {
        const uint32_t v = n_items == n ? 0u : item / n;  // one view: no division
        gi = item - v * n;
        const ViewConst& vc = views[v];
        gx = grid_x(vc.width);
        if (texel.w > 0.0f) {
            uint32_t x0, y0, x1, y1;
            bounding_rect(texel.x, texel.y, texel.w, gx, grid_y(vc.height), x0, y0, x1, y1);
            if (x1 > x0 && y1 > y0) {
                w = x1 - x0;
                h = y1 - y0;
                t0 = vc.tile_base + y0 * gx + x0;
            }
        }
    }
    return ItemRect{t0, w | (gx << 16), w * h, gi};
}

// Writes the keys of a warp's 32 items, `total` in all, to output slots
// base .. base + total - 1 (lane l's item from slot base + excl), in windows
// of kKeyWindow slots, one coalesced store per lane and step (the owner-map
// scheme above). Called by the whole warp.
// With count_rows, each written key also adds one to its 4096-key sort
// partition's count of its low tile-id digit: in s_cnt (kCountWindow rows,
// partitions p0 .. p0 + kCountWindow - 1) when its partition is there, else
// straight into count_rows.
constexpr uint32_t kCountWindow = 8;

__device__ __forceinline__ void write_warp_keys(KeygenSmem& S, uint32_t warp, uint32_t lane, const ItemRect& it,
                                                uint32_t excl, uint32_t total, uint32_t base, uint32_t capacity,
                                                uint32_t* __restrict__ tiles, uint32_t* __restrict__ vals,
                                                uint32_t* s_cnt, uint32_t p0, uint32_t* __restrict__ count_rows) {
    uint32_t* owner = S.owner[warp];
    const uint32_t cnt = it.cnt;
    S.t0[warp][lane] = it.t0;
    S.wgx[warp][lane] = it.wgx;
    S.excl[warp][lane] = excl;
    S.gi[warp][lane] = it.gi;
    for (uint32_t c0 = 0; c0 < total; c0 += kKeyWindow) {
        const uint32_t span = min(kKeyWindow, total - c0);
        // 1. owner map: segment starts, then a prefix max over the window
        //    (owners grow with the slot; slot c0 belongs to the last lane
        //    whose keys start at or before it)
#pragma unroll
        for (uint32_t q = 0; q < kKeyWindow / 32; ++q) owner[lane * (kKeyWindow / 32) + q] = 0;
        __syncwarp();
        if (cnt && excl >= c0 && excl < c0 + kKeyWindow) owner[excl - c0] = lane;
        const uint32_t first_owner = 31u - __clz(__ballot_sync(0xFFFFFFFFu, excl <= c0 && cnt));
        __syncwarp();
        uint32_t run = 0, mine[kKeyWindow / 32];
#pragma unroll
        for (uint32_t q = 0; q < kKeyWindow / 32; ++q) {
            run = max(run, owner[lane * (kKeyWindow / 32) + q]);
            mine[q] = run;
        }
        uint32_t before = run;  // exclusive prefix max of the lanes' maxima
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, before, o);
            if (lane >= o) before = max(before, x);
        }
        before = __shfl_up_sync(0xFFFFFFFFu, before, 1);
        before = max(lane ? before : 0u, first_owner);
        __syncwarp();
#pragma unroll
        for (uint32_t q = 0; q < kKeyWindow / 32; ++q) owner[lane * (kKeyWindow / 32) + q] = max(before, mine[q]);
        __syncwarp();
        // 2. slots lane, lane + 32, ...: one coalesced store group per step
        for (uint32_t q = lane; q < span; q += 32u) {
            if (uint64_t(base) + c0 + q < capacity) {
                const uint32_t j = owner[q];
                const uint32_t local = c0 + q - S.excl[warp][j];  // < 2^24: exact in a float
                const uint32_t jwg = S.wgx[warp][j];
                const uint32_t jw = jwg & 0xFFFFu;
                // row = local / jw from a float quotient, corrected by one step
                uint32_t ty = __float2uint_rz(__fdividef(float(local), float(jw)));
                int32_t rem = int32_t(local) - int32_t(ty * jw);
                if (rem < 0) {
                    --ty;
                    rem += int32_t(jw);
                } else if (rem >= int32_t(jw)) {
                    ++ty;
                    rem -= int32_t(jw);
                }
                const uint32_t tile = S.t0[warp][j] + ty * (jwg >> 16) + uint32_t(rem);
                const uint64_t pos = uint64_t(base) + c0 + q;
                tiles[pos] = tile;
                vals[pos] = S.gi[warp][j];
                if (count_rows) {
                    const uint32_t part = uint32_t(pos >> 12), d = tile & 255u;
                    if (part - p0 < kCountWindow)
                        atomicAdd(&s_cnt[(part - p0) * 256u + d], 1u);
                    else
                        atomicAdd(&count_rows[size_t(part) * 256u + d], 1u);
                }
            }
        }
        __syncwarp();  // the owner map is rebuilt for the next window
    }
    __syncwarp();  // the lane table is rewritten by the next items
}

// The depth-order tile-count scan fused with key duplication. Persistent
// CTAs take partitions of kKeygenPart consecutive items in depth order by an
// atomic ticket; warp w of a CTA owns the partition's items
// [w kKeygenChunks 32, (w + 1) kKeygenChunks 32), in kKeygenChunks chunks of
// 32 (one item per lane). Per partition:
//  1. each lane gathers its items' splat texels and works out their tile
//     rectangles, so its key counts;
//  2. the counts are scanned across the warp, then across the CTA;
//  3. one warp resolves the partition's exclusive prefix with the bounded
//     decoupled look-back (prefix.slang:100-114 as restated in tpd_scan.cuh):
//     the last partition's inclusive prefix is the frame's key count K;
//  4. each lane writes its items' key offsets (the scan's output), and each
//     warp writes its chunks' keys (write_warp_keys).
// A key is stored as its tile id alone: the low 32 bits of the reference's
// key are the depth, already in order (the items come in depth order), and
// the depth of a key is that of its value's splat, so the sort needs only the
// tile ids and the full keys can be rebuilt from (tile, value) when read.
// Keys past the capacity are not written (the frame is flagged and rendered
// again). The digit counts of the tile ids come from the preprocess, which
// counts each Gaussian's tile rectangle row by row.
// A CTA takes a ticket only when it starts on the partition, so every
// partition a look-back waits on is being worked on by a running CTA and
// publishes its aggregate soon. With count_rows, a partition's keys (one
// contiguous run of slots) are also counted per 4096-key sort partition and
// low tile-id digit in shared memory, and the non-zero counts added into
// count_rows with one atomic each once the partition is written: the key
// sort's first pass then needs no counting kernel.
struct KeygenScanSmem {
    KeygenSmem k;
    uint32_t cnt[kCountWindow * 256];  // low-digit counts of sort partitions p0 .. p0 + kCountWindow - 1
    uint32_t wtot[kKeygenWarps];  // key counts of the warps' items
    uint32_t ticket;              // the partition being worked on
    uint32_t excl;                // the partition's exclusive prefix
};

__global__ void __launch_bounds__(kKeygenThreads)
    keygen_scan_kernel(const Splat* __restrict__ splats, const uint32_t* __restrict__ items,
                       const uint32_t* __restrict__ items_other, uint32_t n_items, uint32_t n,
                       const ViewConst* __restrict__ views, uint32_t* __restrict__ offsets,
                       uint32_t* __restrict__ tiles, uint32_t* __restrict__ vals, uint32_t capacity,
                       uint32_t* __restrict__ ranges, uint32_t n_tiles, uint64_t* desc,
                       uint32_t* __restrict__ count_rows, FrameCtl* ctl, uint32_t spin_limit,
                       uint32_t never_publish) {
    __shared__ KeygenScanSmem S;
    pdl_wait();     // launched as a dependent of the depth sort's last pass: its order is read below
    pdl_trigger();  // the key sort's first counting kernel may be scheduled (it waits for this grid)
    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const uint32_t count = min(ctl->depth_count, n_items);
    if (ctl->depth_skips & 1u) items = items_other;  // a skipped depth pass left the order there
    // ranges: (0xFFFFFFFF, 0) until the key sort's last pass narrows them
    for (uint32_t t = blockIdx.x * blockDim.x + tid; t < n_tiles; t += gridDim.x * blockDim.x)
        reinterpret_cast<uint2*>(ranges)[t] = make_uint2(0xFFFFFFFFu, 0u);
    const uint32_t nparts = (count + kKeygenPart - 1) / kKeygenPart;
    const uint32_t tag = ctl->tag * 32u + kTagScan;
#pragma unroll
    for (uint32_t w = 0; w < kCountWindow; ++w) S.cnt[w * 256u + tid] = 0;  // (before the first barrier)
    for (;;) {
        // one thread reads the status for the whole CTA (a look-back of this
        // grid may raise a fatal bit meanwhile, and every thread must take the
        // same way through the barriers): a fatal status ends the CTA as a
        // ticket past the last partition does
        if (tid == 0)
            S.ticket = (ctl->status & kStatusFatal) ? 0xFFFFFFFFu : atomicAdd(&ctl->ticket[kTicketScan], 1u);
        __syncthreads();
        const uint32_t part = S.ticket;
        if (part >= nparts) break;  // (uniform)
        const uint32_t r0 = part * kKeygenPart + warp * (kKeygenChunks * 32u) + lane;
        uint32_t item[kKeygenChunks];
        float4 texel[kKeygenChunks];
#pragma unroll
        for (uint32_t c = 0; c < kKeygenChunks; ++c) item[c] = r0 + 32u * c < count ? items[r0 + 32u * c] : 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t c = 0; c < kKeygenChunks; ++c)
            texel[c] = item[c] < n_items ? reinterpret_cast<const float4*>(splats + item[c])[1]
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
        ItemRect rect[kKeygenChunks];
        uint32_t incl[kKeygenChunks], ctot[kKeygenChunks], wtotal = 0, vis = 0;
#pragma unroll
        for (uint32_t c = 0; c < kKeygenChunks; ++c) {
            rect[c] = item_rect(item[c], r0 + 32u * c < count, texel[c], n_items, n, views, ctl);
            incl[c] = warp_inclusive_scan(rect[c].cnt);
            ctot[c] = __shfl_sync(0xFFFFFFFFu, incl[c], 31);
            wtotal += ctot[c];
            vis += rect[c].cnt ? 1u : 0u;
        }
        vis = warp_sum(vis);
        if (lane == 0) {
            S.wtot[warp] = wtotal;
            if (vis) atomicAdd(&ctl->visible, vis);
        }
        __syncthreads();
        uint32_t wbase = 0, total = 0;
#pragma unroll
        for (uint32_t w = 0; w < kKeygenWarps; ++w) {
            const uint32_t sw = S.wtot[w];
            wbase += w < warp ? sw : 0u;
            total += sw;
        }
        if (warp == 0) {
            const uint32_t ex = warp_lookback(desc, part, total, tag, &ctl->status, spin_limit, never_publish != 0);
            if (lane == 0) {
                S.excl = ex;
                if (part == nparts - 1u) {
                    ctl->total_keys = ex + total;
                    if (ex + total > capacity) atomicOr(&ctl->status, kStatusKeyOverflow);
                }
            }
        }
        __syncthreads();
        const uint32_t p0 = S.excl >> 12;  // the sort partition of the partition's first key
        uint32_t base = S.excl + wbase;
#pragma unroll
        for (uint32_t c = 0; c < kKeygenChunks; ++c) {
            const uint32_t excl = incl[c] - rect[c].cnt;
            if (r0 + 32u * c < count) offsets[r0 + 32u * c] = base + excl;
            write_warp_keys(S.k, warp, lane, rect[c], excl, ctot[c], base, capacity, tiles, vals, S.cnt, p0,
                            count_rows);
            base += ctot[c];
        }
        __syncthreads();  // S.ticket, S.wtot and S.excl are rewritten for the next partition; S.cnt is complete
        if (count_rows) {
            // thread d flushes and clears digit d's counts (the next
            // partition's keys add to them only after its barriers)
#pragma unroll
            for (uint32_t w = 0; w < kCountWindow; ++w) {
                const uint32_t c = S.cnt[w * 256u + tid];
                if (c) {
                    atomicAdd(&count_rows[size_t(p0 + w) * 256u + tid], c);
                    S.cnt[w * 256u + tid] = 0;
                }
            }
        }
    }
}

int keygen_setup() {
    int r = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, keygen_scan_kernel, kKeygenThreads, 0);
    return r > 0 ? r : 1;
}

}  // namespace

void launch_keygen_scan(const Splat* splats, const uint32_t* items, const uint32_t* items_other, uint32_t n_items,
                        uint32_t n, const ViewConst* views, uint32_t* offsets, uint32_t* tiles, uint32_t* vals,
                        uint32_t capacity, uint32_t* ranges, uint32_t n_tiles, uint64_t* desc, uint32_t* count_rows,
                        FrameCtl* ctl, uint32_t spin_limit, uint32_t never_publish, int num_sms, cudaStream_t s) {
    if (n_items == 0 || n == 0) return;
    const uint64_t parts = (uint64_t(n_items) + kKeygenPart - 1) / kKeygenPart;
    const int per_sm = device_once(keygen_setup);  // resident CTAs per SM
    const uint64_t cap = uint64_t(num_sms > 0 ? num_sms : 148) * uint64_t(per_sm);  // persistent
    const uint64_t blocks = parts < cap ? parts : cap;
    launch_dependent(keygen_scan_kernel, dim3(unsigned(blocks)), dim3(kKeygenThreads), 0, s, splats, items,
                     items_other, n_items, n, views, offsets, tiles, vals, capacity, ranges, n_tiles, desc,
                     count_rows, ctl, spin_limit, never_publish);
}

namespace {

__global__ void materialize_keys_kernel(const uint32_t* __restrict__ tiles, const uint32_t* __restrict__ vals,
                                        const Splat* __restrict__ splats, uint32_t n,
                                        const uint32_t* __restrict__ tile_view, uint32_t n_tiles, uint32_t capacity,
                                        const FrameCtl* __restrict__ ctl, uint64_t* __restrict__ keys) {
    const uint32_t K = min(ctl->total_keys, capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
        const uint32_t t = tiles[i], g = vals[i];
        const uint32_t v = tile_view && t < n_tiles ? tile_view[t] : 0u;
        const uint32_t depth = g < n ? __float_as_uint(reinterpret_cast<const float4*>(splats + size_t(v) * n + g)[1].z)
                                     : 0xFFFFFFFFu;
        keys[i] = (uint64_t(t) << 32) | depth;
    }
}

}  // namespace

void launch_materialize_keys(const uint32_t* tiles, const uint32_t* vals, const Splat* splats, uint32_t n,
                             const uint32_t* tile_view, uint32_t n_tiles, uint32_t capacity, const FrameCtl* ctl,
                             uint64_t* keys, cudaStream_t s) {
    if (capacity == 0) return;
    const uint32_t blocks = std::min<uint32_t>((capacity + 255) / 256, 4096u);
    materialize_keys_kernel<<<blocks, 256, 0, s>>>(tiles, vals, splats, n, tile_view, n_tiles, capacity, ctl, keys);
}

}  // namespace tpd
