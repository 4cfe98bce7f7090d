// keygen.cu — kernel (b, second half): key duplication.
//
// Reference: keygen.slang:23-53 (one thread per Gaussian looping over its tile
// rect). It also presets the tile ranges (fillBuffer, GaussianEngine.cpp:843-848)
// that the key sort's last pass fills in (range.slang:18-35, in sort.cu).
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

// Walks the ctl->depth_count (view, Gaussian) items the depth sort kept, in
// depth order (items[r] = v * n + i < n_items, their key offsets in
// offsets[r]); a warp owns 32 consecutive items, whose keys
// are contiguous, and produces them in windows of kKeyWindow output slots:
//  1. each lane with keys marks its first slot in the window's owner map,
//     a prefix-max over the map gives every slot its owning lane;
//  2. lane l fills slots l, l + 32, ...: owner's rectangle from a per-warp
//     table, (row, column) of the slot's index inside the rectangle, the key,
//     one coalesced store of key and value.
// A key is stored as its tile id alone: the low 32 bits of the reference's
// key are the depth, already in order (the items come in depth order), and
// the depth of a key is that of its value's splat, so the sort needs only the
// tile ids and the full keys can be rebuilt from (tile, value) when read.
// Keys past the capacity are not written (the frame is flagged and rendered
// again). The digit counts of the tile ids come from the preprocess, which
// counts each Gaussian's tile rectangle row by row.
constexpr uint32_t kKeyWindow = 256;
constexpr uint32_t kKeygenWarps = kKeygenThreads / 32;

struct KeygenSmem {
    uint32_t owner[kKeygenWarps][kKeyWindow];  // owning lane of each slot of the window
    uint32_t t0[kKeygenWarps][32];             // first tile of the lane's rectangle
    uint32_t wgx[kKeygenWarps][32];            // rectangle width | view grid width << 16
    uint32_t excl[kKeygenWarps][32];           // first slot of the lane's keys (warp-relative)
    uint32_t gi[kKeygenWarps][32];             // Gaussian index
};

__global__ void __launch_bounds__(kKeygenThreads)
    keygen_kernel(const Splat* __restrict__ splats, const uint32_t* __restrict__ items,
                  const uint32_t* __restrict__ items_other, const uint32_t* __restrict__ offsets, uint32_t n_items,
                  uint32_t n,
                  const ViewConst* __restrict__ views, uint32_t* __restrict__ tiles, uint32_t* __restrict__ vals,
                  uint32_t capacity, uint32_t key_bits, uint32_t* __restrict__ ranges, uint32_t n_tiles,
                  FrameCtl* ctl) {
    __shared__ KeygenSmem S;
    pdl_wait();     // launched as a dependent of the depth-order scan: its offsets are read below
    pdl_trigger();  // the key sort's first counting kernel may be scheduled (it waits for this grid)
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t warps_total = (gridDim.x * blockDim.x) >> 5;
    const uint32_t warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0 && ctl->total_keys > capacity) atomicOr(&ctl->status, kStatusKeyOverflow);
    if (ctl->status & kStatusFatal) return;
    const uint32_t count = min(ctl->depth_count, n_items);
    if (ctl->depth_skips & 1u) items = items_other;  // a skipped depth pass left the order there
    // ranges: (0xFFFFFFFF, 0) until the key sort's last pass narrows them
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_tiles; t += gridDim.x * blockDim.x)
        reinterpret_cast<uint2*>(ranges)[t] = make_uint2(0xFFFFFFFFu, 0u);
    uint32_t* owner = S.owner[warp];
    const uint32_t nwarps = (count + 31) / 32;

    // The item index, key offset and splat texel (px, py, viewZ, radius) of a
    // warp's next 32 items are loaded while it writes the keys of the current
    // ones: the texel is a gather in depth order.
    auto load_index = [&](uint32_t wi_, uint32_t& item, uint32_t& off) {
        const uint32_t r = wi_ * 32u + lane;
        item = 0xFFFFFFFFu;
        off = 0;
        if (wi_ < nwarps && r < count) {
            item = items[r];
            off = offsets[r];
        }
    };
    auto load_texel = [&](uint32_t item) {
        return item < n_items ? reinterpret_cast<const float4*>(splats + item)[1] : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    uint32_t item_c, off_c;
    load_index(warp_global, item_c, off_c);
    float4 texel_c = load_texel(item_c);

    for (uint32_t wi = warp_global; wi < nwarps; wi += warps_total) {
        uint32_t item_n, off_n;
        load_index(wi + warps_total, item_n, off_n);
        const uint32_t r = wi * 32u + lane;
        // per item: first tile (row-major in its view), rect width and height, view grid width
        uint32_t w = 1, h = 0, gx = 1, off = 0, gi = 0, t0 = 0;
        if (r < count) {
            const uint32_t item = item_c;
            off = off_c;
            if (TPD_INBOUNDS(ctl, 21, item, n_items)) {
                const uint32_t v = n_items == n ? 0u : item / n;  // one view: no division
                gi = item - v * n;
                const ViewConst& vc = views[v];
                gx = grid_x(vc.width);
                const float4 texel = texel_c;
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
        }
        const uint32_t cnt = w * h;
        const uint32_t incl = warp_inclusive_scan(cnt);
        const uint32_t excl = incl - cnt;
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        const uint32_t base = __shfl_sync(0xFFFFFFFFu, off, 0);
        S.t0[warp][lane] = t0;
        S.wgx[warp][lane] = w | (gx << 16);
        S.excl[warp][lane] = excl;
        S.gi[warp][lane] = gi;
        const float4 texel_n = load_texel(item_n);

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
                }
            }
            __syncwarp();  // the owner map is rebuilt for the next window
        }
        __syncwarp();  // the lane table is rewritten by the next items
        item_c = item_n;
        off_c = off_n;
        texel_c = texel_n;
    }
}

int keygen_setup() {
    int r = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, keygen_kernel, kKeygenThreads, 0);
    return r > 0 ? r : 1;
}

}  // namespace

void launch_keygen(const Splat* splats, const uint32_t* items, const uint32_t* items_other, const uint32_t* offsets,
                   uint32_t n_items, uint32_t n,
                   const ViewConst* views, uint32_t* tiles, uint32_t* vals, uint32_t capacity, uint32_t key_bits,
                   uint32_t* ranges, uint32_t n_tiles, FrameCtl* ctl, int num_sms, cudaStream_t s) {
    if (n_items == 0 || n == 0) return;
    const uint64_t warps = (uint64_t(n_items) + 31) / 32;
    uint64_t blocks = (warps * 32 + kKeygenThreads - 1) / kKeygenThreads;
    const int per_sm = device_once(keygen_setup);  // resident CTAs per SM (shared memory bound)
    const uint64_t cap = uint64_t(num_sms > 0 ? num_sms : 148) * uint64_t(per_sm);  // persistent
    blocks = blocks < cap ? blocks : cap;
    launch_dependent(keygen_kernel, dim3(unsigned(blocks)), dim3(kKeygenThreads), 0, s, splats, items, items_other,
                     offsets, n_items, n, views, tiles, vals, capacity, key_bits, ranges, n_tiles, ctl);
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
