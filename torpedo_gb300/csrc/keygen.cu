// keygen.cu — kernel (b, second half): key duplication, and kernel (d): tile ranges.
//
// Reference: keygen.slang:23-53 (one thread per Gaussian looping over its tile
// rect) and range.slang:18-35 (+ fillBuffer, GaussianEngine.cpp:843-848).
//
// GB300 form of keygen: Gaussians are visited in depth order (a prior sort of
// the (view | depth) keys), so the emitted keys only need a stable sort on
// their tile-id bits afterwards: per tile the order is (depth, index), exactly
// the reference's stable sort of (tile | depth) keys emitted in index order.
// A warp owns 32 consecutive Gaussians and expands their keys cooperatively:
// lane s of each step writes output slot s of the warp's contiguous key range,
// finding its Gaussian by a 5-step shuffle search over the warp's exclusive
// offsets, so stores are fully coalesced and one large Gaussian no longer
// serialises its warp. Keys and values are bit-identical to the reference's.
#include "tpd_common.cuh"
#include "tpd_kernels.h"
#include "tpd_scan.cuh"

namespace tpd {
namespace {

constexpr uint32_t kKeygenThreads = 256;

constexpr uint32_t kNoDigit = 0x1000u;

// Adds 1 per lane to sh[d] for lanes with d != kNoDigit, one atomic per distinct digit.
__device__ __forceinline__ void warp_hist_add(uint32_t* sh, uint32_t d, uint32_t lane) {
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    if (d != kNoDigit && lane == uint32_t(__ffs(peers) - 1)) atomicAdd(&sh[d], uint32_t(__popc(peers)));
}

// Walks the (view, Gaussian) items in depth order (items[r] = v * n + i, their
// key offsets in offsets[r]); a warp owns 32 consecutive items, whose keys are
// contiguous. Besides the keys it counts the digits of the tile-id passes
// (digit positions 4.. of key_bits) into ctl->sort_hist; the low 32 bits of a
// key are its depth, already ordered, so no depth digit is counted or sorted.
__global__ void __launch_bounds__(kKeygenThreads)
    keygen_kernel(const Splat* __restrict__ splats, const uint32_t* __restrict__ items,
                  const uint32_t* __restrict__ offsets, uint32_t count, uint32_t n,
                  const ViewConst* __restrict__ views, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                  uint32_t capacity, uint32_t key_bits, FrameCtl* ctl) {
    __shared__ uint32_t sh[8][256];
    const uint32_t lane = lane_id();
    const uint32_t warps_total = (gridDim.x * blockDim.x) >> 5;
    const uint32_t warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0 && ctl->total_keys > capacity) atomicOr(&ctl->status, kStatusKeyOverflow);
    if (ctl->status & kStatusFatal) return;
    const uint32_t npass = min(8u, (key_bits + 7) / 8);
    for (uint32_t k = threadIdx.x; k < 8 * 256; k += blockDim.x) (&sh[0][0])[k] = 0;
    __syncthreads();
    auto digit_mask = [&](uint32_t p) { return (1u << min(8u, key_bits - 8 * p)) - 1u; };
    const uint32_t nwarps = (count + 31) / 32;

    for (uint32_t wi = warp_global; wi < nwarps; wi += warps_total) {
        const uint32_t r = wi * 32u + lane;
        // per item: its first tile (row-major in its view), rect width | view grid width << 16
        uint32_t x0 = 0, y0 = 0, x1 = 0, y1 = 0, off = 0, depth_bits = 0, gi = 0, t0 = 0, wgx = 1u | (1u << 16);
        if (r < count) {
            const uint32_t item = items[r];
            off = offsets[r];
            if (TPD_INBOUNDS(ctl, 21, item, count)) {
                const uint32_t v = item / n;
                gi = item - v * n;
                const ViewConst& vc = views[v];
                const uint32_t gx = grid_x(vc.width);
                const float4 texel = reinterpret_cast<const float4*>(splats + item)[1];  // px, py, viewZ, radius
                if (texel.w > 0.0f) {
                    bounding_rect(texel.x, texel.y, texel.w, gx, grid_y(vc.height), x0, y0, x1, y1);
                    depth_bits = __float_as_uint(texel.z);
                }
                t0 = vc.tile_base + y0 * gx + x0;
                wgx = max(x1 - x0, 1u) | (gx << 16);
            }
        }
        const uint32_t cnt = (x1 - x0) * (y1 - y0);
        const uint32_t incl = warp_inclusive_scan(cnt);
        const uint32_t excl = incl - cnt;
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        const uint32_t base = __shfl_sync(0xFFFFFFFFu, off, 0);
        for (uint32_t s0 = 0; s0 < total; s0 += 32u) {
            const uint32_t s = s0 + lane;
            // owner: the largest lane j with excl_j <= s
            uint32_t j = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1) {
                const uint32_t cand = j + step;
                const uint32_t e = __shfl_sync(0xFFFFFFFFu, excl, cand & 31u);
                if (cand < 32u && e <= s) j = cand;
            }
            const uint32_t jt0 = __shfl_sync(0xFFFFFFFFu, t0, j);
            const uint32_t jwg = __shfl_sync(0xFFFFFFFFu, wgx, j);
            const uint32_t jex = __shfl_sync(0xFFFFFFFFu, excl, j);
            const uint32_t jdb = __shfl_sync(0xFFFFFFFFu, depth_bits, j);
            const uint32_t jgi = __shfl_sync(0xFFFFFFFFu, gi, j);
            uint32_t tile = 0;
            // a key past the capacity is dropped and not counted, so the sort
            // of an overflowed frame still sees a consistent histogram
            const bool live = s < total && uint64_t(base) + s < capacity;
            if (live) {
                const uint32_t local = s - jex;  // < 2^24: exact in a float
                const uint32_t jw = jwg & 0xFFFFu, jgx = jwg >> 16;
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
                tile = jt0 + ty * jgx + uint32_t(rem);
                const uint64_t pos = uint64_t(base) + s;
                keys[pos] = (uint64_t(tile) << 32) | uint64_t(jdb);
                vals[pos] = jgi;
            }
            for (uint32_t p = 4; p < npass; ++p)
                warp_hist_add(sh[p], live ? ((tile >> (8 * (p - 4))) & digit_mask(p)) : kNoDigit, lane);
        }
    }
    __syncthreads();
    for (uint32_t p = 4; p < npass; ++p)
        for (uint32_t d = threadIdx.x; d < 256; d += blockDim.x)
            if (sh[p][d]) atomicAdd(&ctl->sort_hist[p][d], sh[p][d]);
}

// range.slang:18-35 over K = min(total_keys, capacity) keys; ranges zeroed first.
__global__ void tile_ranges_kernel(const uint64_t* __restrict__ keys, uint32_t* __restrict__ ranges,
                                   uint32_t n_tiles, FrameCtl* ctl, uint32_t capacity) {
    if (ctl->status & kStatusFatal) return;
    const uint32_t K = min(ctl->total_keys, capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < K; idx += stride) {
        if (!TPD_INBOUNDS(ctl, 30, idx, capacity)) continue;
        const uint32_t cur = uint32_t(keys[idx] >> 32);
        if (cur >= n_tiles) continue;  // only reachable with corrupted keys
        if (idx == 0) {
            ranges[cur * 2 + 0] = 0;
        } else {
            const uint32_t prev = uint32_t(keys[idx - 1] >> 32);
            if (cur != prev && TPD_INBOUNDS(ctl, 31, cur, n_tiles)) {
                if (prev < n_tiles) ranges[prev * 2 + 1] = idx;
                ranges[cur * 2 + 0] = idx;
            }
        }
        if (idx == K - 1) ranges[cur * 2 + 1] = idx + 1;
    }
}

}  // namespace

void launch_keygen(const Splat* splats, const uint32_t* items, const uint32_t* offsets, uint32_t count, uint32_t n,
                   const ViewConst* views, uint64_t* keys, uint32_t* vals, uint32_t capacity, uint32_t key_bits,
                   FrameCtl* ctl, int num_sms, cudaStream_t s) {
    if (count == 0 || n == 0) return;
    const uint64_t warps = (uint64_t(count) + 31) / 32;
    uint64_t blocks = (warps * 32 + kKeygenThreads - 1) / kKeygenThreads;
    const uint64_t cap = uint64_t(num_sms > 0 ? num_sms : 148) * 8;  // persistent: bounded histogram flushes
    blocks = blocks < cap ? blocks : cap;
    keygen_kernel<<<unsigned(blocks), kKeygenThreads, 0, s>>>(splats, items, offsets, count, n, views, keys, vals,
                                                              capacity, key_bits, ctl);
}

void launch_tile_ranges(const uint64_t* keys, uint32_t n_tiles, uint32_t* ranges, FrameCtl* ctl, uint32_t capacity,
                        int num_sms, cudaStream_t s) {
    cudaMemsetAsync(ranges, 0, size_t(n_tiles) * 8, s);
    const int blocks = (num_sms > 0 ? num_sms : 148) * 8;
    tile_ranges_kernel<<<blocks, 256, 0, s>>>(keys, ranges, n_tiles, ctl, capacity);
}

}  // namespace tpd
