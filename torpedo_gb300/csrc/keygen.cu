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
// A warp owns 32 consecutive Gaussians and builds their (contiguous) keys in
// a shared-memory window: small Gaussians one lane each, large ones by the
// whole warp, so one large Gaussian does not serialise its warp; each window
// is stored coalesced. Keys and values are bit-identical to the reference's.
#include "tpd_common.cuh"
#include "tpd_kernels.h"
#include "tpd_scan.cuh"

namespace tpd {
namespace {

constexpr uint32_t kKeygenThreads = 256;

// Walks the (view, Gaussian) items in depth order (items[r] = v * n + i, their
// key offsets in offsets[r]); a warp owns 32 consecutive items, whose keys
// are contiguous. The warp builds its keys in windows of kKeyWindow slots of
// shared memory and copies each window out coalesced:
//  - a Gaussian with at most kSmallKeys keys is expanded by its own lane,
//    stepping through its rectangle row-major without any division;
//  - a larger one is expanded by the whole warp, one slot per lane.
// Besides the keys it counts the digits of the tile-id passes (digit
// positions 4.. of key_bits) into ctl->sort_hist, one shared-memory atomic
// per key and pass (the lanes of a step work on different Gaussians, so they
// rarely collide); the low 32 bits of a key are its depth, already ordered,
// so no depth digit is counted or sorted. Keys past the capacity are neither
// written nor counted.
constexpr uint32_t kKeyWindow = 256;
constexpr uint32_t kSmallKeys = 32;
constexpr uint32_t kKeygenWarps = kKeygenThreads / 32;

struct KeygenSmem {
    uint64_t keys[kKeygenWarps][kKeyWindow];
    uint32_t vals[kKeygenWarps][kKeyWindow];
    uint32_t hist[4][256];  // tile-id digit positions 4..7
};

__device__ __forceinline__ void count_tile(KeygenSmem& S, uint32_t tile, uint32_t npass, uint32_t key_bits) {
    for (uint32_t p = 4; p < npass; ++p) {
        const uint32_t mask = (1u << min(8u, key_bits - 8u * p)) - 1u;
        atomicAdd(&S.hist[p - 4][(tile >> (8u * (p - 4))) & mask], 1u);
    }
}

__global__ void __launch_bounds__(kKeygenThreads)
    keygen_kernel(const Splat* __restrict__ splats, const uint32_t* __restrict__ items,
                  const uint32_t* __restrict__ offsets, uint32_t count, uint32_t n,
                  const ViewConst* __restrict__ views, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                  uint32_t capacity, uint32_t key_bits, uint32_t* __restrict__ ranges, uint32_t n_tiles,
                  FrameCtl* ctl) {
    __shared__ KeygenSmem S;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t warps_total = (gridDim.x * blockDim.x) >> 5;
    const uint32_t warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0 && ctl->total_keys > capacity) atomicOr(&ctl->status, kStatusKeyOverflow);
    if (ctl->status & kStatusFatal) return;
    const uint32_t npass = min(8u, (key_bits + 7) / 8);
    // ranges: (0xFFFFFFFF, 0) until the key sort's last pass narrows them
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_tiles; t += gridDim.x * blockDim.x)
        reinterpret_cast<uint2*>(ranges)[t] = make_uint2(0xFFFFFFFFu, 0u);
    for (uint32_t k = threadIdx.x; k < 4 * 256; k += blockDim.x) (&S.hist[0][0])[k] = 0;
    __syncthreads();
    uint64_t* wkeys = S.keys[warp];
    uint32_t* wvals = S.vals[warp];
    const uint32_t nwarps = (count + 31) / 32;

    for (uint32_t wi = warp_global; wi < nwarps; wi += warps_total) {
        const uint32_t r = wi * 32u + lane;
        // per item: first tile (row-major in its view), rect width, view grid width
        uint32_t w = 1, h = 0, gx = 1, off = 0, depth_bits = 0, gi = 0, t0 = 0;
        if (r < count) {
            const uint32_t item = items[r];
            off = offsets[r];
            if (TPD_INBOUNDS(ctl, 21, item, count)) {
                const uint32_t v = item / n;
                gi = item - v * n;
                const ViewConst& vc = views[v];
                gx = grid_x(vc.width);
                const float4 texel = reinterpret_cast<const float4*>(splats + item)[1];  // px, py, viewZ, radius
                if (texel.w > 0.0f) {
                    uint32_t x0, y0, x1, y1;
                    bounding_rect(texel.x, texel.y, texel.w, gx, grid_y(vc.height), x0, y0, x1, y1);
                    depth_bits = __float_as_uint(texel.z);
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
        const uint32_t big_lanes = __ballot_sync(0xFFFFFFFFu, cnt > kSmallKeys);

        for (uint32_t c0 = 0; c0 < total; c0 += kKeyWindow) {
            const uint32_t c1 = min(total, c0 + kKeyWindow);
            // small Gaussians: each lane writes its own slots of the window
            if (cnt <= kSmallKeys) {
                const uint32_t lo = max(excl, c0), hi = min(excl + cnt, c1);
                if (lo < hi) {
                    const uint32_t local = lo - excl;
                    uint32_t ty = local / w, tx = local - ty * w;
                    uint32_t tile = t0 + ty * gx + tx;
                    for (uint32_t k = lo; k < hi; ++k) {
                        wkeys[k - c0] = (uint64_t(tile) << 32) | depth_bits;
                        wvals[k - c0] = gi;
                        if (uint64_t(base) + k < capacity) count_tile(S, tile, npass, key_bits);
                        if (++tx == w) {  // next row of the rectangle
                            tx = 0;
                            tile += gx - w + 1;
                        } else {
                            ++tile;
                        }
                    }
                }
            }
            // large Gaussians: the whole warp, one slot per lane
            for (uint32_t bm = big_lanes; bm; bm &= bm - 1u) {
                const uint32_t j = uint32_t(__ffs(bm) - 1);
                const uint32_t jex = __shfl_sync(0xFFFFFFFFu, excl, j);
                const uint32_t jcnt = __shfl_sync(0xFFFFFFFFu, cnt, j);
                const uint32_t jt0 = __shfl_sync(0xFFFFFFFFu, t0, j);
                const uint32_t jw = __shfl_sync(0xFFFFFFFFu, w, j);
                const uint32_t jgx = __shfl_sync(0xFFFFFFFFu, gx, j);
                const uint32_t jdb = __shfl_sync(0xFFFFFFFFu, depth_bits, j);
                const uint32_t jgi = __shfl_sync(0xFFFFFFFFu, gi, j);
                const uint32_t lo = max(jex, c0), hi = min(jex + jcnt, c1);
                for (uint32_t k = lo + lane; k < hi; k += 32u) {
                    const uint32_t local = k - jex;
                    const uint32_t ty = local / jw;
                    const uint32_t tile = jt0 + ty * jgx + (local - ty * jw);
                    wkeys[k - c0] = (uint64_t(tile) << 32) | jdb;
                    wvals[k - c0] = jgi;
                    if (uint64_t(base) + k < capacity) count_tile(S, tile, npass, key_bits);
                }
            }
            __syncwarp();
            for (uint32_t q = lane; q < c1 - c0; q += 32u) {
                const uint64_t pos = uint64_t(base) + c0 + q;
                if (pos < capacity) {
                    keys[pos] = wkeys[q];
                    vals[pos] = wvals[q];
                }
            }
            __syncwarp();  // the window is refilled next
        }
    }
    __syncthreads();
    for (uint32_t p = 4; p < npass; ++p)
        for (uint32_t d = threadIdx.x; d < 256; d += blockDim.x)
            if (S.hist[p - 4][d]) atomicAdd(&ctl->sort_hist[p][d], S.hist[p - 4][d]);
}

}  // namespace

void launch_keygen(const Splat* splats, const uint32_t* items, const uint32_t* offsets, uint32_t count, uint32_t n,
                   const ViewConst* views, uint64_t* keys, uint32_t* vals, uint32_t capacity, uint32_t key_bits,
                   uint32_t* ranges, uint32_t n_tiles, FrameCtl* ctl, int num_sms, cudaStream_t s) {
    if (count == 0 || n == 0) return;
    const uint64_t warps = (uint64_t(count) + 31) / 32;
    uint64_t blocks = (warps * 32 + kKeygenThreads - 1) / kKeygenThreads;
    static int per_sm = 0;  // resident CTAs per SM (shared memory bound)
    if (per_sm == 0) {
        int r = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, keygen_kernel, kKeygenThreads, 0);
        per_sm = r > 0 ? r : 1;
    }
    const uint64_t cap = uint64_t(num_sms > 0 ? num_sms : 148) * uint64_t(per_sm);  // persistent
    blocks = blocks < cap ? blocks : cap;
    keygen_kernel<<<unsigned(blocks), kKeygenThreads, 0, s>>>(splats, items, offsets, count, n, views, keys, vals,
                                                              capacity, key_bits, ranges, n_tiles, ctl);
}


}  // namespace tpd
