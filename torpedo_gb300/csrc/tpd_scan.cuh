// tpd_scan.cuh — warp scans and the decoupled look-back used by the tile-count
// scan (prefix.slang) and the radix sort (radix-prefixA/B.slang).
//
// The reference runs its look-back on one thread per workgroup with an
// unbounded spin (prefix.slang:100-114). Here one warp inspects 32
// predecessors per step, descriptors carry a launch tag so they never need
// clearing, and every spin has an iteration limit after which the kernel sets
// kStatusLookbackTimeout, treats the missing prefix as 0 and publishes anyway
// (so successors do not wait in turn).
#pragma once
#include "tpd_common.cuh"

namespace tpd {

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v) {
    const uint32_t lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= uint32_t(o)) v += t;
    }
    return v;
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Called by all 32 lanes of one warp. Publishes `aggregate` for partition
// `part`, resolves the exclusive prefix from predecessors and publishes the
// inclusive prefix. `never_publish` (test hook) makes partition 0 skip its
// publication so that successors exercise the bounded spin.
__device__ __forceinline__ uint32_t warp_lookback(uint64_t* desc, uint32_t part, uint32_t aggregate,
                                                  uint32_t tag, uint32_t* status, uint32_t spin_limit,
                                                  bool never_publish = false) {
    const uint32_t lane = lane_id();
    const bool publish = !(never_publish && part == 0);
    if (lane == 0 && publish)
        st_relaxed_u64(&desc[part], make_desc(part == 0 ? kFlagPrefix : kFlagAggregate, tag, aggregate));
    uint32_t excl = 0;
    if (part > 0) {
        int64_t end = part;
        uint32_t spins = 0;
        while (true) {
            const int64_t idx = end - 1 - int64_t(lane);
            uint32_t flag = kFlagPrefix, val = 0;
            if (idx >= 0) {
                const uint64_t d = ld_relaxed_u64(&desc[idx]);
                flag = desc_flag(d, tag);
                val = uint32_t(d);
            }
            const uint32_t pmask = __ballot_sync(0xFFFFFFFFu, flag == kFlagPrefix);
            const uint32_t xmask = __ballot_sync(0xFFFFFFFFu, flag == 0u);
            const uint32_t first_p = pmask ? uint32_t(__ffs(pmask) - 1) : 32u;
            const uint32_t before = first_p >= 32 ? 0xFFFFFFFFu : ((1u << first_p) - 1u);
            if (xmask & before) {
                if (++spins > spin_limit) {
                    if (lane == 0) atomicOr(status, kStatusLookbackTimeout);
                    break;
                }
                __nanosleep(64);
                continue;
            }
            const uint32_t take = first_p >= 32 ? 0xFFFFFFFFu : ((2u << first_p) - 1u);
            excl += warp_sum(((take >> lane) & 1u) ? val : 0u);
            if (first_p < 32) break;
            end -= 32;
        }
        if (lane == 0 && publish) st_relaxed_u64(&desc[part], make_desc(kFlagPrefix, tag, excl + aggregate));
    }
    return __shfl_sync(0xFFFFFFFFu, excl, 0);
}

}  // namespace tpd
