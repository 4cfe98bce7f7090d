// sort.cu — kernel (c): stable LSD radix sort of (u64 or u32 key, u32 value) pairs.
//
// Reference: the 4-way (2-bit digit) LSD sort of radix-shuffle.slang:39-151,
// radix-prefixA.slang:39-170, radix-prefixB.slang:39-169 and
// radix-mapping.slang:40-117, driven by GaussianEngine.cpp:820-841 with
// P = ceil((msb(tiles) + 32) / 2) passes (GaussianEngine.cpp:351-357): four
// dispatches per pass, 21-24 passes per frame.
//
// GB300 form (onesweep): 8-bit digits, so a 45-bit (tile | depth) key takes 6
// passes instead of 23.
//  1. In the frame the digit histograms come from earlier kernels: the
//     preprocess counts the depth keys' digits and the tile ids' digits (from
//     each Gaussian's tile rectangle); sort_histogram_kernel builds them for
//     standalone sorts (one read of the keys, warp match-any aggregation into
//     shared memory, one global atomic per bin per CTA).
//  2. onesweep_kernel, once per pass: a persistent CTA takes 4096-key
//     partitions by atomic ticket, loads them with coalesced warp-striped
//     loads, ranks keys per warp (bit ballots, or match-any in the 512-thread
//     variant; stable within the warp-striped order), combines warps per
//     digit, publishes its digit counts, reorders the partition in shared
//     memory while predecessors publish, resolves each digit's global prefix
//     by a decoupled look-back (one thread per digit, four predecessors per
//     round trip, bounded spin) and writes digit runs out coalesced.
//  3. Counted passes (the frame's key sort, below): a counting kernel, then a
//     scatter kernel per pass, with every partition's digit offsets known
//     before it scatters, so no partition waits on another.
// In the frame the depth presort sorts 64-bit (view | depth) keys with
// onesweep passes and the key sort 32-bit tile ids (their depth order is
// already fixed) with counted passes; the standalone sort takes 64-bit keys
// (onesweep, 256 threads x 16 keys).
// The result is the stable sort of the pairs by the low key_bits bits, the
// same permutation as the reference's sort.
#include <algorithm>
#include <type_traits>

#include "tpd_common.cuh"
#include "tpd_kernels.h"
#include "tpd_scan.cuh"

namespace tpd {
namespace {

constexpr uint32_t kRadixBits = 8;
constexpr uint32_t kRadix = 1u << kRadixBits;
constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortWarps = kSortThreads / 32;
// Keys per thread of a radix pass: 16 (4096-key partitions) for large sorts;
// 8 or 4 give more, shorter partitions when the sort is too small to fill the
// GPU with 4096-key partitions (the depth sort of 1M Gaussians).
constexpr uint32_t kSortItemsMax = 16;
constexpr uint32_t kInvalidDigit = kRadix;                  // keys past K (and dropped keys)

// Pass kinds of onesweep_kernel. The depth sort compacts the culled items
// away in its first pass and sorts the remaining ctl->depth_count items in
// the others, where a pass whose digit is the same for every key is skipped
// (counted in ctl->depth_skips; the later passes swap their buffers).
constexpr int kPassPlain = 0;      // K = fixed_count, else ctl->total_keys
constexpr int kPassDropCulled = 1; // as plain; keys whose low 32 bits are 0xFFFFFFFF are not written
constexpr int kPassCompacted = 2;  // K = ctl->depth_count; a uniform digit skips the pass (ctl->depth_skips)

constexpr uint32_t kHistThreads = 256;
constexpr uint32_t kHistChunk = 2048;  // keys per grid-stride chunk of the histogram kernel

// Reorder buffers hold one pad slot per 16 keys: digit runs of about 16 keys
// (8-bit digits over a 4096-key partition) put the runs of consecutive digits
// 128 B apart, which without padding lands a warp's stores on one bank when
// its lanes carry consecutive digits (keys of one Gaussian's tile rectangle).
__device__ __forceinline__ uint32_t pad16(uint32_t i) { return i + (i >> 4); }

template <int kItems, int kThreads, typename KeyT>
struct OnesweepSmem {
    static constexpr uint32_t kTile = kThreads * kItems;
    KeyT keys[kTile + kTile / 16];
    uint32_t vals[kTile + kTile / 16];
    uint32_t whist[kThreads / 32][kRadix];
    uint32_t gdig[kRadix];    // global exclusive digit offsets of this pass
    uint32_t lstart[kRadix];  // block-local digit start
    uint32_t gmap[kRadix];    // global position of local index 0 of each digit
    uint32_t wsum[kThreads / 32];
    uint32_t part;
    uint32_t valid;  // keys of the partition that are written (all but dropped ones)
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Block-wide exclusive scan of one value per thread (kWarps warps); returns the exclusive prefix.
template <uint32_t kWarps = kSortWarps>
__device__ __forceinline__ uint32_t block_exclusive_scan256(uint32_t v, uint32_t* wsum) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t incl = warp_inclusive_scan(v);
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t base = 0;
#pragma unroll
    for (uint32_t w = 0; w < kWarps; ++w)
        if (w < warp) base += wsum[w];
    __syncthreads();
    return base + incl - v;
}

__global__ void sort_begin_kernel(FrameCtl* ctl, uint32_t total) {
    const uint32_t t = threadIdx.x;
    for (uint32_t i = t; i < 32; i += blockDim.x) ctl->ticket[i] = 0;
    for (uint32_t i = t; i < 8 * 256; i += blockDim.x) {
        (&ctl->sort_hist[0][0])[i] = 0;
        (&ctl->depth_hist[0][0])[i] = 0;
    }
    if (t == 0) {
        ctl->tag = ctl->tag + 1;
        ctl->status = 0;
        ctl->total_keys = total;
    }
}

__device__ __forceinline__ void hist_add(uint32_t* h, uint32_t d) {
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    const uint32_t leader = __ffs(peers) - 1;
    if ((threadIdx.x & 31u) == leader && d < kRadix) atomicAdd(&h[d], __popc(peers));
}

template <typename KeyT>
__global__ void __launch_bounds__(kHistThreads)
    sort_histogram_kernel(const KeyT* __restrict__ keys, uint32_t capacity, uint32_t p0, uint32_t p1,
                          uint32_t key_bits, uint32_t (*hist)[256], FrameCtl* ctl) {
    __shared__ uint32_t sh[8][kRadix];
    // launched as a dependent of the stream's previous kernel: its output is
    // read below. No early trigger: the next kernel is one wave of CTAs, which
    // must be placed on empty SMs, not onto the first ones this grid frees
    pdl_wait();
    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < 8 * kRadix; i += kHistThreads) (&sh[0][0])[i] = 0;
    __syncthreads();
    const uint32_t K = (ctl->status & kStatusFatal) ? 0u : min(ctl->total_keys, capacity);
    uint32_t shift[8], mask[8];
#pragma unroll
    for (uint32_t p = 0; p < 8; ++p) {
        shift[p] = p * kRadixBits;
        const uint32_t b = (p * kRadixBits < key_bits) ? min(kRadixBits, key_bits - p * kRadixBits) : 0u;
        mask[p] = (1u << b) - 1u;
    }
    // grid-stride over chunks of kHistChunk keys; the trip count is uniform per CTA
    const uint32_t nchunks = (K + kHistChunk - 1) / kHistChunk;
    for (uint32_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint32_t base = c * kHistChunk;
#pragma unroll 2
        for (uint32_t j = tid; j < kHistChunk; j += kHistThreads) {
            const uint32_t idx = base + j;
            const bool v = idx < K;
            const uint64_t k = v ? uint64_t(keys[idx]) : 0ull;
            for (uint32_t p = p0; p < p1; ++p)
                hist_add(sh[p], v ? (uint32_t(k >> shift[p]) & mask[p]) : kInvalidDigit);
        }
    }
    __syncthreads();
    for (uint32_t p = p0; p < p1; ++p)
        for (uint32_t d = tid; d < kRadix; d += kHistThreads)
            if (sh[p][d]) atomicAdd(&hist[p][d], sh[p][d]);
}

// Resolves the exclusive prefix of one digit for partition `part` by walking
// predecessors; up to kLookbackWindow descriptors are loaded per round trip
// (8 measured the same, 16 slower: the extra registers spill).
constexpr int kLookbackWindow = 4;
__device__ __forceinline__ uint32_t digit_lookback(const uint64_t* __restrict__ desc, uint32_t part, uint32_t digit,
                                                   uint32_t tag, FrameCtl* ctl, uint32_t spin_limit) {
    constexpr int W = kLookbackWindow;
    uint32_t excl = 0;
    int64_t p = int64_t(part) - 1;
    uint32_t spins = 0;
    while (p >= 0) {
        uint64_t d[W];
        const int cnt = p >= W - 1 ? W : int(p) + 1;
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (j < cnt) d[j] = ld_relaxed_u64(desc + size_t(p - j) * kRadix + digit);  // 0 <= p - j < part
        bool stop = false, wait = false;
#pragma unroll
        for (int j = 0; j < W; ++j) {
            if (j >= cnt || stop || wait) continue;
            const uint32_t f = desc_flag(d[j], tag);
            if (f == 0u) {
                wait = true;  // not yet published: retry from here
            } else {
                excl += uint32_t(d[j]);
                --p;
                if (f == uint32_t(kFlagPrefix)) stop = true;
            }
        }
        if (stop) break;
        if (wait) {
            if (++spins > spin_limit) {
                atomicOr(&ctl->status, kStatusLookbackTimeout);
                break;
            }
            __nanosleep(32);
        }
    }
    return excl;
}

// Tile ranges (range.slang:18-35) from the last pass of the key sort: the
// partition's keys sit in shared memory fully sorted within each digit run,
// and a digit run is contiguous in the output. A tile starts where the run's
// previous key has another tile and ends where the next one has; at the
// edges of a run the neighbour lies in another partition, and min / max
// reductions over all candidates give the range whatever the order.
// A key's tile id: the high 32 bits of a (tile | depth) key, or the whole of
// a 32-bit tile-id key.
__device__ __forceinline__ uint32_t tile_of(uint64_t key) { return uint32_t(key >> 32); }
__device__ __forceinline__ uint32_t tile_of(uint32_t key) { return key; }

template <int kItems, int kThreads, typename KeyT>
__device__ __forceinline__ void tile_range_bounds(const OnesweepSmem<kItems, kThreads, KeyT>& S, uint32_t* ranges,
                                                  uint32_t n_tiles, KeyT key, uint32_t j, uint32_t cnt,
                                                  uint32_t d, uint32_t g, uint32_t shift, uint32_t mask,
                                                  FrameCtl* ctl) {
    const uint32_t t = tile_of(key);
    if (!TPD_INBOUNDS(ctl, 18, t, n_tiles)) return;
    bool first = j == 0, last = j + 1 == cnt;
    if (!first) {
        const KeyT kp = S.keys[pad16(j - 1)];
        first = (uint32_t(kp >> shift) & mask) != d || tile_of(kp) != t;
    }
    if (!last) {
        const KeyT kn = S.keys[pad16(j + 1)];
        last = (uint32_t(kn >> shift) & mask) != d || tile_of(kn) != t;
    }
    if (first) atomicMin(&ranges[2 * t], g);
    if (last) atomicMax(&ranges[2 * t + 1], g + 1);
}

// kThreads = 256 (one digit per thread) or 512 (the digit-wide steps run on
// the first 256 threads); a partition is kThreads * kItems keys. kPass is a
// pass kind (kPassPlain ...): dropped keys are ranked as past-the-end keys.
// KeyT is uint64_t ((tile | depth) or (view | depth) keys) or uint32_t (tile
// ids, whose depth order the depth presort has already fixed).
template <int kItems, int kThreads, int kMinBlocks, int kPass, typename KeyT>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    onesweep_kernel(const KeyT* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                    KeyT* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t capacity,
                    uint32_t pass, uint32_t shift, uint32_t bits, const uint32_t (*hist)[256], uint32_t ticket_slot,
                    uint32_t tag_slot, uint32_t fixed_count, uint64_t* __restrict__ desc, FrameCtl* ctl,
                    uint32_t spin_limit, uint32_t* __restrict__ ranges, uint32_t n_tiles, uint32_t abort_mask) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr uint32_t kSortItems = kItems, kSortTile = kThreads * kItems, kWarps = kThreads / 32;
    // launched as a dependent of the stream's previous kernel: its output is
    // read below. No early trigger: the next kernel is one wave of CTAs, which
    // must be placed on empty SMs, not onto the first ones this grid frees
    pdl_wait();
    // digits ranked with match-any in the 512-thread variant (32 warps per SM
    // hide its latency), with bit ballots otherwise (fixed cost)
    constexpr bool kMatchRank = kThreads == 512;
    OnesweepSmem<kItems, kThreads, KeyT>& S = *reinterpret_cast<OnesweepSmem<kItems, kThreads, KeyT>*>(smem_raw);
    const bool digit_thread = threadIdx.x < kRadix;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    constexpr bool kDrop = kPass == kPassDropCulled;
    static_assert(kPass == kPassPlain || sizeof(KeyT) == 8, "depth-sort pass kinds take 64-bit keys");
    const uint32_t K = (ctl->status & abort_mask)
                           ? 0u
                           : min(kPass == kPassCompacted ? ctl->depth_count
                                                         : (fixed_count ? fixed_count : ctl->total_keys),
                                 capacity);
    if constexpr (kPass == kPassCompacted) {
        if (ctl->depth_skips & 1u) {  // an earlier pass was skipped: its input buffer holds the order
            KeyT* const k = const_cast<KeyT*>(keys_in);
            keys_in = keys_out;
            keys_out = k;
            uint32_t* const v = const_cast<uint32_t*>(vals_in);
            vals_in = vals_out;
            vals_out = v;
        }
    }
    const uint32_t nparts = (K + kSortTile - 1) / kSortTile;
    const uint32_t tag = ctl->tag * 32u + tag_slot;
    const uint32_t mask = (1u << bits) - 1u;
    // digits of this pass's width: only these count, publish and look back
    // (a 5-bit pass leaves 224 of the 256 digit threads idle)
    const bool live_digit = tid <= mask;

    // global exclusive digit offsets (histogram of this pass, scanned)
    const uint32_t h = digit_thread && TPD_INBOUNDS(ctl, 16, pass, 8) ? hist[pass][tid] : 0u;
    {
        const uint32_t ex = block_exclusive_scan256<kWarps>(h, S.wsum);
        if (digit_thread) S.gdig[tid] = ex;
    }
    if constexpr (kPass == kPassCompacted) {
        // a pass whose digit is the same for all K keys leaves their order as
        // it is: it is skipped and counted, and the order stays in its input
        // buffer (every CTA takes the same decision from the same histogram)
        if (__syncthreads_or(digit_thread && K > 0 && h == K)) {
            if (blockIdx.x == 0 && tid == 0) atomicAdd(&ctl->depth_skips, 1u);
            return;
        }
    }

    // Warp-striped items, loaded coalesced straight from global memory: warp w
    // owns [w*32*kItems, (w+1)*32*kItems), item i covers 32 consecutive keys.
    // Variants with registers to spare load the values with the keys. The
    // 256-thread variants load a CTA's next partition while they write out the
    // current one (thread 0 takes its ticket after its look-back), hiding the
    // load latency behind the write-out; the 512-thread variant, at 64
    // registers, takes its ticket and loads at the top of each partition.
    constexpr bool kValsEarly = kItems * kMinBlocks * (kThreads / 256) <= 32;
    constexpr bool kPrefetch = kThreads == 256;
    KeyT k[kSortItems];
    uint32_t vr[kValsEarly ? kSortItems : 1];
    auto load_partition = [&](uint32_t p) {
        const uint32_t b = p * kSortTile, c = p < nparts ? min(kSortTile, K - b) : 0u;
#pragma unroll
        for (uint32_t i = 0; i < kSortItems; ++i) {
            const uint32_t idx = warp * (kSortItems * 32) + i * 32 + lane;
            k[i] = idx < c ? keys_in[b + idx] : KeyT(~KeyT(0));
            if constexpr (kValsEarly) vr[i] = idx < c ? vals_in[b + idx] : 0u;
        }
    };
    uint32_t part = 0;
    if constexpr (kPrefetch) {
        if (tid == 0) S.part = atomicAdd(&ctl->ticket[ticket_slot], 1u);
        __syncthreads();
        part = S.part;
        load_partition(part);
    }

    while (true) {
        if constexpr (!kPrefetch) {
            if (tid == 0) S.part = atomicAdd(&ctl->ticket[ticket_slot], 1u);
        }
#pragma unroll
        for (uint32_t i = tid; i < kWarps * kRadix; i += kThreads) (&S.whist[0][0])[i] = 0;
        __syncthreads();
        if constexpr (!kPrefetch) part = S.part;
        if (part >= nparts) break;
        if constexpr (!kPrefetch) load_partition(part);
        const uint32_t base = part * kSortTile;
        const uint32_t cnt = min(kSortTile, K - base);

        // dr[i] packs the digit (bits 0..8, kInvalidDigit past K) and the
        // key's rank among equal digits earlier in the warp (bits 9..31).
        uint32_t dr[kSortItems];
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (uint32_t i = 0; i < kSortItems; ++i) {
            const uint32_t idx = warp * (kSortItems * 32) + i * 32 + lane;
            const uint32_t d = idx < cnt && !(kDrop && uint32_t(k[i]) == 0xFFFFFFFFu) ? (uint32_t(k[i] >> shift) & mask)
                                                                                     : kInvalidDigit;
            uint32_t peers;
            if constexpr (kMatchRank) {
                peers = __match_any_sync(0xFFFFFFFFu, d);
            } else {
                // lanes with the same digit: one ballot per digit bit (bits
                // above the pass's width are zero in every valid lane and
                // leave the mask as it is), and one for the past-the-end (or
                // dropped) digit in the partitions that can have any
                peers = 0xFFFFFFFFu;
#pragma unroll
                for (uint32_t b = 0; b < kRadixBits; ++b) {
                    const bool on = (d >> b) & 1u;
                    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, on);
                    peers &= on ? bal : ~bal;
                }
                if (kDrop || cnt < kSortTile) {
                    const bool on = d >= kRadix;
                    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, on);
                    peers &= on ? bal : ~bal;
                }
            }
            const uint32_t leader = __ffs(peers) - 1;
            uint32_t prev = 0;
            if (lane == leader && d < kRadix) {
                prev = S.whist[warp][d];
                S.whist[warp][d] = prev + __popc(peers);
            }
            prev = __shfl_sync(0xFFFFFFFFu, prev, leader);
            dr[i] = d | ((prev + __popc(peers & lt)) << 9);
            __syncwarp();
        }
        __syncthreads();

        // per digit (thread = digit): warp prefixes, block count, local start
        uint32_t count = 0;
        uint64_t* dp = nullptr;
        if (live_digit) {
#pragma unroll
            for (uint32_t w = 0; w < kWarps; ++w) {
                const uint32_t c = S.whist[w][tid];
                S.whist[w][tid] = count;
                count += c;
            }
            dp = desc + size_t(TPD_INBOUNDS(ctl, 13, part, nparts) ? part : 0) * kRadix + tid;
            st_relaxed_u64(dp, make_desc(part == 0 ? kFlagPrefix : kFlagAggregate, tag, count));
        }
        const uint32_t lstart = block_exclusive_scan256<kWarps>(count, S.wsum);  // (its barriers cover whist)
        if (digit_thread) S.lstart[tid] = lstart;
        if (kDrop && tid == kRadix - 1) S.valid = lstart + count;
        __syncthreads();

        // reorder the partition in shared memory (stable: warp, then item, then
        // lane) while predecessors publish; values not held in registers are
        // loaded now, coalesced
        if constexpr (kValsEarly) {
            // key and value go to the same slot: one position per item
#pragma unroll
            for (uint32_t i = 0; i < kSortItems; ++i) {
                const uint32_t d = dr[i] & 511u;
                if (d < kRadix) {
                    const uint32_t pos = S.lstart[d] + S.whist[warp][d] + (dr[i] >> 9);
                    if (TPD_INBOUNDS(ctl, 11, pos, cnt)) {
                        S.keys[pad16(pos)] = k[i];
                        S.vals[pad16(pos)] = vr[i];
                    }
                }
            }
        } else {
#pragma unroll
            for (uint32_t i = 0; i < kSortItems; ++i) {
                const uint32_t d = dr[i] & 511u;
                if (d < kRadix) {
                    const uint32_t pos = S.lstart[d] + S.whist[warp][d] + (dr[i] >> 9);
                    if (TPD_INBOUNDS(ctl, 11, pos, cnt)) S.keys[pad16(pos)] = k[i];
                }
            }
#pragma unroll
            for (uint32_t i = 0; i < kSortItems; ++i) {
                const uint32_t idx = warp * (kSortItems * 32) + i * 32 + lane;
                const uint32_t d = dr[i] & 511u;
                if (d < kRadix) {
                    const uint32_t v = vals_in[base + idx];
                    const uint32_t pos = S.lstart[d] + S.whist[warp][d] + (dr[i] >> 9);
                    if (TPD_INBOUNDS(ctl, 12, pos, cnt)) S.vals[pad16(pos)] = v;
                }
            }
        }

        // decoupled look-back for this thread's digit; then (prefetching
        // variants) thread 0 takes the next partition's ticket: every thread
        // has read S.part since it was last written
        if (live_digit) {
            if (part > 0) {
                const uint32_t excl = digit_lookback(desc, part, tid, tag, ctl, spin_limit);
                st_relaxed_u64(dp, make_desc(kFlagPrefix, tag, excl + count));
                S.gmap[tid] = S.gdig[tid] + excl - lstart;
            } else {
                S.gmap[tid] = S.gdig[tid] - lstart;
            }
        }
        if constexpr (kPrefetch) {
            if (tid == 0) S.part = atomicAdd(&ctl->ticket[ticket_slot], 1u);
        }
        __syncthreads();
        if constexpr (kPrefetch) {
            part = S.part;
            load_partition(part);  // k and vr are free since the reorder
        }

        // coalesced write-out of digit runs
        const uint32_t cntv = kDrop ? S.valid : cnt;
        for (uint32_t j = tid; j < cntv; j += kThreads) {
            const KeyT key = S.keys[pad16(j)];
            const uint32_t d = uint32_t(key >> shift) & mask;
            const uint32_t g = S.gmap[d] + j;
            if (g < capacity && TPD_INBOUNDS(ctl, 17, g, K + (K == 0))) {
                keys_out[g] = key;
                vals_out[g] = S.vals[pad16(j)];
                if (ranges) tile_range_bounds(S, ranges, n_tiles, key, j, cntv, d, g, shift, mask, ctl);
            }
        }
        __syncthreads();  // S.keys / S.vals / S.gmap are rewritten by the next partition
    }
}

// ---- counted passes: a radix pass without look-back
//
// The look-back of onesweep_kernel puts a wait on every partition's critical
// path (measured on the key sort of 1M Gaussians at 1080p: 4.4 of 10.5 us per
// partition, after load and rank 3.0, scan 0.4, write-out 2.6). A counted pass
// computes every partition's digit offsets beforehand instead:
//  1. partition_count_kernel, one CTA per 4096-key partition: the partition's
//     digit counts (per-warp shared-memory counts) as a row of work[]. The
//     last CTA of each chunk of kChunkParts partitions to finish (an atomic
//     arrival count; nobody waits) scans the chunk's rows per digit in place
//     into offsets within the chunk and writes the chunk's totals; the last
//     chunk to finish scans the chunk totals, starting from the pass's global
//     digit offsets, into each chunk's base. Arrival counts are reset by the
//     CTA that finishes them, so the work area is zero at rest.
//  2. scatter_kernel, one CTA per partition: load, rank (bit ballots, stable
//     in warp-striped order), reorder in shared memory and write out at
//     chunk base + offset within chunk, as onesweep_kernel does but with its
//     offsets known: no partition waits for another.
// The permutation is the same stable one.
constexpr uint32_t kChunkParts = 32;

// Layout of a counted pass's work area (u32 words), for P partitions:
// [0, 256 P) rows of digit counts, then offsets within their chunk;
// [256 P, 256 P + 256 C) chunk totals, then chunk bases (C chunks);
// [256 (P + C), + C) chunk arrival counts; then one arrival count of chunks.
__host__ __device__ inline size_t counted_chunks(uint32_t parts) { return (parts + kChunkParts - 1) / kChunkParts; }
__host__ __device__ inline size_t counted_work_words(uint32_t parts) {
    const size_t c = counted_chunks(parts);
    return 256 * (size_t(parts) + c) + c + 1;
}

__device__ __forceinline__ uint32_t ld_cg_u32(const uint32_t* p) { return __ldcg(p); }

// Rows of the chunk's partitions [first, first + csize) -> offsets within the
// chunk, in place, and the chunk's total per digit into chunk_rows (thread =
// digit; the rows are loaded together, then scanned).
__device__ __forceinline__ void scan_chunk_rows(uint32_t* rows, uint32_t* chunk_rows, uint32_t chunk, uint32_t first,
                                                uint32_t csize, uint32_t tid) {
    uint32_t c[kChunkParts];
#pragma unroll
    for (uint32_t q = 0; q < kChunkParts; ++q)
        c[q] = q < csize ? ld_cg_u32(rows + size_t(first + q) * 256 + tid) : 0u;
    uint32_t run = 0;
#pragma unroll
    for (uint32_t q = 0; q < kChunkParts; ++q) {
        if (q < csize) rows[size_t(first + q) * 256 + tid] = run;
        run += c[q];
    }
    chunk_rows[size_t(chunk) * 256 + tid] = run;
}

// The last chunk: each chunk's total -> its base, from the pass's global digit
// offsets (the exclusive scan of hist_digit over digits). Called by the whole CTA.
__device__ __forceinline__ void scan_chunk_bases(uint32_t* chunk_rows, uint32_t nchunks, uint32_t hist_digit,
                                                 uint32_t* wsum, uint32_t tid) {
    uint32_t gbase = block_exclusive_scan256<8>(hist_digit, wsum);
    uint32_t c[kChunkParts];
    for (uint32_t c0 = 0; c0 < nchunks; c0 += kChunkParts) {  // chunk totals, kChunkParts at a time
#pragma unroll
        for (uint32_t q = 0; q < kChunkParts; ++q)
            c[q] = c0 + q < nchunks ? ld_cg_u32(chunk_rows + size_t(c0 + q) * 256 + tid) : 0u;
#pragma unroll
        for (uint32_t q = 0; q < kChunkParts; ++q) {
            if (c0 + q < nchunks) chunk_rows[size_t(c0 + q) * 256 + tid] = gbase;
            gbase += c[q];
        }
    }
}

template <int kItems, typename KeyT>
__global__ void __launch_bounds__(256) partition_count_kernel(const KeyT* __restrict__ keys, uint32_t capacity,
                                                              uint32_t pass, uint32_t shift, uint32_t bits,
                                                              const uint32_t (*hist)[256], uint32_t fixed_count,
                                                              uint32_t max_parts, uint32_t* __restrict__ work,
                                                              FrameCtl* ctl, uint32_t abort_mask) {
    constexpr uint32_t kTile = 256 * kItems;
    __shared__ uint32_t hw[8][kRadix];  // per-warp counts
    __shared__ uint32_t wsum[8];
    __shared__ bool last;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    // launched as a dependent of the kernel that wrote the keys: wait for it,
    // then let the scatter be scheduled (it loads its keys and values while
    // the last partitions are counted; they come from the kernel this one
    // waited for)
    pdl_wait();
    pdl_trigger();
    const uint32_t K = (ctl->status & abort_mask) ? 0u : min(fixed_count ? fixed_count : ctl->total_keys, capacity);
    const uint32_t nparts = min((K + kTile - 1) / kTile, max_parts);
    const uint32_t part = blockIdx.x;
    if (part >= nparts) return;  // (uniform)
    const uint32_t mask = (1u << bits) - 1u;
    const uint32_t base = part * kTile, cnt = min(kTile, K - base);
    KeyT k[kItems];
#pragma unroll
    for (uint32_t i = 0; i < kItems; ++i) {
        const uint32_t idx = i * 256 + tid;
        k[i] = idx < cnt ? keys[base + idx] : KeyT(0);
    }
    // (while the loads are in flight) each warp clears its own counts
#pragma unroll
    for (uint32_t j = 0; j < kRadix / 32; ++j) hw[warp][lane + 32 * j] = 0;
    __syncwarp();
    // 32 consecutive keys often share a digit (a Gaussian's row of tiles, in
    // the high digit): then one add of 32, else one shared atomic per key
#pragma unroll
    for (uint32_t i = 0; i < kItems; ++i) {
        const uint32_t idx = i * 256 + tid;
        const uint32_t d = idx < cnt ? (uint32_t(k[i] >> shift) & mask) : kInvalidDigit;
        const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, d, 0);
        if (__all_sync(0xFFFFFFFFu, d == d0)) {
            if (lane == 0 && d < kRadix) hw[warp][d] += 32u;
        } else if (d < kRadix) {
            atomicAdd(&hw[warp][d], 1u);
        }
    }
    __syncthreads();
    uint32_t total = 0;
#pragma unroll
    for (uint32_t w = 0; w < 8; ++w) total += hw[w][tid];
    uint32_t* rows = work;
    const uint32_t nchunks = uint32_t(counted_chunks(nparts));
    uint32_t* chunk_rows = work + 256 * size_t(max_parts);
    uint32_t* arrivals = chunk_rows + 256 * counted_chunks(max_parts);
    rows[size_t(part) * 256 + tid] = total;
    // the CTA's row is visible device-wide before its arrival is counted: the
    // barrier orders every thread's store before thread 0's fence, which
    // makes them visible with its own (a fence is cumulative); the last
    // arriver's fence after its count orders its reads after all rows
    __syncthreads();
    const uint32_t chunk = part / kChunkParts;
    const uint32_t first = chunk * kChunkParts, csize = min(kChunkParts, nparts - first);
    if (tid == 0) {
        __threadfence();
        last = atomicAdd(&arrivals[chunk], 1u) == csize - 1u;
        if (last) __threadfence();
    }
    __syncthreads();
    if (!last) return;
    // the chunk's last CTA: offsets within the chunk, in place, and its total
    scan_chunk_rows(rows, chunk_rows, chunk, first, csize, tid);
    __syncthreads();
    if (tid == 0) {
        arrivals[chunk] = 0;
        __threadfence();
        last = atomicAdd(&arrivals[counted_chunks(max_parts)], 1u) == nchunks - 1u;
        if (last) __threadfence();
    }
    __syncthreads();
    if (!last) return;
    // the last chunk: each chunk's base, from the pass's global digit offsets
    scan_chunk_bases(chunk_rows, nchunks, TPD_INBOUNDS(ctl, 19, pass, 8) ? hist[pass][tid] : 0u, wsum, tid);
    if (tid == 0) arrivals[counted_chunks(max_parts)] = 0;
}

// The first pass of a sort whose partition rows were counted by the kernel
// that wrote the keys (keygen_scan_kernel adds each partition's digit counts
// into rows[] with atomics, on rows that were zero): no keys are read. One
// CTA per chunk of kChunkParts partitions scans its rows in place and writes
// the chunk's totals; the last chunk to finish (an arrival count, reset by
// it) scans the chunk totals into chunk bases, as partition_count_kernel's
// last arrivers do.
__global__ void __launch_bounds__(256) chunk_scan_kernel(uint32_t capacity, uint32_t pass,
                                                         const uint32_t (*hist)[256], uint32_t fixed_count,
                                                         uint32_t max_parts, uint32_t* __restrict__ work,
                                                         FrameCtl* ctl, uint32_t abort_mask) {
    __shared__ uint32_t wsum[8];
    __shared__ bool last;
    const uint32_t tid = threadIdx.x;
    pdl_wait();     // the rows come from the kernel before this one
    pdl_trigger();  // the scatter may be scheduled; it waits for this grid
    const uint32_t K = (ctl->status & abort_mask) ? 0u : min(fixed_count ? fixed_count : ctl->total_keys, capacity);
    const uint32_t nparts = min((K + 4095u) / 4096u, max_parts);
    const uint32_t nchunks = uint32_t(counted_chunks(nparts));
    const uint32_t chunk = blockIdx.x;
    if (chunk >= nchunks) return;  // (uniform)
    uint32_t* rows = work;
    uint32_t* chunk_rows = work + 256 * size_t(max_parts);
    uint32_t* arrivals = chunk_rows + 256 * counted_chunks(max_parts);
    const uint32_t first = chunk * kChunkParts, csize = min(kChunkParts, nparts - first);
    scan_chunk_rows(rows, chunk_rows, chunk, first, csize, tid);
    // the chunk totals are visible device-wide before the arrival is counted
    // (barrier, then thread 0's cumulative fence); the last arriver's fence
    // after its count orders its reads after every chunk's totals
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        last = atomicAdd(&arrivals[counted_chunks(max_parts)], 1u) == nchunks - 1u;
        if (last) __threadfence();
    }
    __syncthreads();
    if (!last) return;
    scan_chunk_bases(chunk_rows, nchunks, TPD_INBOUNDS(ctl, 19, pass, 8) ? hist[pass][tid] : 0u, wsum, tid);
    if (tid == 0) arrivals[counted_chunks(max_parts)] = 0;
}

// kBits: the pass's digit width (1..8); the lanes with the same digit are
// found with one ballot per digit bit (the launch picks the variant of the
// pass's width: a 5-bit pass ranks with 5 ballots, not 8).
template <int kItems, int kThreads, int kMinBlocks, int kBits, typename KeyT>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    scatter_kernel(const KeyT* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, KeyT* __restrict__ keys_out,
                   uint32_t* __restrict__ vals_out, uint32_t capacity, uint32_t shift, uint32_t bits,
                   uint32_t fixed_count, uint32_t max_parts, const uint32_t* __restrict__ work, FrameCtl* ctl,
                   uint32_t* __restrict__ ranges, uint32_t n_tiles, uint32_t abort_mask) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr uint32_t kSortTile = kThreads * kItems, kWarps = kThreads / 32;
    OnesweepSmem<kItems, kThreads, KeyT>& S = *reinterpret_cast<OnesweepSmem<kItems, kThreads, KeyT>*>(smem_raw);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const bool digit_thread = tid < kRadix;
    const uint32_t K = (ctl->status & abort_mask) ? 0u : min(fixed_count ? fixed_count : ctl->total_keys, capacity);
    const uint32_t nparts = min((K + kSortTile - 1) / kSortTile, max_parts);
    const uint32_t part = blockIdx.x;
    if (part >= nparts) return;  // (uniform)
    const uint32_t mask = (1u << bits) - 1u;
    const uint32_t base = part * kSortTile, cnt = min(kSortTile, K - base);
    // kFull: a whole partition (all but the last), without per-key bounds
    // checks and with a fixed write-out loop
    auto partition = [&](auto full_tag) {
        constexpr bool kFull = decltype(full_tag)::value;
        KeyT k[kItems];
        uint32_t vr[kItems];
#pragma unroll
        for (uint32_t i = 0; i < kItems; ++i) {
            const uint32_t idx = warp * (kItems * 32) + i * 32 + lane;
            if (kFull || idx < cnt) {
                k[i] = keys_in[base + idx];
                vr[i] = vals_in[base + idx];
            } else {
                k[i] = KeyT(~KeyT(0));
                vr[i] = 0u;
            }
        }
        // this partition's digit offsets: chunk base + offset within the chunk,
        // written by the counting kernel (this kernel may have started while it
        // ran: its keys and values come from the kernel before that one)
        pdl_wait();
        pdl_trigger();  // the next kernel (the next counting kernel, or the blend) may be scheduled; it waits for this grid
        uint32_t goff = 0;
        if (digit_thread) {
            const uint32_t* chunk_rows = work + 256 * size_t(max_parts);
            goff = ld_cg_u32(chunk_rows + size_t(part / kChunkParts) * 256 + tid) +
                   ld_cg_u32(work + size_t(part) * 256 + tid);
        }
#pragma unroll
        for (uint32_t i = tid; i < kWarps * kRadix; i += kThreads) (&S.whist[0][0])[i] = 0;
        __syncthreads();
        // stable rank within the warp (warp-striped order)
        uint32_t dr[kItems];
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (uint32_t i = 0; i < kItems; ++i) {
            const uint32_t idx = warp * (kItems * 32) + i * 32 + lane;
            const uint32_t d = kFull || idx < cnt ? (uint32_t(k[i] >> shift) & mask) : kInvalidDigit;
            uint32_t peers = 0xFFFFFFFFu;
#pragma unroll
            for (int b = 0; b < kBits; ++b) {
                const bool on = (d >> b) & 1u;
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, on);
                peers &= on ? bal : ~bal;
            }
            if constexpr (!kFull) {
                const bool on = d >= kRadix;
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, on);
                peers &= on ? bal : ~bal;
            }
            const uint32_t leader = __ffs(peers) - 1;
            uint32_t prev = 0;
            if (lane == leader && (kFull || d < kRadix)) {
                prev = S.whist[warp][d];
                S.whist[warp][d] = prev + __popc(peers);
            }
            prev = __shfl_sync(0xFFFFFFFFu, prev, leader);
            dr[i] = d | ((prev + __popc(peers & lt)) << 9);
            __syncwarp();
        }
        __syncthreads();
        uint32_t count = 0;
        if (digit_thread) {
#pragma unroll
            for (uint32_t w = 0; w < kWarps; ++w) {
                const uint32_t c = S.whist[w][tid];
                S.whist[w][tid] = count;
                count += c;
            }
        }
        const uint32_t lstart = block_exclusive_scan256<kWarps>(count, S.wsum);  // (its barriers cover whist)
        if (digit_thread) {
            S.lstart[tid] = lstart;
            S.gmap[tid] = goff - lstart;
        }
        __syncthreads();
#pragma unroll
        for (uint32_t i = 0; i < kItems; ++i) {
            const uint32_t d = dr[i] & 511u;
            if (kFull || d < kRadix) {
                const uint32_t pos = S.lstart[d] + S.whist[warp][d] + (dr[i] >> 9);
                if (TPD_INBOUNDS(ctl, 20, pos, cnt)) {
                    S.keys[pad16(pos)] = k[i];
                    S.vals[pad16(pos)] = vr[i];
                }
            }
        }
        __syncthreads();
        // (g < K <= capacity: the bound check covers the buffer's end)
        auto write_out = [&](uint32_t j) {
            const KeyT key = S.keys[pad16(j)];
            const uint32_t d = uint32_t(key >> shift) & mask;
            const uint32_t g = S.gmap[d] + j;
            if (TPD_INBOUNDS(ctl, 21, g, K)) {
                keys_out[g] = key;
                vals_out[g] = S.vals[pad16(j)];
                if (ranges) tile_range_bounds(S, ranges, n_tiles, key, j, cnt, d, g, shift, mask, ctl);
            }
        };
        if constexpr (kFull) {
#pragma unroll 4
            for (uint32_t q = 0; q < kItems; ++q) write_out(tid + q * kThreads);
        } else {
            for (uint32_t j = tid; j < cnt; j += kThreads) write_out(j);
        }
    };
    if (cnt == kSortTile)
        partition(std::true_type{});
    else
        partition(std::false_type{});
}

// Residencies: the 256-thread, 16-key variant is compiled for 2 CTAs per SM
// (128 registers, no spills; the default) or 3 (80 registers); the 512-thread,
// 8-key variant for 2 (32 warps per SM); the 8- and 4-key 256-thread variants
// (shorter partitions, for small sorts) for 4 and 5.
// Shared-memory opt-in of every pass kind of a variant and its resident CTAs
// per SM, once per device.
template <int kItems, int kThreads, int kMinBlocks, typename KeyT>
int onesweep_setup() {
    const size_t smem = sizeof(OnesweepSmem<kItems, kThreads, KeyT>);
    cudaFuncSetAttribute(onesweep_kernel<kItems, kThreads, kMinBlocks, kPassPlain, KeyT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if constexpr (sizeof(KeyT) == 8) {
        cudaFuncSetAttribute(onesweep_kernel<kItems, kThreads, kMinBlocks, kPassDropCulled, KeyT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        cudaFuncSetAttribute(onesweep_kernel<kItems, kThreads, kMinBlocks, kPassCompacted, KeyT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    }
    int r = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, onesweep_kernel<kItems, kThreads, kMinBlocks, kPassPlain, KeyT>,
                                                  kThreads, smem);
    return r > 0 ? r : 1;
}

template <int kItems, int kThreads, int kMinBlocks, typename KeyT>
int onesweep_occupancy() {
    return device_once(onesweep_setup<kItems, kThreads, kMinBlocks, KeyT>);
}

template <int kItems, int kThreads, int kMinBlocks, typename KeyT>
void launch_passes(KeyT* kin, uint32_t* vin, KeyT* kout, uint32_t* vout, uint32_t capacity, uint32_t p0,
                   uint32_t p1, const SortPlan& plan, uint32_t (*hist)[256], uint64_t* desc, FrameCtl* ctl,
                   uint32_t spin_limit, int sms, cudaStream_t s) {
    const size_t smem = sizeof(OnesweepSmem<kItems, kThreads, KeyT>);
    const int occ = onesweep_occupancy<kItems, kThreads, kMinBlocks, KeyT>();
    const uint32_t tile = kThreads * kItems;
    const uint32_t max_parts = (capacity + tile - 1) / tile;
    const uint32_t grid = std::max(1u, std::min<uint32_t>(max_parts, uint32_t(sms * occ)));
    for (uint32_t p = p0; p < p1; ++p) {
        const uint32_t shift = p * kRadixBits;
        const uint32_t bits = std::min(kRadixBits, plan.key_bits - shift);
        auto kernel = onesweep_kernel<kItems, kThreads, kMinBlocks, kPassPlain, KeyT>;
        if constexpr (sizeof(KeyT) == 8) {
            if (plan.compact_culled)
                kernel = p == p0 ? onesweep_kernel<kItems, kThreads, kMinBlocks, kPassDropCulled, KeyT>
                                 : onesweep_kernel<kItems, kThreads, kMinBlocks, kPassCompacted, KeyT>;
        }
        launch_dependent(kernel, dim3(grid), dim3(kThreads), smem, s, kin, vin, kout, vout, capacity, p, shift, bits,
                         static_cast<const uint32_t(*)[256]>(hist), plan.ticket_base + p, plan.tag_base + p,
                         plan.fixed_count, desc, ctl, spin_limit, p + 1 == p1 ? plan.ranges : nullptr, plan.n_tiles,
                         kStatusFatal | (plan.skip_on_overflow ? kStatusKeyOverflow : 0u));
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
}

template <int kItems, int kThreads, int kMinBlocks, int kBits, typename KeyT>
int scatter_setup() {
    cudaFuncSetAttribute(scatter_kernel<kItems, kThreads, kMinBlocks, kBits, KeyT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(OnesweepSmem<kItems, kThreads, KeyT>)));
    return 1;
}

// Counted passes (see partition_count_kernel): per pass a counting launch and
// a scatter launch, one CTA per 4096-key partition each. work: the counted
// work area (counted_work_words(max partitions) u32, zero at rest).
template <int kItems, int kThreads, int kMinBlocks, int kBits, typename KeyT>
void launch_scatter(KeyT* kin, uint32_t* vin, KeyT* kout, uint32_t* vout, uint32_t capacity, uint32_t shift,
                    uint32_t bits, const SortPlan& plan, uint32_t max_parts, uint32_t* work, FrameCtl* ctl,
                    uint32_t* ranges, uint32_t abort, cudaStream_t s) {
    device_once(scatter_setup<kItems, kThreads, kMinBlocks, kBits, KeyT>);
    launch_dependent(scatter_kernel<kItems, kThreads, kMinBlocks, kBits, KeyT>, dim3(max_parts), dim3(kThreads),
                     sizeof(OnesweepSmem<kItems, kThreads, KeyT>), s, kin, vin, kout, vout, capacity, shift, bits,
                     plan.fixed_count, max_parts, work, ctl, ranges, plan.n_tiles, abort);
}

// The scatter of one pass of `bits` bits: ballots for exactly that width (the
// 3-CTA variant; the 2-CTA one ranks with 8 ballots).
template <int kItems, int kThreads, int kMinBlocks, typename KeyT>
void launch_scatter_bits(KeyT* kin, uint32_t* vin, KeyT* kout, uint32_t* vout, uint32_t capacity, uint32_t shift,
                         uint32_t bits, const SortPlan& plan, uint32_t max_parts, uint32_t* work, FrameCtl* ctl,
                         uint32_t* ranges, uint32_t abort, cudaStream_t s) {
#define TPD_SCATTER(R) \
    launch_scatter<kItems, kThreads, kMinBlocks, R, KeyT>(kin, vin, kout, vout, capacity, shift, bits, plan, \
                                                          max_parts, work, ctl, ranges, abort, s)
    if constexpr (kMinBlocks != 3) {
        TPD_SCATTER(8);
    } else {
        switch (bits) {
            case 1: TPD_SCATTER(1); break;
            case 2: TPD_SCATTER(2); break;
            case 3: TPD_SCATTER(3); break;
            case 4: TPD_SCATTER(4); break;
            case 5: TPD_SCATTER(5); break;
            case 6: TPD_SCATTER(6); break;
            case 7: TPD_SCATTER(7); break;
            default: TPD_SCATTER(8); break;
        }
    }
#undef TPD_SCATTER
}

// Counted passes (see partition_count_kernel): per pass a counting launch and
// a scatter launch, one CTA per 4096-key partition each. work: the counted
// work area (counted_work_words(max partitions) u32, zero at rest).
template <int kItems, int kThreads, int kMinBlocks, typename KeyT>
void launch_counted_passes(KeyT* kin, uint32_t* vin, KeyT* kout, uint32_t* vout, uint32_t capacity, uint32_t p0,
                           uint32_t p1, const SortPlan& plan, uint32_t (*hist)[256], uint32_t* work, FrameCtl* ctl,
                           cudaStream_t s) {
    static_assert(kThreads * kItems == 4096, "counted passes use 4096-key partitions");
    const uint32_t max_parts = std::max(1u, (capacity + 4095u) / 4096u);
    const uint32_t abort = kStatusFatal | (plan.skip_on_overflow ? kStatusKeyOverflow : 0u);
    for (uint32_t p = p0; p < p1; ++p) {
        const uint32_t shift = p * kRadixBits;
        const uint32_t bits = std::min(kRadixBits, plan.key_bits - shift);
        if (p == p0 && plan.precounted)
            launch_dependent(chunk_scan_kernel, dim3(uint32_t(counted_chunks(max_parts))), dim3(256), 0, s, capacity,
                             p, static_cast<const uint32_t(*)[256]>(hist), plan.fixed_count, max_parts, work, ctl,
                             abort);
        else
            launch_dependent(partition_count_kernel<16, KeyT>, dim3(max_parts), dim3(256), 0, s, kin, capacity, p,
                             shift, bits, static_cast<const uint32_t(*)[256]>(hist), plan.fixed_count, max_parts,
                             work, ctl, abort);
        launch_scatter_bits<kItems, kThreads, kMinBlocks, KeyT>(kin, vin, kout, vout, capacity, shift, bits, plan,
                                                                max_parts, work, ctl,
                                                                p + 1 == p1 ? plan.ranges : nullptr, abort, s);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
}

}  // namespace

size_t sort_counted_work_words(uint32_t capacity) {
    return counted_work_words(std::max(1u, (capacity + 4095u) / 4096u));
}

uint32_t sort_pass_count(uint32_t key_bits) { return (key_bits + kRadixBits - 1) / kRadixBits; }

size_t sort_desc_entries(uint32_t capacity, uint32_t items) {
    const size_t tile = size_t(kSortThreads) * (items ? items : kSortItemsMax);
    return (size_t(capacity) + tile - 1) / tile * kRadix + kRadix;
}

void launch_sort_begin(FrameCtl* ctl, uint32_t total, cudaStream_t s) { sort_begin_kernel<<<1, 256, 0, s>>>(ctl, total); }

namespace {
template <typename KeyT>
bool launch_sort_t(KeyT* keys, uint32_t* vals, KeyT* keys_alt, uint32_t* vals_alt, uint32_t capacity,
                 const SortPlan& plan, uint64_t* desc, FrameCtl* ctl, uint32_t spin_limit, int num_sms,
                 cudaStream_t s) {
    const uint32_t p0 = plan.first_bit / kRadixBits;
    const uint32_t p1 = std::min(8u, sort_pass_count(plan.key_bits));
    if (p1 <= p0 || capacity == 0) return false;
    const int sms = num_sms > 0 ? num_sms : 148;
    uint32_t (*hist)[256] = plan.hist ? plan.hist : ctl->sort_hist;
    if (!plan.hist_ready) {
        const uint32_t hist_blocks = std::max(1u, std::min<uint32_t>(uint32_t(sms) * 4u, capacity / kHistChunk + 1u));
        launch_dependent(sort_histogram_kernel<KeyT>, dim3(hist_blocks), dim3(kHistThreads), 0, s,
                         static_cast<const KeyT*>(keys), capacity, p0, p1, plan.key_bits, hist, ctl);
    }
    if (plan.after_hist) cudaEventRecord(plan.after_hist, s);
    if constexpr (sizeof(KeyT) == 4) {  // counted passes: 32-bit keys (for 64-bit keys onesweep is faster)
        if (plan.counted_work) {
            if (plan.ctas_per_sm == 2)
                launch_counted_passes<16, 256, 2>(keys, vals, keys_alt, vals_alt, capacity, p0, p1, plan, hist,
                                                  plan.counted_work, ctl, s);
            else
                launch_counted_passes<16, 256, 3>(keys, vals, keys_alt, vals_alt, capacity, p0, p1, plan, hist,
                                                  plan.counted_work, ctl, s);
            return ((p1 - p0) & 1u) != 0;
        }
    }
    if (plan.threads == 512)
        launch_passes<8, 512, 2>(keys, vals, keys_alt, vals_alt, capacity, p0, p1, plan, hist, desc, ctl, spin_limit,
                                 sms, s);
    else if (plan.items == 8)
        launch_passes<8, 256, 4>(keys, vals, keys_alt, vals_alt, capacity, p0, p1, plan, hist, desc, ctl, spin_limit,
                                 sms, s);
    else if (plan.items == 4)
        launch_passes<4, 256, 5>(keys, vals, keys_alt, vals_alt, capacity, p0, p1, plan, hist, desc, ctl, spin_limit,
                                 sms, s);
    else if (plan.ctas_per_sm == 3)
        launch_passes<16, 256, 3>(keys, vals, keys_alt, vals_alt, capacity, p0, p1, plan, hist, desc, ctl, spin_limit,
                                  sms, s);
    else
        launch_passes<16, 256, 2>(keys, vals, keys_alt, vals_alt, capacity, p0, p1, plan, hist, desc, ctl, spin_limit,
                                  sms, s);
    return ((p1 - p0) & 1u) != 0;
}
}  // namespace

bool launch_sort(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, uint32_t capacity,
                 const SortPlan& plan, uint64_t* desc, FrameCtl* ctl, uint32_t spin_limit, int num_sms,
                 cudaStream_t s) {
    return launch_sort_t(keys, vals, keys_alt, vals_alt, capacity, plan, desc, ctl, spin_limit, num_sms, s);
}

bool launch_sort(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t capacity,
                 const SortPlan& plan, uint64_t* desc, FrameCtl* ctl, uint32_t spin_limit, int num_sms,
                 cudaStream_t s) {
    return launch_sort_t(keys, vals, keys_alt, vals_alt, capacity, plan, desc, ctl, spin_limit, num_sms, s);
}

}  // namespace tpd
