// blend.cu — kernel (e): per-tile front-to-back alpha blending, and its adjoint.
//
// Reference: blend.slang:24-105 (one 16x16 workgroup per tile; rounds of 256
// splats staged in shared memory; per pixel: power, alpha = min(0.99,
// o*exp(power)), skip below 1/255, stop when T*(1-alpha) < 1e-4; colour
// gathered per contributing pair) dispatched by GaussianEngine.cpp:857-862.
// The reference has no backward pass; blend_backward_kernel is new.
//
// GB300 form: one CTA of 128 threads per tile, each lane on two pixels whose
// pair arithmetic runs in packed f32x2 operations; each round stages
// position, conic+opacity and colour of the next list entries into shared
// memory (colour is staged with the rest instead of gathered per pair), the
// whole CTA leaves as soon as every pixel is done (__syncthreads_count), and
// per pixel the final transmittance and the number of list entries up to the
// last contributor are kept for the adjoint. The adjoint walks each tile's
// list back to front, recomputing transmittance as T / (1 - alpha) from the
// final T (no per-pixel lists), and accumulates per-Gaussian gradients
// warp-reduced, then in shared memory, then with one global atomic per
// (round, Gaussian, field).
//
// Every per-pixel operation (p2, alpha, the skip and stop tests) has the same
// operations and explicit rounding in the forward and in the adjoint, so both
// take identical decisions.
//
// Warp culling: a warp owns an 8x8 pixel block of the tile. The thread that
// stages a list entry also works out, once for the whole CTA, which of the
// tile's four blocks the entry can reach: for each block row (a slab of
// pixel rows) it takes the x extent of the entry's alpha >= 1/255 ellipse
// within the slab (closed form, two square roots), enlarged for rounding,
// and compares it with the two block columns. A warp then walks only the
// entries whose bit for its block is set (one ballot per 32 entries). A
// culled pair lies outside that ellipse, where the pair's own test finds
// alpha below 1/255 and skips it, as the reference does; so the culling
// changes which skipped pairs are visited, never a result.
#include <algorithm>

#include "tpd_common.cuh"
#include "tpd_kernels.h"

namespace tpd {
namespace {

constexpr float kAlphaMax = 0.99f;
constexpr float kTMin = 0.0001f;

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;

// Per (pixel, entry) pair, with the conic pre-scaled at staging
//   qa = -0.5 log2e cx, qb = -log2e cy, qc = -0.5 log2e cz,
//   dx = x - px, dy = y - py (rounded subtractions),
//   p2 = fma(fma(qb, dy, qa dx), dx, (qc dy) dy) = log2(e) * power,
//   power = -0.5 * (cx*dx*dx + cz*dy*dy) - cy*dx*dy  (blend.slang:83-84),
// five multiply/fma operations; exp(power) = 2^p2 is one ex2, and
//   alpha = min(0.99, o * 2^p2) < 1/255  <=>  p2 < thr = log2(1 / (255 o))
// is decided before the exponential.

constexpr float kInf = __builtin_huge_valf();

__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Blocks of the tile at pixel origin (ox, oy) that the entry can reach, for
// blocks 8 pixels wide and 16 / kSlabs high: bit 2k + c for block row k
// (pixel rows oy + hk .. oy + hk + h - 1, h = 16 / kSlabs) and block column c
// (pixel columns ox + 8c .. ox + 8c + 7), the block of warp 2k + c.
//
// With a = -qa, b = -qb / 2, c = -qc and d = centre - pixel, a pixel is kept
// only when p2 >= thr, i.e. inside the ellipse a dx^2 + 2b dx dy + c dy^2 <= R
// for R = -thr. R is enlarged by 4e-3 (relative and absolute) plus 1e-5 ac/det
// relative, which bounds the rounding of the per-pixel p2 even for thin
// ellipses (its terms are at most 4 R ac / det in size there). For dy in a
// slab, the ellipse spans dx in [(-b dy - s) / a, (-b dy + s) / a],
// s = sqrt(a R - det dy^2); over the slab the extremes are +-hx (hx =
// sqrt(c R / det)) when the slab holds the extreme point's dy (-+b hx / c),
// else the values at the slab's ends. The x extent is widened by 0.02 px +
// 1e-4 hx for the rounding of this computation. thr > 0 (opacity below
// 1/255) never blends: no block; a conic that is not positive definite is
// never culled: every block.
template <int kSlabs>
__device__ __forceinline__ uint32_t block_mask(float cx, float cy, float4 q, float ox, float oy) {
    constexpr float kSlabRows = float(kBlockY / kSlabs);  // pixel rows per block row
    const float thr = q.w;
    if (!(thr <= 0.0f)) return 0u;
    const float a = -q.x, c = -q.z, b = -0.5f * q.y;
    const float w = b * b;
    const float det = __fmaf_rn(a, c, -w) + __fmaf_rn(-b, b, w);  // compensated a c - b^2
    if (!(a > 0.0f && c > 0.0f && det > 0.0f)) return 0xFFu;
    const float inv_det = rcp_approx(det), inv_a = rcp_approx(a);
    const float R = -thr * (1.0f + 4e-3f + 1e-5f * (a * c * inv_det)) + 4e-3f;
    const float hx = sqrt_approx(c * R * inv_det), hy = sqrt_approx(a * R * inv_det);
    const float dyr = -b * hx * rcp_approx(c);  // dy of the rightmost point; the leftmost at -dyr
    const float aR = a * R;
    const float wx = 0.02f + 1e-4f * hx;
    uint32_t m = 0;
#pragma unroll
    for (int k = 0; k < kSlabs; ++k) {
        const float y0 = oy + kSlabRows * float(k);
        float dlo = cy - (y0 + (kSlabRows - 1.0f)) - 0.01f, dhi = cy - y0 + 0.01f;
        if (dhi < -hy || dlo > hy) continue;
        dlo = fmaxf(dlo, -hy);
        dhi = fminf(dhi, hy);
        const float s0 = sqrt_approx(fmaxf(__fmaf_rn(-det, dlo * dlo, aR), 0.0f));
        const float s1 = sqrt_approx(fmaxf(__fmaf_rn(-det, dhi * dhi, aR), 0.0f));
        float xmax = fmaxf((-b * dlo + s0) * inv_a, (-b * dhi + s1) * inv_a);
        float xmin = fminf((-b * dlo - s0) * inv_a, (-b * dhi - s1) * inv_a);
        if (dyr >= dlo && dyr <= dhi) xmax = hx;
        if (-dyr >= dlo && -dyr <= dhi) xmin = -hx;
        const float pxlo = cx - xmax - wx, pxhi = cx - xmin + wx;  // pixel x = centre x - dx
        if (pxlo <= ox + 7.0f && pxhi >= ox) m |= 1u << (2 * k);
        if (pxlo <= ox + 15.0f && pxhi >= ox + 8.0f) m |= 2u << (2 * k);
    }
    return m;
}

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// UNORM RGBA8 of (r, g, b, 1): round(clamp(c, 0, 1) * 255) per channel.
__device__ __forceinline__ uint32_t rgba8_unorm(float r, float g, float b) {
    const float c[3] = {r, g, b};
    uint32_t out = 0xFF000000u;
#pragma unroll
    for (int k = 0; k < 3; ++k) out |= uint32_t(__float2uint_rn(fminf(fmaxf(c[k], 0.0f), 1.0f) * 255.0f)) << (8 * k);
    return out;
}

// true when the pair is skipped (power > 0 or alpha < 1/255)
__device__ __forceinline__ bool pair_skipped(float p2, float thr) { return p2 > 0.0f || p2 < thr; }

// View of a global tile id, that view's size, and the tile's (column, row) in it.
__device__ __forceinline__ void load_view_tile(const ViewConst* views, const uint32_t* tile_view, uint32_t tile,
                                               uint32_t& vi, uint32_t& width, uint32_t& height, uint32_t& tx,
                                               uint32_t& ty) {
    vi = tile_view ? tile_view[tile] : 0u;
    const ViewConst& v = views[vi];
    width = v.width;
    height = v.height;
    const uint32_t local = tile - v.tile_base;
    const uint32_t gx = grid_x(width);
    tx = local % gx;
    ty = local / gx;
}

// ---- forward
//
// A CTA of 128 threads per tile. Warp w owns the 8x8 block at (8 (w & 1),
// 8 (w >> 1)) of the tile, and lane l the two pixels (l & 7, l >> 3) and
// (l & 7, (l >> 3) + 4) of that block. The two pixels of a lane share dx, and
// the arithmetic of a (pixel, entry) pair runs on both pixels at once with
// packed f32x2 operations: per pixel the operations, order and rounding
// given above for p2, alpha and the tests, as in the adjoint. A staged entry
// holds its values duplicated in register-pair order, so the packed operands
// come straight out of five broadcast shared-memory loads.
constexpr uint32_t kFwdThreads = 128;
// List entries per staged round (the blend's batch depth, an engine setting
// the autotuner picks): 128 by default (20 KB of shared memory, 8 CTAs per
// SM at 64 registers); 64 (8 CTAs) or 256 (41 KB, 5 CTAs).
template <uint32_t kRound>
constexpr int fwd_min_blocks() { return kRound >= 256 ? 5 : 8; }

struct PairStaged {  // 80 bytes
    float4 xy;       // x, x, y, y
    float4 qab;      // qa, qa, qb, qb
    float4 qco;      // qc, qc, opacity, opacity
    float4 rg;       // r, r, g, g
    float4 bt;       // b, b, thr, 0
};

template <uint32_t kRound>
struct FwdStage {
    PairStaged e[2][kRound];
    uint8_t mask[2][kRound];  // bit w: the entry can reach warp w's 8x8 block
};

__device__ __forceinline__ void stage_pair_values(float4 c, float4 tex, float4 co, float ox, float oy, PairStaged& d,
                                                  uint8_t& mask) {
    const float thr = co.w > 0.0f ? -__log2f(255.0f * co.w) : kInf;  // +inf: never blends
    const float4 q = make_float4(-0.5f * kLog2e * co.x, -kLog2e * co.y, -0.5f * kLog2e * co.z, thr);
    d.xy = make_float4(tex.x, tex.x, tex.y, tex.y);
    d.qab = make_float4(q.x, q.x, q.y, q.y);
    d.qco = make_float4(q.z, q.z, co.w, co.w);
    d.rg = make_float4(c.x, c.x, c.y, c.y);
    d.bt = make_float4(c.z, c.z, thr, 0.0f);
    mask = uint8_t(block_mask<2>(tex.x, tex.y, q, ox, oy));
}

__device__ __forceinline__ void stage_pair_entry(const Splat* sp, float ox, float oy, PairStaged& d, uint8_t& mask) {
    const float4* p = reinterpret_cast<const float4*>(sp);
    stage_pair_values(__ldg(p + 0), __ldg(p + 1), __ldg(p + 2), ox, oy, d, mask);
}

__device__ __forceinline__ void stage_pair_empty(PairStaged& d, uint8_t& mask) {
    d.xy = d.qab = d.qco = d.rg = make_float4(0.f, 0.f, 0.f, 0.f);
    d.bt = make_float4(0.f, 0.f, kInf, 0.f);
    mask = 0u;
}

// One tile: rounds of kRound list entries, double-buffered: while the warps
// walk round r, each thread stages its entry of round r + 1 into the other
// buffer, and one barrier per round (which also counts finished pixels)
// separates the two. Called by the whole CTA; the first barrier comes after
// the first staging and the last one after every read of S. kState: also
// track and store each pixel's final transmittance and last contributor (the
// adjoint's inputs); a frame that no backward follows skips that work.
template <uint32_t kRound, bool kState>
__device__ __forceinline__ void blend_tile(const BlendArgs& a, uint32_t tile, FwdStage<kRound>& S) {
    uint32_t vi, W, H, tx, ty;
    load_view_tile(a.views, a.tile_view, tile, vi, W, H, tx, ty);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t px = tx * kBlockX + 8u * (warp & 1u) + (lane & 7u);
    const uint32_t pya = ty * kBlockY + 8u * (warp >> 1) + (lane >> 3), pyb = pya + 4u;
    const float ox = float(tx * kBlockX), oy = float(ty * kBlockY);
    const bool in_a = px < W && pya < H, in_b = px < W && pyb < H;
    const float2 npx = make_float2(-float(px), -float(px));
    const float2 npy = make_float2(-float(pya), -float(pyb));
    const uint32_t K = min(a.ctl->total_keys, a.capacity);
    const uint32_t raw_start = a.ranges[tile * 2 + 0], raw_end = a.ranges[tile * 2 + 1];
    const uint32_t end = min(raw_end, K), start = min(raw_start, end);
    // a tile without keys still holds the sort's preset (0xFFFFFFFF, 0): store
    // the reference's empty range (0, 0)
    if (tid == 0 && raw_start > raw_end) a.ranges[tile * 2 + 0] = 0u;
    const Splat* vsplats = a.splats + size_t(vi) * a.n;

    // entries j0 + tid, j0 + tid + 128, ... (below j0 + kRound) of the list into buffer buf
    auto stage = [&](uint32_t buf, uint32_t j0) {
#pragma unroll
        for (uint32_t k = tid; k < kRound; k += kFwdThreads) {
            const uint32_t j = j0 + k;
            if (j >= end || !TPD_INBOUNDS(a.ctl, 40, j, a.capacity)) continue;
            const uint32_t idx = a.vals[j];
            if (idx < a.n && TPD_INBOUNDS(a.ctl, 42, idx, a.n))
                stage_pair_entry(vsplats + idx, ox, oy, S.e[buf][k], S.mask[buf][k]);
            else
                stage_pair_empty(S.e[buf][k], S.mask[buf][k]);  // only reachable with corrupted lists
        }
    };

    // A pixel that stops is frozen at T = 0: every later pair then adds
    // exactly nothing, so no per-pixel done flags are needed (pixels outside
    // the image start frozen). With the adjoint's inputs, Tk keeps the
    // transmittance at the stop, which is what the reference leaves.
    float2 T = make_float2(in_a ? 1.0f : 0.0f, in_b ? 1.0f : 0.0f);
    float2 Tk = make_float2(1.0f, 1.0f);  // kState: the transmittance to store (it stays at the stop)
    float2 C0 = make_float2(0.f, 0.f), C1 = C0, C2 = C0;
    uint32_t last_a = 0, last_b = 0;
    const float2 one = make_float2(1.0f, 1.0f), mone = make_float2(-1.0f, -1.0f);
    auto pixels_done = [&]() { return T.x == 0.0f && T.y == 0.0f; };
    if (start < end) stage(0, start);
    bool all_done = __syncthreads_count(pixels_done()) == kFwdThreads;
    uint32_t r = 0;
    for (uint32_t b0 = start; b0 < end && !all_done; b0 += kRound, ++r) {
        const uint32_t b = r & 1u;
        // the next round's entries, into the buffer the last barrier released
        if (b0 + kRound < end) stage(b ^ 1u, b0 + kRound);
        const uint32_t n = min(kRound, end - b0);
        const uint32_t lbase = b0 - start + 1u;  // n_contrib of entry jj of this round: lbase + jj
        for (uint32_t g = 0; g < n; g += 32) {
            if (__all_sync(0xFFFFFFFFu, pixels_done())) break;
            const uint32_t e = g + lane;
            uint32_t m = __ballot_sync(0xFFFFFFFFu, e < n && ((S.mask[b][e] >> warp) & 1u));
            // branch-free body: every lane evaluates both pairs and selects
            // the update, so lanes taking different decisions do not run the
            // paths one after another. A skipped pair gets alpha = 0, which
            // leaves T and C exactly as they were.
            // alpha of a staged entry for both pixels (0 when the pair is skipped)
            auto alpha_of = [&](const PairStaged& E) {
                const float4 xy = E.xy, qab = E.qab, qco = E.qco, bt = E.bt;
                const float2 dx = __fadd2_rn(make_float2(xy.x, xy.y), npx);
                const float2 dy = __fadd2_rn(make_float2(xy.z, xy.w), npy);
                const float2 t = __ffma2_rn(make_float2(qab.z, qab.w), dy, __fmul2_rn(make_float2(qab.x, qab.y), dx));
                const float2 p2 = __ffma2_rn(t, dx, __fmul2_rn(__fmul2_rn(make_float2(qco.x, qco.y), dy), dy));
                const float2 ao =
                    __fmul2_rn(make_float2(qco.z, qco.w), make_float2(ex2_approx(p2.x), ex2_approx(p2.y)));
                return make_float2(pair_skipped(p2.x, bt.z) ? 0.0f : fminf(kAlphaMax, ao.x),
                                   pair_skipped(p2.y, bt.z) ? 0.0f : fminf(kAlphaMax, ao.y));
            };
            // the pair's update, in list order. keep = 0 at the stop and after
            // it (T = 0 gives tn = 0): the pair adds alpha T * 0 = 0 and T
            // becomes 0; before the stop keep = 1 and both products are exact
            // copies. With the adjoint's inputs, Tk keeps the transmittance at
            // the stop and the last entry that added is the last with w > 0
            // (alpha >= 1/255 times T >= 1e-4).
            auto apply = [&](float2 alpha, const PairStaged& E, uint32_t jj) {
                const float4 rg = E.rg, bt = E.bt;
                const float2 tn = __fmul2_rn(T, __ffma2_rn(mone, alpha, one));  // T (1 - alpha)
                const bool go_a = !(tn.x < kTMin), go_b = !(tn.y < kTMin);
                const float2 keep = make_float2(go_a ? 1.0f : 0.0f, go_b ? 1.0f : 0.0f);
                const float2 w = __fmul2_rn(__fmul2_rn(alpha, T), keep);
                C0 = __ffma2_rn(make_float2(rg.x, rg.y), w, C0);
                C1 = __ffma2_rn(make_float2(rg.z, rg.w), w, C1);
                C2 = __ffma2_rn(make_float2(bt.x, bt.y), w, C2);
                T = __fmul2_rn(tn, keep);
                if constexpr (kState) {
                    Tk = make_float2(go_a ? tn.x : Tk.x, go_b ? tn.y : Tk.y);
                    last_a = w.x > 0.0f ? lbase + jj : last_a;
                    last_b = w.y > 0.0f ? lbase + jj : last_b;
                }
            };
            // without the adjoint's inputs, two entries per step when there are
            // two: their alphas are independent, only the updates run in order
            // (with them, the extra registers cost more than the overlap gives)
            while (m) {
                const uint32_t j0 = g + uint32_t(__ffs(m) - 1);
                m &= m - 1u;
                if (!kState && m) {
                    const uint32_t j1 = g + uint32_t(__ffs(m) - 1);
                    m &= m - 1u;
                    const PairStaged &E0 = S.e[b][j0], &E1 = S.e[b][j1];
                    const float2 a0 = alpha_of(E0), a1 = alpha_of(E1);
                    apply(a0, E0, j0);
                    apply(a1, E1, j1);
                } else {
                    const PairStaged& E0 = S.e[b][j0];
                    apply(alpha_of(E0), E0, j0);
                }
            }
        }
        all_done = __syncthreads_count(pixels_done()) == kFwdThreads;
    }
    if (TPD_INBOUNDS(a.ctl, 41, tile, a.n_tiles)) {
        const size_t img0 = a.image_offset ? a.image_offset[vi] : 0ull;
        if (in_a) {
            const size_t p = img0 + size_t(pya) * W + px;
            a.image[p * 3 + 0] = C0.x;
            a.image[p * 3 + 1] = C1.x;
            a.image[p * 3 + 2] = C2.x;
            if (a.rgba) a.rgba[p] = rgba8_unorm(C0.x, C1.x, C2.x);
            if constexpr (kState) {
                a.final_T[p] = Tk.x;
                a.n_contrib[p] = last_a;
            }
        }
        if (in_b) {
            const size_t p = img0 + size_t(pyb) * W + px;
            a.image[p * 3 + 0] = C0.y;
            a.image[p * 3 + 1] = C1.y;
            a.image[p * 3 + 2] = C2.y;
            if (a.rgba) a.rgba[p] = rgba8_unorm(C0.y, C1.y, C2.y);
            if constexpr (kState) {
                a.final_T[p] = Tk.y;
                a.n_contrib[p] = last_b;
            }
        }
    }
}

// The tile scheduler of a persistent launch: the CTA takes the next item of
// the frame's tile queue (an atomic ticket in FrameCtl) until the queue is
// empty; item i is tile order[i] (nullptr: tile i). Every tile of every view
// is one item, so one launch balances all views' tiles at once.
__device__ __forceinline__ bool next_tile(FrameCtl* ctl, uint32_t slot, const uint32_t* order, uint32_t n_tiles,
                                          uint32_t& tile) {
    __shared__ uint32_t s_item;
    if (threadIdx.x == 0) s_item = atomicAdd(&ctl->ticket[slot], 1u);
    __syncthreads();
    const uint32_t i = s_item;
    __syncthreads();  // every thread has read s_item before it is written again
    if (i >= n_tiles) return false;
    tile = order ? order[i] : i;
    return true;
}

// One CTA per tile, or (kPersistent) one CTA per resident slot taking tiles
// from the queue.
template <uint32_t kRound, bool kPersistent, bool kState>
__global__ void __launch_bounds__(kFwdThreads, fwd_min_blocks<kRound>()) blend_kernel(BlendArgs a) {
    __shared__ FwdStage<kRound> S;
    pdl_wait();  // launched as a dependent of the key sort's last pass: its lists and ranges
    pdl_trigger();
    // an overflowed frame is re-rendered with larger key buffers; nothing to draw
    if (a.ctl->status & (kStatusFatal | kStatusKeyOverflow)) return;
    if constexpr (kPersistent) {
        uint32_t tile;
        while (next_tile(a.ctl, kTicketBlend, nullptr, a.n_tiles, tile)) blend_tile<kRound, kState>(a, tile, S);
    } else {
        blend_tile<kRound, kState>(a, blockIdx.x, S);
    }
}

// UNORM conversion of (r, g, b, 1): round(clamp(c, 0, 1) * 255).
__global__ void pack_rgba8_kernel(const float* rgb, uint32_t* rgba, size_t pixels) {
    pdl_wait();  // launched as a dependent of the blend
    pdl_trigger();
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= pixels) return;
    rgba[i] = rgba8_unorm(rgb[i * 3 + 0], rgb[i * 3 + 1], rgb[i * 3 + 2]);
}

constexpr int kG2D = 9;  // px, py, conic.x, conic.y, conic.z, opacity, r, g, b

// Sums v[0..7] over the warp with a transposed butterfly: each of the first
// three exchanges halves the values a lane holds, the last two add single
// values. Afterwards lane 4j holds the warp sum of v[j] (j = 0..7).
__device__ __forceinline__ float warp_sum8_transposed(const float (&v)[8], uint32_t lane) {
    float a[4], b[2], c;
    const bool u4 = (lane >> 4) & 1u, u3 = (lane >> 3) & 1u, u2 = (lane >> 2) & 1u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float send = u4 ? v[i] : v[i + 4];
        const float keep = u4 ? v[i + 4] : v[i];
        a[i] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float send = u3 ? a[i] : a[i + 2];
        const float keep = u3 ? a[i + 2] : a[i];
        b[i] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 8);
    }
    {
        const float send = u2 ? b[0] : b[1];
        const float keep = u2 ? b[1] : b[0];
        c = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 4);
    }
    c += __shfl_xor_sync(0xFFFFFFFFu, c, 2);
    c += __shfl_xor_sync(0xFFFFFFFFu, c, 1);
    return c;
}

// The adjoint, with the forward's layout: a CTA of 128 threads per tile,
// warp w on the 8x8 block at (8 (w & 1), 8 (w >> 1)), lane l on pixels
// (l & 7, l >> 3) and (l & 7, (l >> 3) + 4), pair arithmetic packed in f32x2.
// Rounds of kBwdRound list entries from the back: staging double-buffered,
// per-round gradient sums in one of two shared buffers. The barrier at the
// end of a round completes its sums; each thread then adds its share of them
// to global memory and zeroes what it added, so the buffer is clean when it
// comes round again two rounds later. The staged indices that the flush
// reads live in three buffers (the next round's staging overwrites the one of
// the round before the last).
//
// List entries per round (an engine setting the autotuner picks): 64 by
// default (17 KB of shared memory, 8 CTAs per SM at 64 registers); 32 (8 CTAs)
// or 128 (35 KB, 6 CTAs).
template <uint32_t kBwdRound>
constexpr int bwd_min_blocks() { return kBwdRound >= 128 ? 6 : 8; }
template <uint32_t kBwdRound>
struct BlendBackwardSmem {
    PairStaged e[2][kBwdRound];
    uint8_t mask[2][kBwdRound];
    float acc[2][kBwdRound][kG2DStride];
    uint32_t idx[3][kBwdRound];
    uint32_t wmax[kFwdThreads / 32];
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// One tile of the adjoint (the whole CTA; barriers as in blend_tile).
template <uint32_t kBwdRound>
__device__ __forceinline__ void blend_backward_tile(const BlendBackwardArgs& a, uint32_t tile,
                                                    BlendBackwardSmem<kBwdRound>& SM) {
    if (!TPD_INBOUNDS(a.ctl, 44, tile, a.n_tiles)) return;  // (uniform)
    uint32_t vi, W, H, tx, ty;
    load_view_tile(a.views, a.tile_view, tile, vi, W, H, tx, ty);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t px = tx * kBlockX + 8u * (warp & 1u) + (lane & 7u);
    const uint32_t pya = ty * kBlockY + 8u * (warp >> 1) + (lane >> 3), pyb = pya + 4u;
    const float ox = float(tx * kBlockX), oy = float(ty * kBlockY);
    const bool in_a = px < W && pya < H, in_b = px < W && pyb < H;
    const float2 npx = f2(-float(px), -float(px));
    const float2 npy = f2(-float(pya), -float(pyb));
    const uint32_t K = min(a.ctl->total_keys, a.capacity);
    const uint32_t end = min(a.ranges[tile * 2 + 1], K), start = min(a.ranges[tile * 2 + 0], end);
    const Splat* vsplats = a.splats + size_t(vi) * a.n;

    const size_t img0 = a.image_offset ? a.image_offset[vi] : 0ull;
    const size_t pa = img0 + size_t(pya) * W + px, pb = img0 + size_t(pyb) * W + px;
    float2 T = f2(1.0f, 1.0f), g0 = f2(0.f, 0.f), g1 = g0, g2 = g0;
    uint32_t last_a = 0, last_b = 0;
    if (in_a) {
        T.x = a.final_T[pa];
        last_a = min(a.n_contrib[pa], end - start);
        g0.x = a.dL_dimage[pa * 3 + 0];
        g1.x = a.dL_dimage[pa * 3 + 1];
        g2.x = a.dL_dimage[pa * 3 + 2];
    }
    if (in_b) {
        T.y = a.final_T[pb];
        last_b = min(a.n_contrib[pb], end - start);
        g0.y = a.dL_dimage[pb * 3 + 0];
        g1.y = a.dL_dimage[pb * 3 + 1];
        g2.y = a.dL_dimage[pb * 3 + 2];
    }
    // the block walks back from the largest last-contributor index over its
    // pixels; a warp takes entries below its own largest index only
    uint32_t warp_last = max(last_a, last_b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) warp_last = max(warp_last, __shfl_xor_sync(0xFFFFFFFFu, warp_last, o));
    if (lane == 0) SM.wmax[warp] = warp_last;
    for (uint32_t k = tid; k < 2 * kBwdRound * kG2DStride; k += kFwdThreads) (&SM.acc[0][0][0])[k] = 0.f;
    __syncthreads();
    uint32_t max_last = 0;
#pragma unroll
    for (uint32_t w = 0; w < kFwdThreads / 32; ++w) max_last = max(max_last, SM.wmax[w]);

    float2 S0 = f2(0.f, 0.f), S1 = S0, S2 = S0;  // colour accumulated behind the current entry
    float* g2d_view = a.g2d + size_t(vi) * a.g2d_view_stride;
    // stages the round whose list positions (relative) end at r_end: slot k
    // holds position r_end - 1 - k
    auto stage_round = [&](int32_t r_end, uint32_t b, uint32_t bi) {
        const uint32_t n = uint32_t(min(int32_t(kBwdRound), r_end));
        for (uint32_t k = tid; k < n; k += kFwdThreads) {
            const uint32_t e = uint32_t(r_end) - 1u - k;
            uint32_t idx = a.vals[start + e];
            if (idx < a.n) {
                stage_pair_entry(vsplats + idx, ox, oy, SM.e[b][k], SM.mask[b][k]);
            } else {  // only reachable with corrupted lists
                idx = 0;
                stage_pair_empty(SM.e[b][k], SM.mask[b][k]);
            }
            SM.idx[bi][k] = idx;
        }
    };
    if (max_last > 0) stage_round(int32_t(max_last), 0, 0);
    __syncthreads();
    // the next round's entry of this thread (one per thread: kBwdRound <=
    // kFwdThreads), loaded before the current round is walked and staged after
    // it, so the gathers' latency hides behind the walk
    static_assert(kBwdRound <= kFwdThreads, "one staged entry per thread");
    bool pf = false;
    uint32_t pf_idx = 0;
    float4 pf_c = make_float4(0.f, 0.f, 0.f, 0.f), pf_tex = pf_c, pf_co = pf_c;
    auto load_next = [&](int32_t r_end) {
        pf = tid < uint32_t(min(int32_t(kBwdRound), r_end));
        if (!pf) return;
        pf_idx = a.vals[start + uint32_t(r_end) - 1u - tid];
        if (pf_idx < a.n) {
            const float4* p = reinterpret_cast<const float4*>(vsplats + pf_idx);
            pf_c = __ldg(p + 0);
            pf_tex = __ldg(p + 1);
            pf_co = __ldg(p + 2);
        }
    };
    auto store_next = [&](uint32_t b, uint32_t bi) {
        if (!pf) return;
        if (pf_idx < a.n) {
            stage_pair_values(pf_c, pf_tex, pf_co, ox, oy, SM.e[b][tid], SM.mask[b][tid]);
        } else {  // only reachable with corrupted lists
            pf_idx = 0;
            stage_pair_empty(SM.e[b][tid], SM.mask[b][tid]);
        }
        SM.idx[bi][tid] = pf_idx;
    };
    const float2 one = f2(1.0f, 1.0f), mone = f2(-1.0f, -1.0f), mhalf = f2(-0.5f, -0.5f), ln2 = f2(kLn2, kLn2);
    uint32_t r = 0;
    for (int32_t r_end = int32_t(max_last); r_end > 0; r_end -= int32_t(kBwdRound), ++r) {
        const uint32_t b = r & 1u, bi = r % 3u;
        const uint32_t n = uint32_t(min(int32_t(kBwdRound), r_end));
        if (r_end > int32_t(kBwdRound)) load_next(r_end - int32_t(kBwdRound));
        else pf = false;
        // entries jj >= skip have list positions r_end - 1 - jj below warp_last
        const uint32_t skip = uint32_t(r_end) > warp_last ? uint32_t(r_end) - warp_last : 0u;
        for (uint32_t g = skip & ~31u; g < n; g += 32) {
            const uint32_t jl = g + lane;
            uint32_t m = __ballot_sync(0xFFFFFFFFu, jl < n && jl >= skip && ((SM.mask[b][jl] >> warp) & 1u));
            while (m) {
                const uint32_t jj = g + uint32_t(__ffs(m) - 1);
                m &= m - 1u;
                const uint32_t e = uint32_t(r_end) - 1u - jj;
                const PairStaged& E = SM.e[b][jj];
                const float4 xy = E.xy, qab = E.qab, qco = E.qco, rg = E.rg, bt = E.bt;
                // p2 for both pixels, as in the forward
                const float2 dx = __fadd2_rn(f2(xy.x, xy.y), npx);
                const float2 dy = __fadd2_rn(f2(xy.z, xy.w), npy);
                const float2 qadx = __fmul2_rn(f2(qab.x, qab.y), dx);
                const float2 t = __ffma2_rn(f2(qab.z, qab.w), dy, qadx);
                const float2 qcdy = __fmul2_rn(f2(qco.x, qco.y), dy);
                const float2 p2 = __ffma2_rn(t, dx, __fmul2_rn(qcdy, dy));
                const bool ca = in_a && e < last_a && !pair_skipped(p2.x, bt.z);
                const bool cb = in_b && e < last_b && !pair_skipped(p2.y, bt.z);
                // branch-free body: zero weight and gradient scale for pairs
                // that do not count; every term below is finite, so they add
                // exactly nothing
                const float2 G = f2(ex2_approx(p2.x), ex2_approx(p2.y));
                const float2 raw = __fmul2_rn(f2(qco.z, qco.w), G);
                const float2 alpha = f2(fminf(kAlphaMax, raw.x), fminf(kAlphaMax, raw.y));
                const float2 om = __ffma2_rn(mone, alpha, one);  // 1 - alpha >= 0.01
                const float2 inv = f2(__fdividef(1.0f, om.x), __fdividef(1.0f, om.y));
                const float2 Tb = __fmul2_rn(T, inv);  // transmittance in front of this entry
                const float2 aTb = __fmul2_rn(alpha, Tb);
                const float2 w = f2(ca ? aTb.x : 0.0f, cb ? aTb.y : 0.0f);
                // dL/dalpha = sum_c g_c (col_c Tb - S_c / (1 - alpha))
                const float2 ninv = __fmul2_rn(inv, mone);
                const float2 d0 = __ffma2_rn(f2(rg.x, rg.y), Tb, __fmul2_rn(S0, ninv));
                const float2 d1 = __ffma2_rn(f2(rg.z, rg.w), Tb, __fmul2_rn(S1, ninv));
                const float2 d2 = __ffma2_rn(f2(bt.x, bt.y), Tb, __fmul2_rn(S2, ninv));
                const float2 dA = __ffma2_rn(g2, d2, __ffma2_rn(g1, d1, __fmul2_rn(g0, d0)));
                S0 = __ffma2_rn(f2(rg.x, rg.y), w, S0);
                S1 = __ffma2_rn(f2(rg.z, rg.w), w, S1);
                S2 = __ffma2_rn(f2(bt.x, bt.y), w, S2);
                T = f2(ca ? Tb.x : T.x, cb ? Tb.y : T.y);
                // power = p2 ln2; d power / d(dx, dy) = ln2 (2 qa dx + qb dy, 2 qc dy + qb dx)
                const bool ua = ca && raw.x <= kAlphaMax, ub = cb && raw.y <= kAlphaMax;
                const float2 dAa = __fmul2_rn(dA, alpha);
                const float2 dpow = f2(ua ? dAa.x : 0.0f, ub ? dAa.y : 0.0f);
                const float2 dpl = __fmul2_rn(dpow, ln2), hdp = __fmul2_rn(dpow, mhalf);
                const float2 dAG = __fmul2_rn(dA, G);
                float2 gv[kG2D];
                gv[0] = __fmul2_rn(dpl, __fadd2_rn(t, qadx));                                  // 2 qa dx + qb dy
                gv[1] = __fmul2_rn(dpl, __ffma2_rn(f2(qab.z, qab.w), dx, __fadd2_rn(qcdy, qcdy)));  // 2 qc dy + qb dx
                gv[2] = __fmul2_rn(hdp, __fmul2_rn(dx, dx));
                gv[3] = __fmul2_rn(__fmul2_rn(dpow, mone), __fmul2_rn(dx, dy));
                gv[4] = __fmul2_rn(hdp, __fmul2_rn(dy, dy));
                gv[5] = f2(ua ? dAG.x : 0.0f, ub ? dAG.y : 0.0f);
                gv[6] = __fmul2_rn(g0, w);
                gv[7] = __fmul2_rn(g1, w);
                gv[8] = __fmul2_rn(g2, w);
                if (__any_sync(0xFFFFFFFFu, ca || cb)) {
                    // the lane's two pixels first, then the warp
                    const float lo[8] = {gv[0].x + gv[0].y, gv[1].x + gv[1].y, gv[2].x + gv[2].y, gv[3].x + gv[3].y,
                                         gv[4].x + gv[4].y, gv[5].x + gv[5].y, gv[6].x + gv[6].y, gv[7].x + gv[7].y};
                    const float rs = warp_sum8_transposed(lo, lane);
                    float b9 = gv[8].x + gv[8].y;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) b9 += __shfl_xor_sync(0xFFFFFFFFu, b9, o);
                    if ((lane & 3u) == 0) atomicAdd(&SM.acc[b][jj][lane >> 2], rs);
                    if (lane == 0) atomicAdd(&SM.acc[b][jj][8], b9);
                }
            }
        }
        store_next(b ^ 1u, (r + 1) % 3u);
        __syncthreads();  // round r's sums complete; the other stage buffer is filled
        // one 16-byte vector atomic per non-zero quarter of an entry's record;
        // the thread that adds a quarter also zeroes it for round r + 2
        for (uint32_t k = tid; k < n * 3; k += kFwdThreads) {
            const uint32_t jj = k / 3, c = k % 3;
            float4* slot = reinterpret_cast<float4*>(&SM.acc[b][jj][0]) + c;
            const float4 v = *slot;
            if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f) {
                atomicAdd(reinterpret_cast<float4*>(g2d_view + size_t(SM.idx[bi][jj]) * kG2DStride) + c, v);
                *slot = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    }
    __syncthreads();  // the flush of the last round is done before SM is used again
}

// One CTA per tile, tile order[b] for CTA b; or (kPersistent) one CTA per
// resident slot taking the tiles from the queue in that order.
template <uint32_t kBwdRound, bool kPersistent>
__global__ void __launch_bounds__(kFwdThreads, bwd_min_blocks<kBwdRound>())
    blend_backward_kernel(BlendBackwardArgs a) {
    __shared__ __align__(16) BlendBackwardSmem<kBwdRound> SM;
    pdl_wait();  // launched as a dependent of the stream's previous kernel: its output is read below
    pdl_trigger();
    if (a.ctl->status & (kStatusFatal | kStatusKeyOverflow)) return;  // no valid frame to differentiate
    if constexpr (kPersistent) {
        uint32_t tile;
        while (next_tile(a.ctl, kTicketBlendBackward, a.tile_order, a.n_tiles, tile))
            blend_backward_tile<kBwdRound>(a, tile, SM);
    } else {
        blend_backward_tile<kBwdRound>(a, a.tile_order ? a.tile_order[blockIdx.x] : blockIdx.x, SM);
    }
}

// One CTA: a counting sort of the tiles into 32 classes of list length
// (floor(log2(length + 1)), longest class first).
constexpr uint32_t kOrderThreads = 1024;

__global__ void __launch_bounds__(kOrderThreads)
    tile_order_kernel(const uint32_t* __restrict__ ranges, uint32_t n_tiles, FrameCtl* __restrict__ ctl,
                      uint32_t capacity, uint32_t* __restrict__ order) {
    __shared__ uint32_t count[32], base[32];
    pdl_wait();  // launched as a dependent of the stream's previous kernel: its output is read below
    pdl_trigger();
    const uint32_t tid = threadIdx.x;
    if (tid < 32) count[tid] = 0;
    if (tid == 0) ctl->ticket[kTicketBlendBackward] = 0;  // the adjoint's tile queue starts again
    __syncthreads();
    const uint32_t K = min(ctl->total_keys, capacity);
    // class c = floor(log2(len + 1)) in 0..31; slot 31 - c puts long lists first
    auto slot = [&](uint32_t t) {
        const uint32_t end = min(ranges[2 * t + 1], K), start = min(ranges[2 * t], end);
        const uint32_t len = end - start;
        const uint32_t c = 31u - __clz(len + 1u);  // len < 2^31
        return 31u - c;
    };
    for (uint32_t t = tid; t < n_tiles; t += kOrderThreads) atomicAdd(&count[slot(t)], 1u);
    __syncthreads();
    if (tid == 0) {
        uint32_t run = 0;
        for (uint32_t c = 0; c < 32; ++c) {
            base[c] = run;
            run += count[c];
        }
    }
    __syncthreads();
    for (uint32_t t = tid; t < n_tiles; t += kOrderThreads) {
        const uint32_t pos = atomicAdd(&base[slot(t)], 1u);
        if (pos < n_tiles) order[pos] = t;
    }
}

}  // namespace

void launch_tile_order(const uint32_t* ranges, uint32_t n_tiles, FrameCtl* ctl, uint32_t capacity,
                       uint32_t* order, cudaStream_t s) {
    if (n_tiles == 0) return;
    launch_dependent(tile_order_kernel, dim3(1), dim3(kOrderThreads), 0, s, ranges, n_tiles, ctl, capacity, order);
}

namespace {

template <typename Kernel>
int resident_ctas(Kernel k) {
    int r = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k, kFwdThreads, 0);
    return r > 0 ? r : 1;
}
template <uint32_t R, bool P, bool K>
int blend_occupancy() { return resident_ctas(blend_kernel<R, P, K>); }
template <uint32_t R, bool P>
int blend_backward_occupancy() { return resident_ctas(blend_backward_kernel<R, P>); }

template <uint32_t R, bool P, bool K>
void launch_blend_k(const BlendArgs& a, int num_sms, cudaStream_t s) {
    const uint32_t grid =
        P ? std::min<uint32_t>(a.n_tiles, uint32_t(num_sms * device_once(blend_occupancy<R, P, K>))) : a.n_tiles;
    if (P)  // a persistent grid is placed once: on SMs the key sort has left, not while its last CTAs run
        blend_kernel<R, P, K><<<grid, kFwdThreads, 0, s>>>(a);
    else
        launch_dependent(blend_kernel<R, P, K>, dim3(grid), dim3(kFwdThreads), 0, s, a);
}

// with the adjoint's inputs (final T, last contributor) when both buffers are given
template <uint32_t R, bool P>
void launch_blend_t(const BlendArgs& a, int num_sms, cudaStream_t s) {
    if (a.final_T && a.n_contrib)
        launch_blend_k<R, P, true>(a, num_sms, s);
    else
        launch_blend_k<R, P, false>(a, num_sms, s);
}

template <uint32_t R, bool P>
void launch_blend_backward_t(const BlendBackwardArgs& a, int num_sms, cudaStream_t s) {
    const uint32_t grid = P ? std::min<uint32_t>(a.n_tiles, uint32_t(num_sms * device_once(blend_backward_occupancy<R, P>)))
                            : a.n_tiles;
    launch_dependent(blend_backward_kernel<R, P>, dim3(grid), dim3(kFwdThreads), 0, s, a);
}

}  // namespace

void launch_blend(const BlendArgs& a, const BlendLaunch& l, cudaStream_t s) {
    if (a.n_tiles == 0) return;
    const int sms = l.num_sms > 0 ? l.num_sms : 148;
    switch (l.round) {
        case 64: l.persistent ? launch_blend_t<64, true>(a, sms, s) : launch_blend_t<64, false>(a, sms, s); break;
        case 256: l.persistent ? launch_blend_t<256, true>(a, sms, s) : launch_blend_t<256, false>(a, sms, s); break;
        default: l.persistent ? launch_blend_t<128, true>(a, sms, s) : launch_blend_t<128, false>(a, sms, s); break;
    }
}

void launch_pack_rgba8(const float* rgb, uint32_t* rgba, size_t pixels, cudaStream_t s) {
    if (pixels == 0) return;
    launch_dependent(pack_rgba8_kernel, dim3(unsigned((pixels + 255) / 256)), dim3(256), 0, s,
                     static_cast<const float*>(rgb), rgba, pixels);
}

void launch_blend_backward(const BlendBackwardArgs& a, const BlendLaunch& l, cudaStream_t s) {
    if (a.n_tiles == 0) return;
    const int sms = l.num_sms > 0 ? l.num_sms : 148;
    switch (l.backward_round) {
        case 32:
            l.persistent ? launch_blend_backward_t<32, true>(a, sms, s) : launch_blend_backward_t<32, false>(a, sms, s);
            break;
        case 128:
            l.persistent ? launch_blend_backward_t<128, true>(a, sms, s)
                         : launch_blend_backward_t<128, false>(a, sms, s);
            break;
        default:
            l.persistent ? launch_blend_backward_t<64, true>(a, sms, s) : launch_blend_backward_t<64, false>(a, sms, s);
            break;
    }
}

}  // namespace tpd
