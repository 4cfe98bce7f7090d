// blend.cu — kernel (e): per-tile front-to-back alpha blending, and its adjoint.
//
// Reference: blend.slang:24-105 (one 16x16 workgroup per tile; rounds of 256
// splats staged in shared memory; per pixel: power, alpha = min(0.99,
// o*exp(power)), skip below 1/255, stop when T*(1-alpha) < 1e-4; colour
// gathered per contributing pair) dispatched by GaussianEngine.cpp:857-862.
// The reference has no backward pass; blend_backward_kernel is new.
//
// GB300 form: one CTA per tile; each round stages position, conic+opacity
// and colour of the next list entries into shared memory (colour is staged
// with the rest instead of gathered per pair), the whole CTA leaves as soon
// as every pixel is done (__syncthreads_count), and per pixel the final
// transmittance and the number of list entries up to the last contributor
// are kept for the adjoint. The forward runs 128 threads with two pixels per
// lane, whose pair arithmetic uses packed f32x2 operations. The adjoint (256
// threads, one pixel each) walks each tile's list back to front, recomputing
// transmittance as T / (1 - alpha) from the final T (no per-pixel lists), and
// accumulates per-Gaussian gradients warp-reduced, then in shared memory,
// then with one global atomic per (round, Gaussian, field).
//
// Every per-pixel operation (p2, alpha, the skip and stop tests) has the same
// operations and explicit rounding in the forward and in the adjoint, so both
// take identical decisions.
//
// Warp culling: a warp owns a pixel block of the tile (8x8 in the forward,
// 8x4 in the adjoint). The thread that stages a list entry also works out,
// once for the whole CTA, which of the tile's blocks the entry can reach: for
// each block row (a slab of pixel rows) it takes the x extent of the entry's
// alpha >= 1/255 ellipse within the slab (closed form, two square roots),
// enlarged for rounding, and compares it with the two block columns. A warp
// then walks only the entries whose bit for its block is set (one ballot per
// 32 entries). A culled pair lies outside that ellipse, where the pair's own
// test finds alpha below 1/255 and skips it, as the reference does; so the
// culling changes which skipped pairs are visited, never a result, and the
// forward and the adjoint may use different blocks.
#include "tpd_common.cuh"
#include "tpd_kernels.h"

namespace tpd {
namespace {

constexpr uint32_t kBlendThreads = kTilePixels;  // 256
constexpr float kAlphaMax = 0.99f;
constexpr float kTMin = 0.0001f;

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;

// A list entry staged in shared memory. The conic is pre-scaled so that
//   p2 = log2(e) * power,  power = -0.5 * (cx*dx*dx + cz*dy*dy) - cy*dx*dy  (blend.slang:83-84)
// costs five multiply/fma operations, exp(power) = 2^p2 is one ex2, and
//   alpha = min(0.99, o * 2^p2) < 1/255  <=>  p2 < thr = log2(1 / (255 o))
// is decided before the exponential. Forward and adjoint stage and test
// entries with the same functions, so they take identical decisions.
//   xy    px, py
//   q     qa = -0.5 log2e cx, qb = -log2e cy, qc = -0.5 log2e cz, thr
//   col   r, g, b, opacity
//   mask  bit w: the entry can reach alpha >= 1/255 in warp w's 8x4 block

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

__device__ __forceinline__ void stage_entry(const Splat* sp, float ox, float oy, float2& xy, float4& q, float4& col,
                                            uint8_t& mask) {
    const float4* p = reinterpret_cast<const float4*>(sp);
    const float4 c = __ldg(p + 0), tex = __ldg(p + 1), co = __ldg(p + 2);
    xy = make_float2(tex.x, tex.y);
    const float thr = co.w > 0.0f ? -__log2f(255.0f * co.w) : kInf;  // +inf: never blends
    q = make_float4(-0.5f * kLog2e * co.x, -kLog2e * co.y, -0.5f * kLog2e * co.z, thr);
    col = make_float4(c.x, c.y, c.z, co.w);
    mask = uint8_t(block_mask<4>(tex.x, tex.y, q, ox, oy));
}

__device__ __forceinline__ void stage_empty(float2& xy, float4& q, float4& col, uint8_t& mask) {
    xy = make_float2(0.f, 0.f);
    q = make_float4(0.f, 0.f, 0.f, kInf);
    col = make_float4(0.f, 0.f, 0.f, 0.f);
    mask = 0u;
}

// Pixel of thread tid within its tile, and the 8x4 block of its warp.
__device__ __forceinline__ void warp_block_pixel(uint32_t tid, uint32_t& lx, uint32_t& ly, uint32_t& bx, uint32_t& by) {
    const uint32_t warp = tid >> 5, lane = tid & 31u;
    bx = 8u * (warp & 1u);
    by = 4u * (warp >> 1);
    lx = bx + (lane & 7u);
    ly = by + (lane >> 3);
}

__device__ __forceinline__ float pair_p2(float2 xy, float4 q, float pxf, float pyf, float& dx, float& dy) {
    dx = __fsub_rn(xy.x, pxf);
    dy = __fsub_rn(xy.y, pyf);
    const float t = __fmaf_rn(q.y, dy, __fmul_rn(q.x, dx));
    return __fmaf_rn(t, dx, __fmul_rn(__fmul_rn(q.z, dy), dy));
}

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// true when the pair is skipped (power > 0 or alpha < 1/255)
__device__ __forceinline__ bool pair_skipped(float p2, float thr) { return p2 > 0.0f || p2 < thr; }

__device__ __forceinline__ void load_view_tile(const BlendArgs* /*unused*/, const ViewConst* views,
                                               const uint32_t* tile_view, uint32_t tile, uint32_t& vi,
                                               uint32_t& width, uint32_t& height, uint32_t& tx, uint32_t& ty) {
    vi = tile_view ? tile_view[tile] : 0u;
    const ViewConst& v = views[vi];
    width = v.width;
    height = v.height;
    const uint32_t local = tile - v.tile_base;
    const uint32_t gx = grid_x(width);
    tx = local % gx;
    ty = local / gx;
}

// Staging buffers of the adjoint: list entry tid of a round in slot tid.
struct BlendStage {
    float2 xy[2][kBlendThreads];
    float4 q[2][kBlendThreads];
    float4 col[2][kBlendThreads];
    uint8_t mask[2][kBlendThreads];
};

// ---- forward
//
// A CTA of 128 threads per tile. Warp w owns the 8x8 block at (8 (w & 1),
// 8 (w >> 1)) of the tile, and lane l the two pixels (l & 7, l >> 3) and
// (l & 7, (l >> 3) + 4) of that block. The two pixels of a lane share dx, and
// the arithmetic of a (pixel, entry) pair runs on both pixels at once with
// packed f32x2 operations: per pixel the same operations, in the same order
// and rounding, as the scalar form in pair_p2 and the adjoint. A staged entry
// holds its values duplicated in register-pair order, so the packed operands
// come straight out of five broadcast shared-memory loads.
constexpr uint32_t kFwdThreads = 128;
// 128 list entries per staged round (20 KB of shared memory) and at most 64
// registers: 8 CTAs (32 warps) per SM, measured faster than 256-entry rounds
// at 5 CTAs, 64-entry rounds, or 10 CTAs at 48 registers
constexpr uint32_t kRound = 128;
constexpr uint32_t kFwdMinBlocks = 8;

struct PairStaged {  // 80 bytes
    float4 xy;       // x, x, y, y
    float4 qab;      // qa, qa, qb, qb
    float4 qco;      // qc, qc, opacity, opacity
    float4 rg;       // r, r, g, g
    float4 bt;       // b, b, thr, 0
};

struct FwdStage {
    PairStaged e[2][kRound];
    uint8_t mask[2][kRound];  // bit w: the entry can reach warp w's 8x8 block
};

__device__ __forceinline__ void stage_pair_entry(const Splat* sp, float ox, float oy, PairStaged& d, uint8_t& mask) {
    const float4* p = reinterpret_cast<const float4*>(sp);
    const float4 c = __ldg(p + 0), tex = __ldg(p + 1), co = __ldg(p + 2);
    const float thr = co.w > 0.0f ? -__log2f(255.0f * co.w) : kInf;  // +inf: never blends
    const float4 q = make_float4(-0.5f * kLog2e * co.x, -kLog2e * co.y, -0.5f * kLog2e * co.z, thr);
    d.xy = make_float4(tex.x, tex.x, tex.y, tex.y);
    d.qab = make_float4(q.x, q.x, q.y, q.y);
    d.qco = make_float4(q.z, q.z, co.w, co.w);
    d.rg = make_float4(c.x, c.x, c.y, c.y);
    d.bt = make_float4(c.z, c.z, thr, 0.0f);
    mask = uint8_t(block_mask<2>(tex.x, tex.y, q, ox, oy));
}

__device__ __forceinline__ void stage_pair_empty(PairStaged& d, uint8_t& mask) {
    d.xy = d.qab = d.qco = d.rg = make_float4(0.f, 0.f, 0.f, 0.f);
    d.bt = make_float4(0.f, 0.f, kInf, 0.f);
    mask = 0u;
}

// Rounds of kRound list entries, double-buffered: while the warps walk round
// r, each thread stages its entry of round r + 1 into the other buffer, and
// one barrier per round (which also counts finished pixels) separates the
// two.
__global__ void __launch_bounds__(kFwdThreads, kFwdMinBlocks) blend_kernel(BlendArgs a) {
    __shared__ FwdStage S;

    const uint32_t tile = blockIdx.x;
    // an overflowed frame is re-rendered with larger key buffers; nothing to draw
    if (a.ctl->status & (kStatusFatal | kStatusKeyOverflow)) return;
    uint32_t vi, W, H, tx, ty;
    load_view_tile(nullptr, a.views, a.tile_view, tile, vi, W, H, tx, ty);
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

    bool done_a = !in_a, done_b = !in_b;
    float2 T = make_float2(1.0f, 1.0f), C0 = make_float2(0.f, 0.f), C1 = C0, C2 = C0;
    uint32_t last_a = 0, last_b = 0;
    const float2 one = make_float2(1.0f, 1.0f), mone = make_float2(-1.0f, -1.0f);
    if (start < end) stage(0, start);
    bool all_done = __syncthreads_count(done_a && done_b) == kFwdThreads;
    uint32_t r = 0;
    for (uint32_t b0 = start; b0 < end && !all_done; b0 += kRound, ++r) {
        const uint32_t b = r & 1u;
        // the next round's entries, into the buffer the last barrier released
        if (b0 + kRound < end) stage(b ^ 1u, b0 + kRound);
        const uint32_t n = min(kRound, end - b0);
        const uint32_t lbase = b0 - start + 1u;  // n_contrib of entry jj of this round: lbase + jj
        for (uint32_t g = 0; g < n; g += 32) {
            if (__all_sync(0xFFFFFFFFu, done_a && done_b)) break;
            const uint32_t e = g + lane;
            uint32_t m = __ballot_sync(0xFFFFFFFFu, e < n && ((S.mask[b][e] >> warp) & 1u));
            // branch-free body: every lane evaluates both pairs and selects
            // the update, so lanes taking different decisions do not run the
            // paths one after another. A skipped pair gets alpha = 0, which
            // leaves T and C exactly as they were.
            while (m) {
                const uint32_t jj = g + uint32_t(__ffs(m) - 1);
                m &= m - 1u;
                const PairStaged& E = S.e[b][jj];
                const float4 xy = E.xy, qab = E.qab, qco = E.qco, rg = E.rg, bt = E.bt;
                // pair_p2 for both pixels: dx = x - px, dy = y - py,
                // p2 = fma(fma(qb, dy, qa dx), dx, (qc dy) dy)
                const float2 dx = __fadd2_rn(make_float2(xy.x, xy.y), npx);
                const float2 dy = __fadd2_rn(make_float2(xy.z, xy.w), npy);
                const float2 t = __ffma2_rn(make_float2(qab.z, qab.w), dy, __fmul2_rn(make_float2(qab.x, qab.y), dx));
                const float2 p2 = __ffma2_rn(t, dx, __fmul2_rn(__fmul2_rn(make_float2(qco.x, qco.y), dy), dy));
                const float2 ao =
                    __fmul2_rn(make_float2(qco.z, qco.w), make_float2(ex2_approx(p2.x), ex2_approx(p2.y)));
                const bool skip_a = done_a || pair_skipped(p2.x, bt.z);
                const bool skip_b = done_b || pair_skipped(p2.y, bt.z);
                const float2 alpha = make_float2(skip_a ? 0.0f : fminf(kAlphaMax, ao.x),
                                                 skip_b ? 0.0f : fminf(kAlphaMax, ao.y));
                const float2 tn = __fmul2_rn(T, __ffma2_rn(mone, alpha, one));  // T (1 - alpha)
                const bool term_a = tn.x < kTMin, term_b = tn.y < kTMin;  // false when skipped: tn = T
                const bool add_a = !skip_a && !term_a, add_b = !skip_b && !term_b;
                done_a = done_a || term_a;
                done_b = done_b || term_b;
                const float2 aT = __fmul2_rn(alpha, T);
                const float2 w = make_float2(term_a ? 0.0f : aT.x, term_b ? 0.0f : aT.y);
                C0 = __ffma2_rn(make_float2(rg.x, rg.y), w, C0);
                C1 = __ffma2_rn(make_float2(rg.z, rg.w), w, C1);
                C2 = __ffma2_rn(make_float2(bt.x, bt.y), w, C2);
                T = make_float2(term_a ? T.x : tn.x, term_b ? T.y : tn.y);
                last_a = add_a ? lbase + jj : last_a;
                last_b = add_b ? lbase + jj : last_b;
            }
        }
        all_done = __syncthreads_count(done_a && done_b) == kFwdThreads;
    }
    if (TPD_INBOUNDS(a.ctl, 41, tile, a.n_tiles)) {
        const size_t img0 = a.image_offset ? a.image_offset[vi] : 0ull;
        if (in_a) {
            const size_t p = img0 + size_t(pya) * W + px;
            a.image[p * 3 + 0] = C0.x;
            a.image[p * 3 + 1] = C1.x;
            a.image[p * 3 + 2] = C2.x;
            if (a.final_T) a.final_T[p] = T.x;
            if (a.n_contrib) a.n_contrib[p] = last_a;
        }
        if (in_b) {
            const size_t p = img0 + size_t(pyb) * W + px;
            a.image[p * 3 + 0] = C0.y;
            a.image[p * 3 + 1] = C1.y;
            a.image[p * 3 + 2] = C2.y;
            if (a.final_T) a.final_T[p] = T.y;
            if (a.n_contrib) a.n_contrib[p] = last_b;
        }
    }
}

// UNORM conversion of (r, g, b, 1): round(clamp(c, 0, 1) * 255).
__global__ void pack_rgba8_kernel(const float* rgb, uint32_t* rgba, size_t pixels) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= pixels) return;
    uint32_t out = 0xFF000000u;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float v = fminf(fmaxf(rgb[i * 3 + c], 0.0f), 1.0f);
        out |= uint32_t(__float2uint_rn(v * 255.0f)) << (8 * c);
    }
    rgba[i] = out;
}

__device__ __forceinline__ float warp_red(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
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

// Rounds of 256 list entries from the back, as in the forward: staging
// double-buffered, per-round gradient sums in one of two shared buffers. The
// barrier at the end of a round completes its sums; each thread then adds its
// share of them to global memory and zeroes what it added, so the buffer is
// clean when it comes round again two rounds later. The staged indices that
// the flush reads live in three buffers (the next round's staging overwrites
// the one of the round before the last).
struct BlendBackwardSmem {
    BlendStage stage;
    float acc[2][kBlendThreads][kG2DStride];
    uint32_t idx[3][kBlendThreads];
};

__global__ void __launch_bounds__(kBlendThreads) blend_backward_kernel(BlendBackwardArgs a) {
    extern __shared__ __align__(16) unsigned char bwd_smem[];
    BlendBackwardSmem& SM = *reinterpret_cast<BlendBackwardSmem*>(bwd_smem);
    BlendStage& S = SM.stage;
    auto& s_idx = SM.idx;
    auto& s_acc = SM.acc;

    const uint32_t tile = blockIdx.x;
    if (a.ctl->status & (kStatusFatal | kStatusKeyOverflow)) return;  // no valid frame to differentiate
    uint32_t vi, W, H, tx, ty;
    load_view_tile(nullptr, a.views, a.tile_view, tile, vi, W, H, tx, ty);
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    uint32_t lx, ly, bx, by;
    warp_block_pixel(tid, lx, ly, bx, by);
    const uint32_t pxl = tx * kBlockX + lx, pyl = ty * kBlockY + ly;
    const float ox = float(tx * kBlockX), oy = float(ty * kBlockY);
    const uint32_t warp = tid >> 5;
    const bool inside = pxl < W && pyl < H;
    const float pxf = float(pxl), pyf = float(pyl);
    const uint32_t K = min(a.ctl->total_keys, a.capacity);
    const uint32_t end = min(a.ranges[tile * 2 + 1], K), start = min(a.ranges[tile * 2 + 0], end);
    const Splat* vsplats = a.splats + size_t(vi) * a.n;

    const size_t p = (a.image_offset ? a.image_offset[vi] : 0ull) + size_t(pyl) * W + pxl;
    float T = 1.0f, g0 = 0.f, g1 = 0.f, g2 = 0.f;
    uint32_t last = 0;
    if (inside) {
        T = a.final_T[p];
        last = min(a.n_contrib[p], end - start);
        g0 = a.dL_dimage[p * 3 + 0];
        g1 = a.dL_dimage[p * 3 + 1];
        g2 = a.dL_dimage[p * 3 + 2];
    }
    // the block walks back from the largest last-contributor index over its
    // pixels; a warp takes entries below its own largest index only
    uint32_t warp_last = last;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) warp_last = max(warp_last, __shfl_xor_sync(0xFFFFFFFFu, warp_last, o));
    __shared__ uint32_t s_max[kBlendThreads / 32];
    if (lane == 0) s_max[tid >> 5] = warp_last;
    __syncthreads();
    uint32_t max_last = 0;
#pragma unroll
    for (uint32_t w = 0; w < kBlendThreads / 32; ++w) max_last = max(max_last, s_max[w]);

    float S0 = 0.f, S1 = 0.f, S2 = 0.f;  // colour accumulated behind the current entry
    float* g2d_view = a.g2d + size_t(vi) * a.g2d_view_stride;
    // stages the round whose list positions (relative) end at r_end: entry
    // tid is position r_end - 1 - tid
    auto stage_round = [&](int32_t r_end, uint32_t b, uint32_t bi) {
        const uint32_t n = uint32_t(min(int32_t(kBlendThreads), r_end));
        if (tid < n) {
            const uint32_t e = uint32_t(r_end) - 1u - tid;
            uint32_t idx = a.vals[start + e];
            if (idx < a.n) {
                stage_entry(vsplats + idx, ox, oy, S.xy[b][tid], S.q[b][tid], S.col[b][tid], S.mask[b][tid]);
            } else {  // only reachable with corrupted lists
                idx = 0;
                stage_empty(S.xy[b][tid], S.q[b][tid], S.col[b][tid], S.mask[b][tid]);
            }
            s_idx[bi][tid] = idx;
        }
    };
    for (uint32_t k = tid; k < 2 * kBlendThreads * kG2DStride; k += kBlendThreads) (&s_acc[0][0][0])[k] = 0.f;
    if (max_last > 0) stage_round(int32_t(max_last), 0, 0);
    __syncthreads();
    uint32_t r = 0;
    for (int32_t r_end = int32_t(max_last); r_end > 0; r_end -= int32_t(kBlendThreads), ++r) {
        const uint32_t b = r & 1u, bi = r % 3u;
        const uint32_t n = uint32_t(min(int32_t(kBlendThreads), r_end));
        if (r_end > int32_t(kBlendThreads)) stage_round(r_end - int32_t(kBlendThreads), b ^ 1u, (r + 1) % 3u);
        // entries jj >= skip have list positions r_end - 1 - jj below warp_last
        const uint32_t skip = uint32_t(r_end) > warp_last ? uint32_t(r_end) - warp_last : 0u;
        for (uint32_t g = skip & ~31u; g < n; g += 32) {
            const uint32_t jl = g + lane;
            uint32_t m = __ballot_sync(0xFFFFFFFFu, jl < n && jl >= skip && ((S.mask[b][jl] >> warp) & 1u));
            while (m) {
                const uint32_t jj = g + uint32_t(__ffs(m) - 1);
                m &= m - 1u;
                const uint32_t e = uint32_t(r_end) - 1u - jj;
                // branch-free body (as in the forward): every lane evaluates,
                // the selects keep only contributing pairs
                float dx, dy;
                const float4 q = S.q[b][jj];
                const float p2 = pair_p2(S.xy[b][jj], q, pxf, pyf, dx, dy);
                const float4 col = S.col[b][jj];
                const bool contrib = inside && e < last && !pair_skipped(p2, q.w);
                const float G = ex2_approx(p2);
                const float raw = __fmul_rn(col.w, G);
                const float alpha = fminf(kAlphaMax, raw);
                const float inv = __fdividef(1.0f, 1.0f - alpha);  // 1 - alpha >= 0.01
                const float Tb = T * inv;  // transmittance in front of this entry
                // zero weight and gradient scale for pairs that do not count:
                // every term below is finite, so it adds exactly nothing
                const float w = contrib ? alpha * Tb : 0.0f;
                const float dA = g0 * (col.x * Tb - S0 * inv) + g1 * (col.y * Tb - S1 * inv) +
                                 g2 * (col.z * Tb - S2 * inv);
                S0 = fmaf(col.x, w, S0);
                S1 = fmaf(col.y, w, S1);
                S2 = fmaf(col.z, w, S2);
                T = contrib ? Tb : T;
                // power = p2 ln2; d power / d(dx, dy) = ln2 (2 qa dx + qb dy, 2 qc dy + qb dx)
                const bool unclamped = contrib && raw <= kAlphaMax;
                const float dpow = unclamped ? dA * alpha : 0.0f;
                float gv[kG2D];
                gv[0] = dpow * kLn2 * (2.0f * q.x * dx + q.y * dy);
                gv[1] = dpow * kLn2 * (2.0f * q.z * dy + q.y * dx);
                gv[2] = dpow * (-0.5f * dx * dx);
                gv[3] = dpow * (-dx * dy);
                gv[4] = dpow * (-0.5f * dy * dy);
                gv[5] = unclamped ? dA * G : 0.0f;
                gv[6] = g0 * w;
                gv[7] = g1 * w;
                gv[8] = g2 * w;
                if (__any_sync(0xFFFFFFFFu, contrib)) {
                    const float lo[8] = {gv[0], gv[1], gv[2], gv[3], gv[4], gv[5], gv[6], gv[7]};
                    const float rs = warp_sum8_transposed(lo, lane);
                    float b9 = gv[8];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) b9 += __shfl_xor_sync(0xFFFFFFFFu, b9, o);
                    if ((lane & 3u) == 0) atomicAdd(&s_acc[b][jj][lane >> 2], rs);
                    if (lane == 0) atomicAdd(&s_acc[b][jj][8], b9);
                }
            }
        }
        __syncthreads();  // round r's sums complete; the other stage buffer is filled
        // one 16-byte vector atomic per non-zero quarter of an entry's record;
        // the thread that adds a quarter also zeroes it for round r + 2
        for (uint32_t k = tid; k < n * 3; k += kBlendThreads) {
            const uint32_t jj = k / 3, c = k % 3;
            float4* slot = reinterpret_cast<float4*>(&s_acc[b][jj][0]) + c;
            const float4 v = *slot;
            if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f) {
                atomicAdd(reinterpret_cast<float4*>(g2d_view + size_t(s_idx[bi][jj]) * kG2DStride) + c, v);
                *slot = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    }
}

}  // namespace

void launch_blend(const BlendArgs& a, cudaStream_t s) {
    if (a.n_tiles == 0) return;
    blend_kernel<<<a.n_tiles, kFwdThreads, 0, s>>>(a);
}

void launch_pack_rgba8(const float* rgb, uint32_t* rgba, size_t pixels, cudaStream_t s) {
    if (pixels == 0) return;
    pack_rgba8_kernel<<<unsigned((pixels + 255) / 256), 256, 0, s>>>(rgb, rgba, pixels);
}

void launch_blend_backward(const BlendBackwardArgs& a, cudaStream_t s) {
    if (a.n_tiles == 0) return;
    static bool configured = false;  // more than 48 KB of shared memory needs the opt-in
    if (!configured) {
        cudaFuncSetAttribute(blend_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(sizeof(BlendBackwardSmem)));
        configured = true;
    }
    blend_backward_kernel<<<a.n_tiles, kBlendThreads, sizeof(BlendBackwardSmem), s>>>(a);
}

}  // namespace tpd
