// tpd_common.cuh — shared device-side definitions for the splatting kernels.
//
// Layouts shared with the reference (paths relative to its project root):
//   Gaussian record, 240 B  : splat.slang:24-31, GaussianGeometry.h:10-18
//   Splat, 48 B             : splat.slang:33-39
//   16x16 tiles, 256-wide   : splat.slang:7-9, GaussianEngine.h:121-124
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tpd {

constexpr uint32_t kBlockX = 16;          // tile width in pixels
constexpr uint32_t kBlockY = 16;          // tile height in pixels
constexpr uint32_t kTilePixels = kBlockX * kBlockY;
constexpr uint32_t kRecordFloats = 60;    // 240-byte Gaussian record
constexpr uint32_t kRecordBytes = 240;

// Status bits written by kernels to the device status word (never traps).
constexpr uint32_t kStatusKeyOverflow = 1u << 0;     // more keys than key capacity
constexpr uint32_t kStatusLookbackTimeout = 1u << 1; // a decoupled look-back spin ran out
constexpr uint32_t kStatusMbarTimeout = 1u << 2;     // a TMA mbarrier wait ran out
constexpr uint32_t kStatusBadInput = 1u << 3;        // an input outside the documented range
constexpr uint32_t kStatusBadIndex = 1u << 4;        // checked builds: an index failed its bounds check
// Statuses after which the rest of the frame is skipped (its lists are unusable).
constexpr uint32_t kStatusFatal = kStatusLookbackTimeout | kStatusMbarTimeout;

// Splat record: color[3], tiles, texel = (px, py, viewZ, radius), copac = (conic.xyz, opacity).
struct __align__(16) Splat {
    float r, g, b;
    uint32_t tiles;
    float px, py, depth, radius;
    float cx, cy, cz, opacity;
};
static_assert(sizeof(Splat) == 48, "Splat must be 48 bytes");

// Camera constants of one view, as updateCameraBuffer packs them
// (GaussianEngine.cpp:764-775) plus the image size.
struct ViewConst {
    float view[16];      // world -> view, row-major
    float projview[16];  // proj * view, row-major
    float focal[2];      // (P00, P11)
    uint32_t width, height;
    uint32_t tile_base;  // first global tile id of this view (batched form)
    uint32_t pad[3];
};

__host__ __device__ inline uint32_t grid_x(uint32_t w) { return (w + kBlockX - 1) / kBlockX; }
__host__ __device__ inline uint32_t grid_y(uint32_t h) { return (h + kBlockY - 1) / kBlockY; }

// ---------------------------------------------------------------------------
// PTX helpers (sm_90+ forms, used on sm_103a).

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// One-dimensional bulk copy global -> shared, completing on an mbarrier.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase. Returns false (and sets the status bit)
// when the limit runs out; the caller then skips the staged data.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t* status,
                                                  uint32_t limit = (1u << 20)) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, phase)) return true;
    atomicOr(status, kStatusMbarTimeout);
    return false;
}

// Relaxed, device-scope 64-bit load / store: single-copy atomic, used for
// self-contained look-back descriptors (flag + tag + value in one word).
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Look-back descriptor: [63:62] flag, [61:32] tag, [31:0] value.
// The tag identifies the launch that wrote it, so descriptors never need
// clearing between launches: a stale tag reads as "not yet published".
constexpr uint64_t kFlagAggregate = 1ull;
constexpr uint64_t kFlagPrefix = 2ull;
__device__ __forceinline__ uint64_t make_desc(uint64_t flag, uint32_t tag, uint32_t value) {
    return (flag << 62) | (uint64_t(tag & 0x3FFFFFFFu) << 32) | value;
}
__device__ __forceinline__ uint32_t desc_flag(uint64_t d, uint32_t tag) {
    return (uint32_t((d >> 32) & 0x3FFFFFFFu) == (tag & 0x3FFFFFFFu)) ? uint32_t(d >> 62) : 0u;
}

// (int) conversion of the shaders: truncation toward zero, saturated
// (cvt.rzi.s32.f32 saturates; NaN -> 0).
__device__ __forceinline__ int trunc_to_int(float v) { return __float2int_rz(v); }

// getBoundingRect (splat/volume.slang:12-17). Same float operations as the shader:
// ((p - r) / 16) and ((p + r) + 15) / 16, truncated toward zero, clamped to the grid.
// Dividing by 16 is multiplying by 2^-4: both round the same exact quotient,
// so the product gives the division's result bit for bit.
static_assert(kBlockX == 16, "the tile rect divides by 16 as a multiply by 2^-4");
__device__ __forceinline__ void bounding_rect(float px, float py, float radius, uint32_t gx, uint32_t gy,
                                              uint32_t& x0, uint32_t& y0, uint32_t& x1, uint32_t& y1) {
    const float inv = 0.0625f, b1 = float(kBlockX - 1);
    const int a = trunc_to_int(__fmul_rn(__fsub_rn(px, radius), inv));
    const int b = trunc_to_int(__fmul_rn(__fsub_rn(py, radius), inv));
    const int c = trunc_to_int(__fmul_rn(__fadd_rn(__fadd_rn(px, radius), b1), inv));
    const int d = trunc_to_int(__fmul_rn(__fadd_rn(__fadd_rn(py, radius), b1), inv));
    x0 = min(gx, uint32_t(max(0, a)));
    y0 = min(gy, uint32_t(max(0, b)));
    x1 = min(gx, uint32_t(max(0, c)));
    y1 = min(gy, uint32_t(max(0, d)));
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// TPD_INBOUNDS(ctl, site, index, bound) guards a computed index: when
// index >= bound it records (site, index, bound) of the first such event in
// ctl->debug, raises kStatusBadIndex (the host reports it as an error) and
// returns false so the caller skips the access. Always compiled in: one
// compare per guarded access, and inconsistent lists end in an error status
// instead of an out-of-bounds access.
template <typename Ctl>
__device__ __forceinline__ bool tpd_inbounds(Ctl* ctl, uint32_t site, uint64_t index, uint64_t bound) {
    if (index < bound) return true;
    if (atomicOr(&ctl->status, kStatusBadIndex) & kStatusBadIndex) return false;
    ctl->debug[0] = site;
    ctl->debug[1] = uint32_t(index);
    ctl->debug[2] = uint32_t(bound);
    ctl->debug[3] = uint32_t(index >> 32);
    return false;
}
#define TPD_INBOUNDS(ctl, site, index, bound) ::tpd::tpd_inbounds((ctl), (site), (index), (bound))

}  // namespace tpd
