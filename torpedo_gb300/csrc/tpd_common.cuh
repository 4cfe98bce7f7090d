// tpd_common.cuh — shared device-side definitions for the splatting kernels.
//
// Layouts shared with the reference (paths relative to its project root):
//   Gaussian record, 240 B  : splat.slang:24-31, GaussianGeometry.h:10-18
//   Splat, 48 B             : splat.slang:33-39
//   16x16 tiles, 256-wide   : splat.slang:7-9, GaussianEngine.h:121-124
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tpdsplat.h"

namespace tpd {

constexpr uint32_t kBlockX = 16;          // tile width in pixels
constexpr uint32_t kBlockY = 16;          // tile height in pixels
constexpr uint32_t kTilePixels = kBlockX * kBlockY;
constexpr uint32_t kRecordFloats = 60;    // 240-byte Gaussian record
constexpr uint32_t kRecordBytes = 240;

// Status bits written by kernels to the device status word (never traps).
constexpr uint32_t kStatusKeyOverflow = 1u << 0;     // more keys than key capacity
constexpr uint32_t kStatusLookbackTimeout = 1u << 1; // a decoupled look-back spin ran out
constexpr uint32_t kStatusMbarTimeout = 1u << 2;     // reserved: no kernel waits on an mbarrier
constexpr uint32_t kStatusBadInput = 1u << 3;        // an input outside the documented range
constexpr uint32_t kStatusBadIndex = 1u << 4;        // checked builds: an index failed its bounds check
// Statuses after which the rest of the frame is skipped (its lists are unusable).
constexpr uint32_t kStatusFatal = kStatusLookbackTimeout | kStatusMbarTimeout;
static_assert(kStatusKeyOverflow == TPD_DEVSTAT_KEY_OVERFLOW && kStatusLookbackTimeout == TPD_DEVSTAT_LOOKBACK_TIMEOUT &&
                  kStatusBadInput == TPD_DEVSTAT_BAD_INPUT && kStatusBadIndex == TPD_DEVSTAT_BAD_INDEX,
              "device status bits as the C ABI documents them");

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

// 16-byte asynchronous copy global -> shared (cp.async, L2 only), grouped
// by cp_async_commit and completed by the hardware waits below: a thread
// waits for its own copies; a barrier afterwards publishes them to the CTA.
// Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Every committed group of this thread but the newest has completed.
__device__ __forceinline__ void cp_async_wait_all_but_newest() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
// Every committed group of this thread has completed.
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Programmatic dependent launch (launch_dependent below). pdl_trigger: this
// CTA allows the stream's next kernel to be scheduled (once every CTA of this
// grid has done so or exited, so all of them are resident by then).
// pdl_wait: blocks until the grids this one depends on have completed and
// their memory is visible (hardware-managed, like a kernel boundary); reads of
// their results come after it. Both are no-ops in a kernel launched without
// the attribute.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launches kernel on s as a programmatic dependent of the kernel before it on
// the stream: it may start while that kernel's last CTAs run, and must
// pdl_wait() before it reads what that kernel writes.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                    Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
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
// ((p - r) / 16) and (p + r + 16 - 1) / 16, the latter two rounded additions
// ((p + r) + 16) then a rounded subtraction of 1, left to right as the shader
// writes p + r + BLOCK_X - 1 (which can differ from (p + r) + 15 when p + r + 16
// crosses a power of two), truncated toward zero and clamped to the grid.
// Dividing by 16 is multiplying by 2^-4: both round the same exact quotient,
// so the product gives the division's result bit for bit.
static_assert(kBlockX == 16 && kBlockY == 16, "the tile rect divides by 16 as a multiply by 2^-4");
__device__ __forceinline__ void bounding_rect(float px, float py, float radius, uint32_t gx, uint32_t gy,
                                              uint32_t& x0, uint32_t& y0, uint32_t& x1, uint32_t& y1) {
    const float inv = 0.0625f, bx = float(kBlockX);
    const int a = trunc_to_int(__fmul_rn(__fsub_rn(px, radius), inv));
    const int b = trunc_to_int(__fmul_rn(__fsub_rn(py, radius), inv));
    const int c = trunc_to_int(__fmul_rn(__fsub_rn(__fadd_rn(__fadd_rn(px, radius), bx), 1.0f), inv));
    const int d = trunc_to_int(__fmul_rn(__fsub_rn(__fadd_rn(__fadd_rn(py, radius), bx), 1.0f), inv));
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
