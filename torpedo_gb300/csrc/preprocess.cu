// preprocess.cu — kernel (a): per-Gaussian projection to a 48-byte Splat, the
// depth-sort input, and the tile-count exclusive scan (b, first half).
//
// Reference: project.slang:33-107 with splat/common.slang (SH, frustum test,
// camera position) and splat/volume.slang (ndc2pix, bounding rect, 3D
// covariance, EWA projection, Jacobian); prefix.slang:40-158 for the scan.
//
// GB300 layout: a CTA of 128 threads owns 128 consecutive records (30,720 B).
// The CTA stages them into shared memory with coalesced 16-byte asynchronous
// copies (cp.async, 15 per thread), double-buffered so the next chunk streams
// in while this one is projected; threads then read their record with
// conflict-free 16-byte loads (record stride 60 words). The copies complete
// by a hardware wait (cp.async.wait_group), not a software spin, so no wait
// can give up with a copy in flight, and the CTA drains every copy it issued
// before it exits. Besides the splat, each (view, Gaussian) gets a
// depth-sort key (view << 32 | bits(viewZ)) whose digit histograms are
// accumulated here, and the digits of the tile ids its keys will carry are
// counted from its tile rectangle for the key sort (count_tile_row). The tile
// counts are scanned afterwards in depth order, inside keygen.cu's fused scan
// and key duplication (scan_tiles_kernel is the standalone scan). Arithmetic
// follows the shader source left to right with matrix products accumulated
// k = 0..n-1; this file is compiled with --fmad=false so no product is fused
// into an add.
#include <algorithm>

#include "tpd_common.cuh"
#include "tpd_kernels.h"
#include "tpd_scan.cuh"

namespace tpd {
namespace {

constexpr uint32_t kPreThreads = 128;

// SH constants (splat/common.slang:3-20).
__constant__ float cSH_C0 = 0.28209479177387814f;
__constant__ float cSH_C1 = 0.4886025119029199f;
__constant__ float cSH_C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                                -1.0925484305920792f, 0.5462742152960396f};
__constant__ float cSH_C3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                                0.3731763325901154f, -0.4570457994644658f, 1.445305721320277f,
                                -0.5900435899266435f};

__device__ __forceinline__ void mat4mul(const float* A, const float* B, float* C) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            C[i * 4 + j] = A[i * 4 + 0] * B[0 * 4 + j] + A[i * 4 + 1] * B[1 * 4 + j] +
                           A[i * 4 + 2] * B[2 * 4 + j] + A[i * 4 + 3] * B[3 * 4 + j];
}

__device__ __forceinline__ void mat3mul(const float* A, const float* B, float* C) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            C[i * 3 + j] = A[i * 3 + 0] * B[0 * 3 + j] + A[i * 3 + 1] * B[1 * 3 + j] + A[i * 3 + 2] * B[2 * 3 + j];
}

__device__ __forceinline__ void mat3T(const float* A, float* B) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B[j * 3 + i] = A[i * 3 + j];
}

// frame_begin: one CTA. Clears tickets / sort histograms, advances the tag and
// computes per-entity view*model and projview*model (the products of
// passFrustumClipping, common.slang:102,106, hoisted out of the per-Gaussian loop;
// identical values since they do not depend on the Gaussian).
__global__ void frame_begin_kernel(FrameCtl* ctl, const float* transforms, uint32_t n_ent, const ViewConst* views,
                                   uint32_t n_views, float* ent_mats) {
    pdl_trigger();  // the preprocess may be scheduled; it waits for this kernel
    const uint32_t t = threadIdx.x;
    for (uint32_t i = t; i < 32; i += blockDim.x) ctl->ticket[i] = 0;
    for (uint32_t i = t; i < 8 * 256; i += blockDim.x) {
        (&ctl->sort_hist[0][0])[i] = 0;
        (&ctl->depth_hist[0][0])[i] = 0;
    }
    if (t == 0) {
        ctl->tag = ctl->tag + 1;
        ctl->status = 0;
        ctl->total_keys = 0;
        ctl->visible = 0;
        ctl->depth_count = 0;
        ctl->depth_skips = 0;
    }
    if (!views || !ent_mats) return;
    for (uint32_t ve = t; ve < n_views * n_ent; ve += blockDim.x) {
        const uint32_t v = ve / n_ent, e = ve % n_ent;
        float M[16];
        if (transforms) {
            for (int k = 0; k < 16; ++k) M[k] = transforms[size_t(e) * 16 + k];
        } else {
            for (int k = 0; k < 16; ++k) M[k] = (k % 5) == 0 ? 1.0f : 0.0f;
        }
        float V[16], P[16], VM[16], PM[16];
        for (int k = 0; k < 16; ++k) { V[k] = views[v].view[k]; P[k] = views[v].projview[k]; }
        mat4mul(V, M, VM);
        mat4mul(P, M, PM);
        float* o = ent_mats + size_t(ve) * kEntityMatFloats;
        for (int k = 0; k < 12; ++k) o[k] = VM[k];
        for (int k = 0; k < 16; ++k) o[12 + k] = PM[k];
    }
}

// Reads float k of a record staged in shared memory.
struct Rec {
    const float* p;
    __device__ __forceinline__ float operator[](int k) const { return p[k]; }
    __device__ __forceinline__ float4 f4(int q) const { return reinterpret_cast<const float4*>(p)[q]; }
};

// project() for one Gaussian. Returns the tile count (0 when culled) and fills
// s; rect gets the tile rectangle (x0, y0, x1, y1) when the count is not 0,
// the one key duplication derives from the stored splat's px, py and radius.
__device__ __forceinline__ uint32_t project_one(const Rec& rec, const float* em, const ViewConst& v,
                                                uint32_t deg, bool compat, Splat& s, uint4& rect) {
    s = Splat{0.f, 0.f, 0.f, 0u, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const float4 pos_op = rec.f4(0);
    const float mean[3] = {pos_op.x, pos_op.y, pos_op.z};

    // passFrustumClipping (common.slang:98-119)
    float vp[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        vp[i] = em[i * 4 + 0] * mean[0] + em[i * 4 + 1] * mean[1] + em[i * 4 + 2] * mean[2] + em[i * 4 + 3] * 1.0f;
    if (vp[2] <= 0.0f) return 0;
    float cp[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        cp[i] = em[12 + i * 4 + 0] * mean[0] + em[12 + i * 4 + 1] * mean[1] + em[12 + i * 4 + 2] * mean[2] +
                em[12 + i * 4 + 3] * 1.0f;
    const float k13 = 1.3f;
    if (cp[0] < -k13 * cp[3] || cp[0] > k13 * cp[3]) return 0;
    if (cp[1] < -k13 * cp[3] || cp[1] > k13 * cp[3]) return 0;
    if (cp[2] < 0.0f || cp[2] > cp[3]) return 0;
    const float inv_w = 1.0f / cp[3];
    const float ndc_x = cp[0] * inv_w, ndc_y = cp[1] * inv_w;

    // focal = 0.5 * imageSize * focalNDC (project.slang:55)
    const float fx = (0.5f * float(v.width)) * v.focal[0];
    const float fy = (0.5f * float(v.height)) * v.focal[1];

    // computeCovariance (volume.slang:20-41)
    const float4 q = rec.f4(1), sc = rec.f4(2);
    const float S[9] = {sc.x * sc.w, 0.f, 0.f, 0.f, sc.y * sc.w, 0.f, 0.f, 0.f, sc.z * sc.w};
    const float x = q.x, y = q.y, z = q.z, w = q.w;
    const float R[9] = {1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y - w * z), 2.0f * (x * z + w * y),
                        2.0f * (x * y + w * z), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z - w * x),
                        2.0f * (x * z - w * y), 2.0f * (y * z + w * x), 1.0f - 2.0f * (x * x + y * y)};
    float sigma[9], sigmaT[9], cov3[9];
    mat3mul(R, S, sigma);
    mat3T(sigma, sigmaT);
    mat3mul(sigma, sigmaT, cov3);

    // projectCovariance + computeJacobian (volume.slang:44-63)
    const float W3[9] = {v.view[0], v.view[1], v.view[2], v.view[4], v.view[5],
                         v.view[6], v.view[8], v.view[9], v.view[10]};
    const float f0 = fx / vp[2], f1 = fy / vp[2];
    const float t0 = vp[0] / vp[2], t1 = vp[1] / vp[2];
    const float J[9] = {f0, 0.f, -f0 * t0, 0.f, f1, -f1 * t1, 0.f, 0.f, 0.f};
    float Tm[9], TmT[9], inner[9], cov2[9];
    mat3mul(J, W3, Tm);
    mat3T(Tm, TmT);
    mat3mul(cov3, TmT, inner);
    mat3mul(Tm, inner, cov2);

    // low-pass filter and inverse (project.slang:60-66)
    const float ca = cov2[0] + 0.3f, cb = cov2[3], cc = cov2[4] + 0.3f;
    const float det = ca * cc - cb * cb;
    if (det == 0.0f) return 0;
    const float det_inv = 1.0f / det;
    const float conic0 = cc * det_inv, conic1 = -cb * det_inv, conic2 = ca * det_inv;

    // screen-space extent (project.slang:69-72)
    const float mid = 0.5f * (ca + cc);
    const float l1 = mid + sqrtf(fmaxf(0.1f, mid * mid - det));
    const float l2 = mid - sqrtf(fmaxf(0.1f, mid * mid - det));
    const float radius = ceilf(3.0f * sqrtf(fmaxf(l1, l2)));

    // ndc2pix (volume.slang:3-8) and getBoundingRect
    const float px = ((ndc_x + 1.0f) * float(v.width) - 1.0f) * 0.5f;
    const float py = ((ndc_y + 1.0f) * float(v.height) - 1.0f) * 0.5f;
    uint32_t x0, y0, x1, y1;
    bounding_rect(px, py, radius, grid_x(v.width), grid_y(v.height), x0, y0, x1, y1);
    const uint32_t touched = (x1 - x0) * (y1 - y0);
    if (touched == 0) return 0;
    rect = make_uint4(x0, y0, x1, y1);

    // camera position (common.slang:88-92) and view direction from the pre-model mean
    float campos[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        campos[i] = -(v.view[0 * 4 + i] * v.view[0 * 4 + 3] + v.view[1 * 4 + i] * v.view[1 * 4 + 3] +
                      v.view[2 * 4 + i] * v.view[2 * 4 + 3]);
    const float d0 = mean[0] - campos[0], d1 = mean[1] - campos[1], d2 = mean[2] - campos[2];
    const float len = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
    const float dx = d0 / len, dy = d1 / len, dz = d2 / len;

    // evaluateSphericalHarmonics (common.slang:35-80)
    float res[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) res[c] = cSH_C0 * rec[12 + c];
    if (deg > 0) {
        auto F = [&](int idx, int c) { return rec[12 + (idx - 1) + c * 15 + 3]; };
#pragma unroll
        for (int c = 0; c < 3; ++c)
            res[c] = res[c] - (cSH_C1 * dy) * F(1, c) + (cSH_C1 * dz) * F(2, c) - (cSH_C1 * dx) * F(3, c);
        if (deg > 1) {
            const float xx = dx * dx, yy = dy * dy, zz = dz * dz, xy = dx * dy, yz = dy * dz, zx = dz * dx;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                res[c] = res[c] + (cSH_C2[0] * xy) * F(4, c) + (cSH_C2[1] * yz) * F(5, c) +
                         (cSH_C2[2] * (2.0f * zz - xx - yy)) * F(6, c) + (cSH_C2[3] * zx) * F(7, c) +
                         (cSH_C2[4] * (xx - yy)) * F(8, c);
            if (deg > 2) {
                const float s12 = (cSH_C3[3] * dz) * (2.0f * zz - 3.0f * xx - 3.0f * yy);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float r = res[c] + ((cSH_C3[0] * dy) * (3.0f * xx - yy)) * F(9, c) +
                              ((cSH_C3[1] * xy) * dz) * F(10, c) +
                              ((cSH_C3[2] * dy) * (4.0f * zz - xx - yy)) * F(11, c);
                    if (compat) r = r + s12 + F(12, c);  // common.slang:69 as written
                    else r = r + s12 * F(12, c);
                    r = r + ((cSH_C3[4] * dx) * (4.0f * zz - xx - yy)) * F(13, c) +
                        ((cSH_C3[5] * dz) * (xx - yy)) * F(14, c) + ((cSH_C3[6] * dx) * (xx - 3.0f * yy)) * F(15, c);
                    res[c] = r;
                }
            }
        }
    }

    s.r = fmaxf(res[0] + 0.5f, 0.0f);
    s.g = fmaxf(res[1] + 0.5f, 0.0f);
    s.b = fmaxf(res[2] + 0.5f, 0.0f);
    s.tiles = touched;
    s.px = px;
    s.py = py;
    s.depth = vp[2];
    s.radius = radius;
    s.cx = conic0;
    s.cy = conic1;
    s.cz = conic2;
    s.opacity = pos_op.w;
    return touched;
}

// Persistent CTAs over chunks of kPreThreads records: while a chunk is
// projected, the next chunk's records stream into the other shared-memory
// stage (asynchronous 16-byte copies, one commit group per chunk), so HBM
// reads overlap the arithmetic.
constexpr uint32_t kPreStages = 2;
constexpr uint32_t kDepthPassesMax = 5;  // depth keys: 32 bits + log2(256 views)

constexpr uint32_t kTileDigitsMax = 4;   // tile ids: at most 32 bits

struct PreSmem {
    float rec[kPreStages][kPreThreads * kRecordFloats];  // 30,720 B per stage, 16-byte multiple
    uint32_t hist[kDepthPassesMax][256];                  // depth-key digit counts of this CTA
    // tile-id digit counts of this CTA: digit 0 as a difference array over
    // the 256 values (+ tall added to every value), the others directly
    uint32_t tdiff[257];
    uint32_t tall;
    uint32_t thist[kTileDigitsMax - 1][256];
    uint32_t kept;                                        // depth keys of visible items in this CTA
};

// Adds the w consecutive tile ids a0 .. a0 + w - 1 (one row of a Gaussian's
// tile rectangle, all below 2^tile_bits) to the CTA's digit counts of the
// key sort: digit 0 (t & 255) takes w / 256 on every value and a range of
// w % 256 values (wrapping) in the difference array; digit p >= 1 takes, for
// each value v of t >> 8p in the row, the number of ids with that value.
__device__ __forceinline__ void count_tile_row(PreSmem& S, uint32_t a0, uint32_t w, uint32_t ndig) {
    if (w >= 256u) atomicAdd(&S.tall, w >> 8);
    const uint32_t rem = w & 255u;
    if (rem) {
        const uint32_t st = a0 & 255u, e = st + rem;
        atomicAdd(&S.tdiff[st], 1u);
        if (e <= 256u) {
            atomicAdd(&S.tdiff[e], 0xFFFFFFFFu);  // -1 (tdiff[256] is never read)
        } else {
            atomicAdd(&S.tdiff[0], 1u);
            atomicAdd(&S.tdiff[e - 256u], 0xFFFFFFFFu);
        }
    }
    const uint32_t last = a0 + (w - 1u);  // tile ids stay below 2^31
    for (uint32_t p = 1; p < ndig; ++p) {
        const uint32_t sh = 8u * p, v0 = a0 >> sh, v1 = last >> sh;
        if (v0 == v1) {
            atomicAdd(&S.thist[p - 1][v0 & 255u], w);
        } else {
            atomicAdd(&S.thist[p - 1][v0 & 255u], ((v0 + 1u) << sh) - a0);
            for (uint32_t v = v0 + 1u; v < v1; ++v) atomicAdd(&S.thist[p - 1][v & 255u], 1u << sh);
            atomicAdd(&S.thist[p - 1][v1 & 255u], last - (v1 << sh) + 1u);
        }
    }
}

// (3 CTAs per SM fit in shared memory: registers up to 170 per thread are free)
__global__ void __launch_bounds__(kPreThreads, 3) preprocess_kernel(PreprocessArgs a) {
    extern __shared__ __align__(128) unsigned char pre_smem[];
    PreSmem& S = *reinterpret_cast<PreSmem*>(pre_smem);

    const uint32_t tid = threadIdx.x;
    for (uint32_t k = tid; k < kDepthPassesMax * 256; k += kPreThreads) (&S.hist[0][0])[k] = 0;
    for (uint32_t k = tid; k < 257; k += kPreThreads) S.tdiff[k] = 0;
    // launched as a dependent of frame_begin_kernel (the frame's control block).
    // No early trigger: the depth sort's first pass is one wave of CTAs, which
    // must be placed on empty SMs, not onto the first ones this grid frees
    pdl_wait();
    for (uint32_t k = tid; k < (kTileDigitsMax - 1) * 256; k += kPreThreads) (&S.thist[0][0])[k] = 0;
    if (tid == 0) S.tall = 0;
    const uint32_t ndig = min(kTileDigitsMax, (a.tile_bits + 7) / 8);  // 0: no tile-digit counts
    if (tid == 0) S.kept = 0;
    uint32_t kept = 0;  // this thread's visible items (the depth sort drops the others)
    const uint32_t nchunks = (a.n + kPreThreads - 1) / kPreThreads;
    const uint32_t npass = min(kDepthPassesMax, (a.depth_key_bits + 7) / 8);
    // chunk's records into stage: piece q (16 bytes) by thread q % 128, so a
    // warp's copies are 512 consecutive bytes; a record is 15 whole pieces
    auto issue = [&](uint32_t chunk, uint32_t stage) {
        const uint32_t base = chunk * kPreThreads;
        const uint32_t pieces = min(kPreThreads, a.n - base) * (kRecordBytes / 16u);
        const char* src = reinterpret_cast<const char*>(a.recs + size_t(base) * kRecordFloats);
        char* dst = reinterpret_cast<char*>(S.rec[stage]);
        for (uint32_t q = tid; q < pieces; q += kPreThreads) cp_async16(dst + 16u * q, src + 16u * q);
    };
    if (blockIdx.x < nchunks) issue(blockIdx.x, 0);
    cp_async_commit();
    // (while the first records arrive) the words to clear: the key sort's
    // precounted rows, which keygen adds its digit counts into
    if (a.zero_words) {
        uint4* z = reinterpret_cast<uint4*>(a.zero_words);
        const uint64_t n4 = a.zero_count / 4u;
        for (uint64_t k = uint64_t(blockIdx.x) * kPreThreads + tid; k < n4; k += uint64_t(gridDim.x) * kPreThreads)
            z[k] = make_uint4(0u, 0u, 0u, 0u);
    }

    uint32_t it = 0;
    for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x, ++it) {
        const uint32_t stage = it & 1u;
        // the other stage was released by the barrier that ended the last
        // iteration; a commit group per iteration (empty after the last
        // chunk) keeps "all but the newest group" = this chunk
        if (chunk + gridDim.x < nchunks) issue(chunk + gridDim.x, stage ^ 1u);
        cp_async_commit();
        cp_async_wait_all_but_newest();  // this thread's pieces of the chunk have landed
        __syncthreads();                 // and every other thread's

        const uint32_t base = chunk * kPreThreads;
        const uint32_t cnt = min(kPreThreads, a.n - base);
        const uint32_t i = base + tid;
        const uint32_t e = (tid < cnt && a.ent_idx) ? a.ent_idx[i] : 0u;
        for (uint32_t v = 0; v < a.n_views; ++v) {
            Splat sp;
            uint4 rect = make_uint4(0u, 0u, 0u, 0u);
            uint32_t tiles = 0;
            if (tid < cnt) {
                const float* em = a.ent_mats + (size_t(v) * a.n_ent + e) * kEntityMatFloats;
                float emr[kEntityMatFloats];
#pragma unroll
                for (int k = 0; k < kEntityMatFloats; ++k) emr[k] = __ldg(em + k);
                tiles = project_one(Rec{S.rec[stage] + tid * kRecordFloats}, emr, a.views[v], a.sh_degree,
                                    a.band3_compat != 0, sp, rect);
            } else {
                sp = Splat{0.f, 0.f, 0.f, 0u, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            }
            if (tid < cnt) {
                const size_t item = size_t(v) * a.n + i;
                float4* dst = reinterpret_cast<float4*>(a.splats + item);
                const float4* src = reinterpret_cast<const float4*>(&sp);
                dst[0] = src[0];
                dst[1] = src[1];
                dst[2] = src[2];
                if (a.depth_keys) {
                    // culled: low 32 bits 0xFFFFFFFF, dropped by the depth sort's first pass
                    const uint64_t key = (uint64_t(v) << 32) | (tiles ? __float_as_uint(sp.depth) : 0xFFFFFFFFu);
                    a.depth_keys[item] = key;
                    a.depth_items[item] = uint32_t(item);
                    if (tiles) {
                        ++kept;
                        for (uint32_t p = 0; p < npass; ++p) {
                            const uint32_t bits = min(8u, a.depth_key_bits - 8 * p);
                            atomicAdd(&S.hist[p][uint32_t(key >> (8 * p)) & ((1u << bits) - 1u)], 1u);
                        }
                    }
                }
            }
            if (ndig) {
                // the keys the warp's items will emit, the tile ids of their
                // rectangles: the rows of all 32 rectangles are spread over the
                // lanes (row r goes to lane r % 32, which finds the rectangle
                // holding it by a binary search over the warp's row prefix)
                const uint32_t lane = tid & 31u;
                const uint32_t h = tiles ? rect.w - rect.y : 0u;
                const uint32_t incl = warp_inclusive_scan(h);
                const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
                if (total) {
                    const ViewConst& vc = a.views[v];
                    const uint32_t gx = grid_x(vc.width);
                    const uint32_t row0 = vc.tile_base + rect.y * gx + rect.x, w = rect.z - rect.x, excl = incl - h;
                    for (uint32_t r0 = 0; r0 < total; r0 += 32u) {
                        const uint32_t r = r0 + lane;
                        uint32_t own = 0;  // lanes whose rows all come before row r
#pragma unroll
                        for (uint32_t step = 16; step; step >>= 1)
                            if (__shfl_sync(0xFFFFFFFFu, incl, own + step - 1u) <= r) own += step;
                        own = min(own, 31u);
                        const uint32_t o_row0 = __shfl_sync(0xFFFFFFFFu, row0, own);
                        const uint32_t o_w = __shfl_sync(0xFFFFFFFFu, w, own);
                        const uint32_t o_excl = __shfl_sync(0xFFFFFFFFu, excl, own);
                        if (r < total) count_tile_row(S, o_row0 + (r - o_excl) * gx, o_w, ndig);
                    }
                }
            }
        }
        __syncthreads();  // every thread is done with this stage before it is refilled
    }
    cp_async_wait_all();  // nothing is left in flight (the last groups are empty)
    if (ndig) {
        __syncthreads();
        // digit 0: inclusive prefix of the difference array (two values per
        // thread, 128 threads), plus the counts added to every value
        const uint32_t d0 = 2u * tid, d1 = d0 + 1u;
        const uint32_t v0 = S.tdiff[d0], pair = v0 + S.tdiff[d1];
        const uint32_t incl = warp_inclusive_scan(pair);
        __shared__ uint32_t wsum[kPreThreads / 32];
        if ((tid & 31u) == 31u) wsum[tid >> 5] = incl;
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t w = 0; w < (tid >> 5); ++w) before += wsum[w];
        const uint32_t c1 = before + incl + S.tall, c0 = c1 - S.tdiff[d1];
        if (c0) atomicAdd(&a.ctl->sort_hist[0][d0], c0);
        if (c1) atomicAdd(&a.ctl->sort_hist[0][d1], c1);
        for (uint32_t p = 1; p < ndig; ++p)
            for (uint32_t d = tid; d < 256; d += kPreThreads)
                if (S.thist[p - 1][d]) atomicAdd(&a.ctl->sort_hist[p][d], S.thist[p - 1][d]);
    }
    if (!a.depth_keys) return;
    kept = warp_sum(kept);
    if ((tid & 31u) == 0 && kept) atomicAdd(&S.kept, kept);
    __syncthreads();
    if (tid == 0 && S.kept) atomicAdd(&a.ctl->depth_count, S.kept);
    for (uint32_t p = 0; p < npass; ++p)
        for (uint32_t d = tid; d < 256; d += kPreThreads)
            if (S.hist[p][d]) atomicAdd(&a.ctl->depth_hist[p][d], S.hist[p][d]);
}

// Exclusive scan of Splat.tiles over partitions of 256 threads x 4 items
// (prefix.slang:40-158), partitions taken by atomic ticket. Total ->
// ctl->total_keys, non-empty count -> ctl->visible. (The frame scans its
// counts in depth order inside keygen_scan_kernel.)
constexpr uint32_t kScanThreads = 256;
constexpr uint32_t kScanItems = 4;

__global__ void __launch_bounds__(kScanThreads)
    scan_tiles_kernel(const Splat* splats, uint32_t n, uint32_t* offsets, uint64_t* desc, FrameCtl* ctl,
                      uint32_t spin_limit, uint32_t never_publish) {
    constexpr uint32_t kScanTile = kScanThreads * kScanItems;
    __shared__ uint32_t s_part, s_excl;
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_part = atomicAdd(&ctl->ticket[kTicketScan], 1u);
    __syncthreads();
    const uint32_t part = s_part;
    if (part * kScanTile >= n) return;  // (uniform) past the items; nothing waits on it
    const uint32_t base = part * kScanTile + tid * kScanItems;
    uint32_t v[kScanItems], sum = 0, vis = 0;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? splats[base + k].tiles : 0u;
        sum += v[k];
        vis += v[k] ? 1u : 0u;
    }
    const uint32_t incl = warp_inclusive_scan(sum);
    if (lane == 31) s_warp[warp] = incl;
    vis = warp_sum(vis);
    if (lane == 0 && vis) atomicAdd(&ctl->visible, vis);
    __syncthreads();
    uint32_t wbase = 0, total = 0;
#pragma unroll
    for (uint32_t w = 0; w < kScanThreads / 32; ++w) {
        const uint32_t sw = s_warp[w];
        if (w < warp) wbase += sw;
        total += sw;
    }
    if (warp == 0) {
        const uint32_t ex = warp_lookback(desc, part, total, ctl->tag * 32u + kTagScan, &ctl->status, spin_limit,
                                          never_publish != 0);
        if (lane == 0) {
            s_excl = ex;
            const uint32_t nparts = (n + kScanTile - 1) / kScanTile;
            if (part == nparts - 1) ctl->total_keys = ex + total;
        }
    }
    __syncthreads();
    uint32_t run = s_excl + wbase + incl - sum;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        if (base + k < n) offsets[base + k] = run;
        run += v[k];
    }
}

// Raw parameters -> records (activation as in GaussianGeometry.cpp:112-115:
// sigmoid opacity, exp scale, modifier 1; the quaternion is copied as given).
__global__ void pack_records_kernel(const float* means, const float* log_scales, const float* quats,
                                    const float* logits, const float* sh, uint32_t n, float* recs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* r = recs + size_t(i) * kRecordFloats;
    r[0] = means[i * 3 + 0];
    r[1] = means[i * 3 + 1];
    r[2] = means[i * 3 + 2];
    r[3] = 1.0f / (1.0f + expf(-logits[i]));
    for (int k = 0; k < 4; ++k) r[4 + k] = quats[i * 4 + k];
    for (int k = 0; k < 3; ++k) r[8 + k] = expf(log_scales[i * 3 + k]);
    r[11] = 1.0f;
    for (int k = 0; k < 48; ++k) r[12 + k] = sh[size_t(i) * 48 + k];
}

}  // namespace

void launch_frame_begin(FrameCtl* ctl, const float* transforms, uint32_t n_ent, const ViewConst* views,
                        uint32_t n_views, float* ent_mats, cudaStream_t s) {
    frame_begin_kernel<<<1, 256, 0, s>>>(ctl, transforms, n_ent, views, n_views, ent_mats);
}

namespace {
// The shared-memory opt-in (PreSmem is above 48 KB) and the resident CTAs per
// SM, for the current device.
int preprocess_setup() {
    cudaFuncSetAttribute(preprocess_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(PreSmem)));
    int r = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, preprocess_kernel, kPreThreads, sizeof(PreSmem));
    return r > 0 ? r : 1;
}
}  // namespace

void launch_preprocess(const PreprocessArgs& a, int num_sms, cudaStream_t s) {
    if (a.n == 0 || a.n_views == 0) return;
    const int per_sm = device_once(preprocess_setup);
    const uint32_t chunks = (a.n + kPreThreads - 1) / kPreThreads;
    const uint32_t blocks = std::min<uint32_t>(chunks, uint32_t((num_sms > 0 ? num_sms : 148) * per_sm));
    launch_dependent(preprocess_kernel, dim3(blocks), dim3(kPreThreads), sizeof(PreSmem), s, a);
}

void launch_scan_tiles(const Splat* splats, uint32_t n, uint32_t* offsets, uint64_t* desc, FrameCtl* ctl,
                       uint32_t spin_limit, uint32_t never_publish, cudaStream_t s) {
    if (n == 0) return;
    const uint32_t blocks = (n + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
    scan_tiles_kernel<<<blocks, kScanThreads, 0, s>>>(splats, n, offsets, desc, ctl, spin_limit, never_publish);
}

void launch_pack_records(const float* means, const float* log_scales, const float* quats, const float* logits,
                         const float* sh, uint32_t n, float* recs, cudaStream_t s) {
    if (n == 0) return;
    pack_records_kernel<<<(n + 255) / 256, 256, 0, s>>>(means, log_scales, quats, logits, sh, n, recs);
}

}  // namespace tpd
