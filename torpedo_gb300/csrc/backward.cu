// backward.cu — preprocess adjoint: dL/d(px, py, conic, opacity, colour) of each
// (view, Gaussian) -> dL/d(mean, log-scale, quaternion, opacity logit, SH).
//
// The reference has no backward pass (differential/ is an empty placeholder);
// this is the adjoint of its forward maths, project.slang:33-90 with
// splat/volume.slang:20-63 and splat/common.slang:35-92:
//   colour  = max(SH(dir) + 0.5, 0), dir = normalize(mean - campos) (pre-model mean)
//   (px,py) = ndc2pix(clip.xy / clip.w), clip = projview*model*(mean, 1)
//   conic   = inverse(T Sigma T^T + 0.3 I), T = J(view*model*(mean,1)) * W(view)
//   Sigma   = (R S)(R S)^T, R from the quaternion as stored (not normalised),
//             S = diag(exp(log_scale) * modifier)
//   opacity = sigmoid(logit)
// One thread per Gaussian loops over views, so gradients of the batched
// form accumulate in registers and are written once (no atomics).
#include "tpd_common.cuh"
#include "tpd_kernels.h"

namespace tpd {
namespace {

constexpr float SH_C0 = 0.28209479177387814f;
constexpr float SH_C1 = 0.4886025119029199f;
constexpr float C2_0 = 1.0925484305920792f, C2_1 = -1.0925484305920792f, C2_2 = 0.31539156525252005f,
                C2_3 = -1.0925484305920792f, C2_4 = 0.5462742152960396f;
constexpr float C3_0 = -0.5900435899266435f, C3_1 = 2.890611442640554f, C3_2 = -0.4570457994644658f,
                C3_3 = 0.3731763325901154f, C3_4 = -0.4570457994644658f, C3_5 = 1.445305721320277f,
                C3_6 = -0.5900435899266435f;

// SH basis value b and its direction gradient g for feature k = 1..15.
__device__ __forceinline__ void sh_basis(int k, float x, float y, float z, float& b, float& g0, float& g1, float& g2) {
    const float xx = x * x, yy = y * y, zz = z * z;
    g0 = g1 = g2 = 0.f;
    switch (k) {
        case 1: b = -SH_C1 * y; g1 = -SH_C1; break;
        case 2: b = SH_C1 * z; g2 = SH_C1; break;
        case 3: b = -SH_C1 * x; g0 = -SH_C1; break;
        case 4: b = C2_0 * x * y; g0 = C2_0 * y; g1 = C2_0 * x; break;
        case 5: b = C2_1 * y * z; g1 = C2_1 * z; g2 = C2_1 * y; break;
        case 6: b = C2_2 * (2.f * zz - xx - yy); g0 = -2.f * C2_2 * x; g1 = -2.f * C2_2 * y; g2 = 4.f * C2_2 * z; break;
        case 7: b = C2_3 * z * x; g0 = C2_3 * z; g2 = C2_3 * x; break;
        case 8: b = C2_4 * (xx - yy); g0 = 2.f * C2_4 * x; g1 = -2.f * C2_4 * y; break;
        case 9: b = C3_0 * y * (3.f * xx - yy); g0 = C3_0 * 6.f * x * y; g1 = C3_0 * (3.f * xx - 3.f * yy); break;
        case 10: b = C3_1 * x * y * z; g0 = C3_1 * y * z; g1 = C3_1 * x * z; g2 = C3_1 * x * y; break;
        case 11: b = C3_2 * y * (4.f * zz - xx - yy); g0 = C3_2 * (-2.f * x * y); g1 = C3_2 * (4.f * zz - xx - 3.f * yy); g2 = C3_2 * 8.f * y * z; break;
        case 12: b = C3_3 * z * (2.f * zz - 3.f * xx - 3.f * yy); g0 = C3_3 * (-6.f * x * z); g1 = C3_3 * (-6.f * y * z); g2 = C3_3 * (6.f * zz - 3.f * xx - 3.f * yy); break;
        case 13: b = C3_4 * x * (4.f * zz - xx - yy); g0 = C3_4 * (4.f * zz - 3.f * xx - yy); g1 = C3_4 * (-2.f * x * y); g2 = C3_4 * 8.f * x * z; break;
        case 14: b = C3_5 * z * (xx - yy); g0 = C3_5 * 2.f * x * z; g1 = -C3_5 * 2.f * y * z; g2 = C3_5 * (xx - yy); break;
        case 15: b = C3_6 * x * (xx - 3.f * yy); g0 = C3_6 * (3.f * xx - 3.f * yy); g1 = C3_6 * (-6.f * x * y); break;
        default: b = 0.f;
    }
}

constexpr uint32_t kBwdThreads = 128;

// A block's records are staged into shared memory with coalesced 16-byte
// loads (a record is 240 B, so thread-per-record loads would stride), and its
// SH gradients leave through the same buffer as coalesced 16-byte stores.
__global__ void __launch_bounds__(kBwdThreads) preprocess_backward_kernel(PreprocessBackwardArgs a) {
    __shared__ __align__(16) float srec[kBwdThreads * kRecordFloats];  // 30 KB; reused for the SH gradients
    pdl_wait();  // launched as a dependent of the stream's previous kernel: its output is read below
    pdl_trigger();
    const uint32_t base = blockIdx.x * kBwdThreads;
    const uint32_t cnt = min(kBwdThreads, a.n - base);
    {
        const float4* src = reinterpret_cast<const float4*>(a.recs + size_t(base) * kRecordFloats);
        float4* dst = reinterpret_cast<float4*>(srec);
        for (uint32_t k = threadIdx.x; k < cnt * (kRecordFloats / 4); k += kBwdThreads) dst[k] = src[k];
    }
    __syncthreads();
    const uint32_t i = base + threadIdx.x;
    const bool active = threadIdx.x < cnt;
    const float* rec = srec + threadIdx.x * kRecordFloats;
    if (!active) rec = srec;  // any staged record: results of inactive threads are not stored
    const float m[3] = {rec[0], rec[1], rec[2]};
    const float op = rec[3];
    const float qx = rec[4], qy = rec[5], qz = rec[6], qw = rec[7];
    const float s[3] = {rec[8] * rec[11], rec[9] * rec[11], rec[10] * rec[11]};
    const uint32_t e = (a.ent_idx && active) ? a.ent_idx[i] : 0u;
    const int nf = a.sh_degree >= 3 ? 15 : a.sh_degree == 2 ? 8 : a.sh_degree == 1 ? 3 : 0;
    const bool compat = a.band3_compat != 0;

    // R and M = R S are view independent
    const float R[9] = {1.f - 2.f * (qy * qy + qz * qz), 2.f * (qx * qy - qw * qz), 2.f * (qx * qz + qw * qy),
                        2.f * (qx * qy + qw * qz), 1.f - 2.f * (qx * qx + qz * qz), 2.f * (qy * qz - qw * qx),
                        2.f * (qx * qz - qw * qy), 2.f * (qy * qz + qw * qx), 1.f - 2.f * (qx * qx + qy * qy)};
    float M[9], Sig[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) M[r * 3 + c] = R[r * 3 + c] * s[c];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) Sig[r * 3 + c] = M[r * 3 + 0] * M[c * 3 + 0] + M[r * 3 + 1] * M[c * 3 + 1] + M[r * 3 + 2] * M[c * 3 + 2];

    float gm[3] = {0.f, 0.f, 0.f}, gSigAcc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) gSigAcc[k] = 0.f;
    float glogit = 0.f;
    float gsh[48];
#pragma unroll
    for (int k = 0; k < 48; ++k) gsh[k] = 0.f;

    // the splat (colour, tiles | texel | conic, opacity) and its gradient
    // record of view v, 16 bytes at a time; view v + 1's are loaded while
    // view v is worked on (a gradient record is read whether or not the
    // Gaussian is visible in that view: it is zero then)
    float4 n_c, n_t, n_g0, n_g1, n_g2;
    auto load_view = [&](uint32_t v) {
        const float4* sp4 = reinterpret_cast<const float4*>(a.splats + size_t(v) * a.n + i);
        n_c = sp4[0];
        n_t = sp4[1];
        const float4* g4 = reinterpret_cast<const float4*>(a.g2d + (size_t(v) * a.n + i) * kG2DStride);
        n_g0 = g4[0];
        n_g1 = g4[1];
        n_g2 = g4[2];
    };
    if (active && a.n_views) load_view(0);
    for (uint32_t v = 0; v < a.n_views && active; ++v) {
        const float4 sp_c = n_c, sp_t = n_t, ga4 = n_g0, gb4 = n_g1, gc4 = n_g2;
        if (v + 1 < a.n_views) load_view(v + 1);
        if (!(sp_t.w > 0.0f)) continue;
        const float g[9] = {ga4.x, ga4.y, ga4.z, ga4.w, gb4.x, gb4.y, gb4.z, gb4.w, gc4.x};
        const ViewConst& vc = a.views[v];
        const float* em = a.ent_mats + (size_t(v) * a.n_ent + e) * kEntityMatFloats;
        float vp[3], cp[4];
#pragma unroll
        for (int r = 0; r < 3; ++r) vp[r] = em[r * 4] * m[0] + em[r * 4 + 1] * m[1] + em[r * 4 + 2] * m[2] + em[r * 4 + 3];
#pragma unroll
        for (int r = 0; r < 4; ++r)
            cp[r] = em[12 + r * 4] * m[0] + em[12 + r * 4 + 1] * m[1] + em[12 + r * 4 + 2] * m[2] + em[12 + r * 4 + 3];
        const float Wd = float(vc.width), Hd = float(vc.height);
        const float fxp = 0.5f * Wd * vc.focal[0], fyp = 0.5f * Hd * vc.focal[1];

        // opacity
        glogit += g[5] * op * (1.f - op);

        // colour -> SH coefficients and view direction
        float campos[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            campos[k] = -(vc.view[k] * vc.view[3] + vc.view[4 + k] * vc.view[7] + vc.view[8 + k] * vc.view[11]);
        const float d0 = m[0] - campos[0], d1 = m[1] - campos[1], d2 = m[2] - campos[2];
        const float vlen = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
        const float x = d0 / vlen, y = d1 / vlen, z = d2 / vlen;
        const float col[3] = {sp_c.x, sp_c.y, sp_c.z};
        float graw[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) graw[c] = col[c] > 0.f ? g[6 + c] : 0.f;
        float gd0 = 0.f, gd1 = 0.f, gd2 = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) gsh[c] += graw[c] * SH_C0;
#pragma unroll
        for (int k = 1; k <= 15; ++k) {
            if (k > nf) break;
            float b, b0, b1, b2;
            sh_basis(k, x, y, z, b, b0, b1, b2);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int slot = 3 + c * 15 + (k - 1);
                if (k == 12 && compat) {
                    gsh[slot] += graw[c];
                    gd0 += graw[c] * b0;
                    gd1 += graw[c] * b1;
                    gd2 += graw[c] * b2;
                } else {
                    const float coef = rec[12 + slot];
                    gsh[slot] += graw[c] * b;
                    gd0 += graw[c] * coef * b0;
                    gd1 += graw[c] * coef * b1;
                    gd2 += graw[c] * coef * b2;
                }
            }
        }
        const float dd = x * gd0 + y * gd1 + z * gd2;
        gm[0] += (gd0 - x * dd) / vlen;
        gm[1] += (gd1 - y * dd) / vlen;
        gm[2] += (gd2 - z * dd) / vlen;

        // pixel position -> clip -> mean
        const float w = cp[3];
        const float gcp[4] = {g[0] * Wd / (2.f * w), g[1] * Hd / (2.f * w), 0.f,
                              -(g[0] * Wd * cp[0] + g[1] * Hd * cp[1]) / (2.f * w * w)};
#pragma unroll
        for (int d = 0; d < 3; ++d)
            gm[d] += em[12 + 0 * 4 + d] * gcp[0] + em[12 + 1 * 4 + d] * gcp[1] + em[12 + 3 * 4 + d] * gcp[3];

        // 2D covariance
        const float vz = vp[2];
        const float J0 = fxp / vz, J2 = -fxp * vp[0] / (vz * vz), J4 = fyp / vz, J5 = -fyp * vp[1] / (vz * vz);
        const float* V = vc.view;
        float Tm[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            Tm[c] = J0 * V[0 * 4 + c] + J2 * V[2 * 4 + c];
            Tm[3 + c] = J4 * V[1 * 4 + c] + J5 * V[2 * 4 + c];
        }
        float TS[6];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                TS[r * 3 + c] = Tm[r * 3 + 0] * Sig[0 * 3 + c] + Tm[r * 3 + 1] * Sig[1 * 3 + c] + Tm[r * 3 + 2] * Sig[2 * 3 + c];
        const float ca = TS[0] * Tm[0] + TS[1] * Tm[1] + TS[2] * Tm[2] + 0.3f;
        const float cb = TS[3] * Tm[0] + TS[4] * Tm[1] + TS[5] * Tm[2];
        const float cc = TS[3] * Tm[3] + TS[4] * Tm[4] + TS[5] * Tm[5] + 0.3f;
        const float det = ca * cc - cb * cb;
        const float idet2 = 1.f / (det * det);
        const float gA = g[2], gB = g[3], gC = g[4];
        const float ga = (-gA * cc * cc + gB * cb * cc - gC * cb * cb) * idet2;
        const float gb = (2.f * gA * cb * cc - gB * (ca * cc + cb * cb) + 2.f * gC * ca * cb) * idet2;
        const float gc = (-gA * cb * cb + gB * ca * cb - gC * ca * ca) * idet2;
        // G = [[ga, 0], [gb, gc]]: dL/dSig = T^T G T, dL/dT = (G + G^T) T Sig
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                gSigAcc[r * 3 + c] += Tm[r] * (ga * Tm[c]) + Tm[3 + r] * (gb * Tm[c] + gc * Tm[3 + c]);
        float gT[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            gT[c] = 2.f * ga * TS[c] + gb * TS[3 + c];
            gT[3 + c] = gb * TS[c] + 2.f * gc * TS[3 + c];
        }
        // T = J W: dL/dJ = dL/dT W^T (only J0, J2, J4, J5 are non-zero functions of vp)
        float gJ[6];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                gJ[r * 3 + c] = gT[r * 3 + 0] * V[c * 4 + 0] + gT[r * 3 + 1] * V[c * 4 + 1] + gT[r * 3 + 2] * V[c * 4 + 2];
        const float ivz2 = 1.f / (vz * vz), ivz3 = ivz2 / vz;
        const float gvp0 = gJ[2] * (-fxp * ivz2);
        const float gvp1 = gJ[5] * (-fyp * ivz2);
        const float gvp2 = gJ[0] * (-fxp * ivz2) + gJ[2] * (2.f * fxp * vp[0] * ivz3) + gJ[4] * (-fyp * ivz2) +
                           gJ[5] * (2.f * fyp * vp[1] * ivz3);
#pragma unroll
        for (int d = 0; d < 3; ++d) gm[d] += em[0 * 4 + d] * gvp0 + em[1 * 4 + d] * gvp1 + em[2 * 4 + d] * gvp2;
    }

    // Sigma = M M^T, M = R S
    float gM[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            gM[r * 3 + c] = (gSigAcc[r * 3 + 0] + gSigAcc[0 * 3 + r]) * M[0 * 3 + c] +
                            (gSigAcc[r * 3 + 1] + gSigAcc[1 * 3 + r]) * M[1 * 3 + c] +
                            (gSigAcc[r * 3 + 2] + gSigAcc[2 * 3 + r]) * M[2 * 3 + c];
    float gR[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) gR[r * 3 + c] = gM[r * 3 + c] * s[c];
    float gq[4], glsv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) glsv[c] = (gM[0 * 3 + c] * R[0 * 3 + c] + gM[1 * 3 + c] * R[1 * 3 + c] + gM[2 * 3 + c] * R[2 * 3 + c]) * s[c];
    gq[0] = gR[1] * 2.f * qy + gR[2] * 2.f * qz + gR[3] * 2.f * qy + gR[4] * (-4.f * qx) + gR[5] * (-2.f * qw) +
            gR[6] * 2.f * qz + gR[7] * 2.f * qw + gR[8] * (-4.f * qx);
    gq[1] = gR[0] * (-4.f * qy) + gR[1] * 2.f * qx + gR[2] * 2.f * qw + gR[3] * 2.f * qx + gR[5] * 2.f * qz +
            gR[6] * (-2.f * qw) + gR[7] * 2.f * qz + gR[8] * (-4.f * qy);
    gq[2] = gR[0] * (-4.f * qz) + gR[1] * (-2.f * qw) + gR[2] * 2.f * qx + gR[3] * 2.f * qw + gR[4] * (-4.f * qz) +
            gR[5] * 2.f * qy + gR[6] * 2.f * qx + gR[7] * 2.f * qy;
    gq[3] = gR[1] * (-2.f * qz) + gR[2] * 2.f * qy + gR[3] * 2.f * qz + gR[5] * (-2.f * qx) + gR[6] * (-2.f * qy) +
            gR[7] * 2.f * qx;
    if (active) {
        float* gls = a.g_log_scales + size_t(i) * 3;
        gls[0] = glsv[0];
        gls[1] = glsv[1];
        gls[2] = glsv[2];
        if ((reinterpret_cast<uintptr_t>(a.g_quats) & 15u) == 0) {
            reinterpret_cast<float4*>(a.g_quats)[i] = make_float4(gq[0], gq[1], gq[2], gq[3]);
        } else {
            float* gqo = a.g_quats + size_t(i) * 4;
            gqo[0] = gq[0];
            gqo[1] = gq[1];
            gqo[2] = gq[2];
            gqo[3] = gq[3];
        }
    }
    __syncthreads();  // every thread is done with the staged records
    if (active) {
        float* gmo = a.g_means + size_t(i) * 3;
        gmo[0] = gm[0];
        gmo[1] = gm[1];
        gmo[2] = gm[2];
        a.g_logits[i] = glogit;
        float4* mine = reinterpret_cast<float4*>(srec + threadIdx.x * 48);
#pragma unroll
        for (int k = 0; k < 12; ++k) mine[k] = make_float4(gsh[4 * k], gsh[4 * k + 1], gsh[4 * k + 2], gsh[4 * k + 3]);
    }
    __syncthreads();
    if ((reinterpret_cast<uintptr_t>(a.g_sh) & 15u) == 0) {
        float4* gs = reinterpret_cast<float4*>(a.g_sh + size_t(base) * 48);
        const float4* from = reinterpret_cast<const float4*>(srec);
        for (uint32_t k = threadIdx.x; k < cnt * 12; k += kBwdThreads) gs[k] = from[k];
    } else {  // a caller's buffer that is not 16-byte aligned
        float* gs = a.g_sh + size_t(base) * 48;
        for (uint32_t k = threadIdx.x; k < cnt * 48; k += kBwdThreads) gs[k] = srec[k];
    }
}

}  // namespace

void launch_preprocess_backward(const PreprocessBackwardArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    launch_dependent(preprocess_backward_kernel, dim3((a.n + kBwdThreads - 1) / kBwdThreads), dim3(kBwdThreads), 0,
                     s, a);
}

}  // namespace tpd
