// tpd_oracle_bwd.cpp — FP64 forward from raw parameters and its analytic
// gradient. TEST INFRASTRUCTURE ONLY (see tpd_oracle.h).
//
// The reference has no backward pass (its differential/ module is an empty
// placeholder), so this is a restatement of the mathematics of its forward:
// project.slang / splat/volume.slang / splat/common.slang for the per-Gaussian
// part and blend.slang for compositing. Conventions shared with the GPU adjoint:
//  - the quaternion is used as stored (the shaders do not normalise it);
//  - scale = exp(log_scale) with modifier 1, opacity = sigmoid(logit);
//  - the model matrix moves the mean only; covariance uses the view matrix;
//  - the SH direction uses the pre-model mean;
//  - colour clamp max(c, 0): no gradient where the unclamped colour is < 0;
//  - alpha = min(0.99, o*exp(power)): no gradient to o / power where o*exp(power) > 0.99;
//  - lists (which Gaussians each tile visits, in order) are fixed inputs.
#include "tpd_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr uint32_t BLOCK = 16;
constexpr double SH_C0 = 0.28209479177387814;
constexpr double SH_C1 = 0.4886025119029199;
constexpr double C2[5] = {1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
                          -1.0925484305920792, 0.5462742152960396};
constexpr double C3[7] = {-0.5900435899266435, 2.890611442640554, -0.4570457994644658,
                          0.3731763325901154, -0.4570457994644658, 1.445305721320277,
                          -0.5900435899266435};

// SH basis value and gradient w.r.t. the direction for feature k = 1..15.
// band3_compat: feature 12 has coefficient 1 and the scalar term s12 is added
// to every channel (splat/common.slang:69 as written).
inline void sh_basis(int k, const double d[3], double& b, double g[3]) {
    const double x = d[0], y = d[1], z = d[2];
    const double xx = x * x, yy = y * y, zz = z * z;
    g[0] = g[1] = g[2] = 0;
    switch (k) {
        case 1: b = -SH_C1 * y; g[1] = -SH_C1; break;
        case 2: b = SH_C1 * z; g[2] = SH_C1; break;
        case 3: b = -SH_C1 * x; g[0] = -SH_C1; break;
        case 4: b = C2[0] * x * y; g[0] = C2[0] * y; g[1] = C2[0] * x; break;
        case 5: b = C2[1] * y * z; g[1] = C2[1] * z; g[2] = C2[1] * y; break;
        case 6: b = C2[2] * (2 * zz - xx - yy); g[0] = -2 * C2[2] * x; g[1] = -2 * C2[2] * y; g[2] = 4 * C2[2] * z; break;
        case 7: b = C2[3] * z * x; g[0] = C2[3] * z; g[2] = C2[3] * x; break;
        case 8: b = C2[4] * (xx - yy); g[0] = 2 * C2[4] * x; g[1] = -2 * C2[4] * y; break;
        case 9: b = C3[0] * y * (3 * xx - yy); g[0] = C3[0] * 6 * x * y; g[1] = C3[0] * (3 * xx - 3 * yy); break;
        case 10: b = C3[1] * x * y * z; g[0] = C3[1] * y * z; g[1] = C3[1] * x * z; g[2] = C3[1] * x * y; break;
        case 11: b = C3[2] * y * (4 * zz - xx - yy); g[0] = C3[2] * (-2 * x * y); g[1] = C3[2] * (4 * zz - xx - 3 * yy); g[2] = C3[2] * 8 * y * z; break;
        case 12: b = C3[3] * z * (2 * zz - 3 * xx - 3 * yy); g[0] = C3[3] * (-6 * x * z); g[1] = C3[3] * (-6 * y * z); g[2] = C3[3] * (6 * zz - 3 * xx - 3 * yy); break;
        case 13: b = C3[4] * x * (4 * zz - xx - yy); g[0] = C3[4] * (4 * zz - 3 * xx - yy); g[1] = C3[4] * (-2 * x * y); g[2] = C3[4] * 8 * x * z; break;
        case 14: b = C3[5] * z * (xx - yy); g[0] = C3[5] * 2 * x * z; g[1] = -C3[5] * 2 * y * z; g[2] = C3[5] * (xx - yy); break;
        case 15: b = C3[6] * x * (xx - 3 * yy); g[0] = C3[6] * (3 * xx - 3 * yy); g[1] = C3[6] * (-6 * x * y); break;
        default: b = 0;
    }
}

inline int nfeat(uint32_t deg) { return deg >= 3 ? 15 : deg == 2 ? 8 : deg == 1 ? 3 : 0; }

struct Fwd {
    bool visible;
    double m[3], s[3], q[4], op;
    double VM[16], PM[16];
    double vp[3], cp[4];
    double R[9], M[9], Sig[9];
    double Tm[6];  // top two rows of J*W
    double a, b, c, det;
    double px, py, conic[3], color[3], raw[3];
    double dir[3], vlen;
};

void mat4mul(const double* A, const double* B, double* C) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double acc = 0;
            for (int k = 0; k < 4; ++k) acc += A[i * 4 + k] * B[k * 4 + j];
            C[i * 4 + j] = acc;
        }
}

// Forward of one Gaussian from raw parameters (project.slang:33-90 in double).
// Visibility is decided here only to pick which Gaussians get outputs; which
// tiles a Gaussian is blended into comes from the fixed lists.
Fwd forward_one(const orc_params64* p, uint32_t i, const orc_camera* cam, const double* model,
                uint32_t deg, int compat) {
    Fwd f{};
    f.visible = false;
    for (int k = 0; k < 3; ++k) { f.m[k] = p->means[i * 3 + k]; f.s[k] = std::exp(p->log_scales[i * 3 + k]); }
    for (int k = 0; k < 4; ++k) f.q[k] = p->quats[i * 4 + k];
    f.op = 1.0 / (1.0 + std::exp(-p->opacity_logits[i]));
    double V[16], P[16];
    for (int k = 0; k < 16; ++k) { V[k] = cam->view[k]; P[k] = cam->projview[k]; }
    mat4mul(V, model, f.VM);
    mat4mul(P, model, f.PM);
    for (int r = 0; r < 3; ++r)
        f.vp[r] = f.VM[r * 4] * f.m[0] + f.VM[r * 4 + 1] * f.m[1] + f.VM[r * 4 + 2] * f.m[2] + f.VM[r * 4 + 3];
    for (int r = 0; r < 4; ++r)
        f.cp[r] = f.PM[r * 4] * f.m[0] + f.PM[r * 4 + 1] * f.m[1] + f.PM[r * 4 + 2] * f.m[2] + f.PM[r * 4 + 3];
    if (f.vp[2] <= 0 || f.cp[3] == 0) return f;
    const double W = cam->width, H = cam->height;
    const double fx = 0.5 * W * cam->focal[0], fy = 0.5 * H * cam->focal[1];
    const double x = f.q[0], y = f.q[1], z = f.q[2], w = f.q[3];
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
    std::memcpy(f.R, R, sizeof(R));
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) f.M[r * 3 + c] = R[r * 3 + c] * f.s[c];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double acc = 0;
            for (int k = 0; k < 3; ++k) acc += f.M[r * 3 + k] * f.M[c * 3 + k];
            f.Sig[r * 3 + c] = acc;
        }
    const double vz = f.vp[2];
    const double J[6] = {fx / vz, 0, -fx * f.vp[0] / (vz * vz), 0, fy / vz, -fy * f.vp[1] / (vz * vz)};
    const double W3[9] = {V[0], V[1], V[2], V[4], V[5], V[6], V[8], V[9], V[10]};
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c) {
            double acc = 0;
            for (int k = 0; k < 3; ++k) acc += J[r * 3 + k] * W3[k * 3 + c];
            f.Tm[r * 3 + c] = acc;
        }
    double cov2[4];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            double acc = 0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) acc += f.Tm[r * 3 + k] * f.Sig[k * 3 + l] * f.Tm[c * 3 + l];
            cov2[r * 2 + c] = acc;
        }
    f.a = cov2[0] + (double)0.3f;
    f.b = cov2[2];
    f.c = cov2[3] + (double)0.3f;
    f.det = f.a * f.c - f.b * f.b;
    if (f.det == 0) return f;
    f.conic[0] = f.c / f.det; f.conic[1] = -f.b / f.det; f.conic[2] = f.a / f.det;
    f.px = ((f.cp[0] / f.cp[3] + 1) * W - 1) * 0.5;
    f.py = ((f.cp[1] / f.cp[3] + 1) * H - 1) * 0.5;
    // colour
    double campos[3];
    for (int k = 0; k < 3; ++k) campos[k] = -(V[k] * V[3] + V[4 + k] * V[7] + V[8 + k] * V[11]);
    double v[3] = {f.m[0] - campos[0], f.m[1] - campos[1], f.m[2] - campos[2]};
    f.vlen = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) f.dir[k] = v[k] / f.vlen;
    const double* sh = p->sh + (size_t)i * 48;
    double s12 = 0, g12[3];
    if (deg >= 3 && compat) sh_basis(12, f.dir, s12, g12);
    for (int ch = 0; ch < 3; ++ch) {
        double r = SH_C0 * sh[ch];
        for (int k = 1; k <= nfeat(deg); ++k) {
            double b, g[3];
            sh_basis(k, f.dir, b, g);
            const double coef = sh[3 + ch * 15 + (k - 1)];
            if (k == 12 && compat) r += s12 + coef;
            else r += b * coef;
        }
        f.raw[ch] = r + 0.5;
        f.color[ch] = std::max(f.raw[ch], 0.0);
    }
    f.visible = true;
    return f;
}

void identity(double* M) { for (int k = 0; k < 16; ++k) M[k] = (k % 5) == 0 ? 1.0 : 0.0; }

struct Splat64 { double px, py, A, B, C, op, col[3]; bool ok; };

}  // namespace

extern "C" {

void orc_render_params_f64(const orc_params64* p, uint32_t n, const orc_camera* cam, uint32_t sh_degree,
                           int band3_compat, const uint32_t* vals, const uint32_t* ranges, double* image) {
    double M[16];
    identity(M);
    const uint32_t deg = std::min<uint32_t>(sh_degree, 3);
    std::vector<double> sp((size_t)n * ORC_SPLAT_WORDS, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const Fwd f = forward_one(p, (uint32_t)i, cam, M, deg, band3_compat);
        double* s = sp.data() + i * ORC_SPLAT_WORDS;
        if (!f.visible) continue;
        s[0] = f.color[0]; s[1] = f.color[1]; s[2] = f.color[2];
        s[4] = f.px; s[5] = f.py; s[6] = f.vp[2];
        s[8] = f.conic[0]; s[9] = f.conic[1]; s[10] = f.conic[2]; s[11] = f.op;
    }
    orc_blend_f64(sp.data(), vals, ranges, cam->width, cam->height, image, nullptr, nullptr, nullptr);
}

void orc_backward_f64(const orc_params64* p, uint32_t n, const orc_camera* cam, uint32_t sh_degree,
                      int band3_compat, const uint32_t* vals, const uint32_t* ranges,
                      const double* dL_dimage, double* g_means, double* g_log_scales, double* g_quats,
                      double* g_logits, double* g_sh, double* g2d_out) {
    double Mid[16];
    identity(Mid);
    const uint32_t deg = std::min<uint32_t>(sh_degree, 3);
    const uint32_t W = cam->width, H = cam->height;
    const uint32_t gx = (W + BLOCK - 1) / BLOCK, gy = (H + BLOCK - 1) / BLOCK;
    std::vector<Fwd> fw(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) fw[i] = forward_one(p, (uint32_t)i, cam, Mid, deg, band3_compat);

    // ---- blend adjoint (per pixel, sequential over tiles for a deterministic sum)
    std::vector<double> g2d((size_t)n * 9, 0.0);
    const double a_min = (double)(1.0f / 255.0f);
    struct Contrib { uint32_t idx; double alpha, T, G, dx, dy; bool clamped; };
    std::vector<Contrib> list;
    for (uint32_t tile = 0; tile < gx * gy; ++tile) {
        const uint32_t tx = tile % gx, ty = tile / gx;
        const uint32_t start = ranges[tile * 2], end = ranges[tile * 2 + 1];
        for (uint32_t ly = 0; ly < BLOCK; ++ly)
            for (uint32_t lx = 0; lx < BLOCK; ++lx) {
                const uint32_t px = tx * BLOCK + lx, py = ty * BLOCK + ly;
                if (px >= W || py >= H) continue;
                list.clear();
                double T = 1.0;
                for (uint32_t k = start; k < end; ++k) {
                    const Fwd& f = fw[vals[k]];
                    if (!f.visible) continue;
                    const double dx = f.px - px, dy = f.py - py;
                    const double power = -0.5 * (f.conic[0] * dx * dx + f.conic[2] * dy * dy) - f.conic[1] * dx * dy;
                    if (power > 0.0) continue;
                    const double G = std::exp(power);
                    const double raw_a = f.op * G;
                    const double alpha = std::min(0.99, raw_a);
                    if (alpha < a_min) continue;
                    const double tn = T * (1.0 - alpha);
                    if (tn < 1e-4) break;
                    list.push_back({vals[k], alpha, T, G, dx, dy, raw_a > 0.99});
                    T = tn;
                }
                const double* gI = dL_dimage + ((size_t)py * W + px) * 3;
                double S[3] = {0, 0, 0};
                for (size_t j = list.size(); j-- > 0;) {
                    const Contrib& c = list[j];
                    const Fwd& f = fw[c.idx];
                    double* g = g2d.data() + (size_t)c.idx * 9;
                    double dA = 0;
                    for (int ch = 0; ch < 3; ++ch) {
                        g[6 + ch] += gI[ch] * c.alpha * c.T;
                        dA += gI[ch] * (f.color[ch] * c.T - S[ch] / (1.0 - c.alpha));
                        S[ch] += f.color[ch] * c.alpha * c.T;
                    }
                    if (c.clamped) continue;
                    const double dpow = dA * c.alpha;  // d alpha / d power = alpha
                    g[5] += dA * c.G;                 // d alpha / d opacity = exp(power)
                    const double A = f.conic[0], B = f.conic[1], C = f.conic[2];
                    g[0] += dpow * (-A * c.dx - B * c.dy);
                    g[1] += dpow * (-C * c.dy - B * c.dx);
                    g[2] += dpow * (-0.5 * c.dx * c.dx);
                    g[3] += dpow * (-c.dx * c.dy);
                    g[4] += dpow * (-0.5 * c.dy * c.dy);
                }
            }
    }
    if (g2d_out) std::memcpy(g2d_out, g2d.data(), g2d.size() * sizeof(double));

    // ---- preprocess adjoint (per Gaussian)
    const double Wd = W, Hd = H;
    const double fxp = 0.5 * Wd * cam->focal[0], fyp = 0.5 * Hd * cam->focal[1];
    double V[16];
    for (int k = 0; k < 16; ++k) V[k] = cam->view[k];
    const double W3[9] = {V[0], V[1], V[2], V[4], V[5], V[6], V[8], V[9], V[10]};
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        double* gm = g_means + i * 3; double* gs = g_log_scales + i * 3; double* gq = g_quats + i * 4;
        double* gsh = g_sh + (size_t)i * 48;
        for (int k = 0; k < 3; ++k) { gm[k] = 0; gs[k] = 0; }
        for (int k = 0; k < 4; ++k) gq[k] = 0;
        for (int k = 0; k < 48; ++k) gsh[k] = 0;
        g_logits[i] = 0;
        const Fwd& f = fw[i];
        if (!f.visible) continue;
        const double* g = g2d.data() + (size_t)i * 9;
        // opacity
        g_logits[i] = g[5] * f.op * (1.0 - f.op);
        // colour -> SH and direction
        double graw[3];
        for (int ch = 0; ch < 3; ++ch) graw[ch] = f.raw[ch] < 0 ? 0.0 : g[6 + ch];
        const double* sh = p->sh + (size_t)i * 48;
        double gdir[3] = {0, 0, 0};
        for (int ch = 0; ch < 3; ++ch) gsh[ch] = graw[ch] * SH_C0;
        for (int k = 1; k <= nfeat(deg); ++k) {
            double b, gb[3];
            sh_basis(k, f.dir, b, gb);
            for (int ch = 0; ch < 3; ++ch) {
                const double coef = sh[3 + ch * 15 + (k - 1)];
                if (k == 12 && band3_compat) {
                    gsh[3 + ch * 15 + (k - 1)] = graw[ch];
                    for (int d = 0; d < 3; ++d) gdir[d] += graw[ch] * gb[d];
                } else {
                    gsh[3 + ch * 15 + (k - 1)] = graw[ch] * b;
                    for (int d = 0; d < 3; ++d) gdir[d] += graw[ch] * coef * gb[d];
                }
            }
        }
        const double dd = f.dir[0] * gdir[0] + f.dir[1] * gdir[1] + f.dir[2] * gdir[2];
        for (int d = 0; d < 3; ++d) gm[d] += (gdir[d] - f.dir[d] * dd) / f.vlen;

        // pixel position -> clip -> mean
        const double w = f.cp[3];
        double gcp[4] = {g[0] * Wd / (2 * w), g[1] * Hd / (2 * w), 0,
                         -(g[0] * Wd * f.cp[0] + g[1] * Hd * f.cp[1]) / (2 * w * w)};
        for (int d = 0; d < 3; ++d)
            for (int r = 0; r < 4; ++r) gm[d] += f.PM[r * 4 + d] * gcp[r];

        // conic -> (a, b, c)
        const double a = f.a, b = f.b, c = f.c, det2 = f.det * f.det;
        const double gA = g[2], gB = g[3], gC = g[4];
        const double ga = (-gA * c * c + gB * b * c - gC * b * b) / det2;
        const double gbb = (2 * gA * b * c - gB * (a * c + b * b) + 2 * gC * a * b) / det2;
        const double gc = (-gA * b * b + gB * a * b - gC * a * a) / det2;
        // cov2 = T Sig T^T, reading [0][0], [1][0], [1][1]: G = [[ga, 0], [gbb, gc]]
        const double G[4] = {ga, 0.0, gbb, gc};
        // dL/dSig = T^T G T
        double gSig[9];
        for (int r = 0; r < 3; ++r)
            for (int cc = 0; cc < 3; ++cc) {
                double acc = 0;
                for (int u = 0; u < 2; ++u)
                    for (int v2 = 0; v2 < 2; ++v2) acc += f.Tm[u * 3 + r] * G[u * 2 + v2] * f.Tm[v2 * 3 + cc];
                gSig[r * 3 + cc] = acc;
            }
        // dL/dT = (G + G^T) T Sig
        double GG[4] = {G[0] + G[0], G[1] + G[2], G[2] + G[1], G[3] + G[3]};
        double TS[6];
        for (int r = 0; r < 2; ++r)
            for (int cc = 0; cc < 3; ++cc) {
                double acc = 0;
                for (int k = 0; k < 3; ++k) acc += f.Tm[r * 3 + k] * f.Sig[k * 3 + cc];
                TS[r * 3 + cc] = acc;
            }
        double gT[6];
        for (int r = 0; r < 2; ++r)
            for (int cc = 0; cc < 3; ++cc) gT[r * 3 + cc] = GG[r * 2 + 0] * TS[0 * 3 + cc] + GG[r * 2 + 1] * TS[1 * 3 + cc];
        // T = J W -> dL/dJ = dL/dT W^T
        double gJ[6];
        for (int r = 0; r < 2; ++r)
            for (int cc = 0; cc < 3; ++cc) {
                double acc = 0;
                for (int k = 0; k < 3; ++k) acc += gT[r * 3 + k] * W3[cc * 3 + k];
                gJ[r * 3 + cc] = acc;
            }
        const double vx = f.vp[0], vy = f.vp[1], vz = f.vp[2];
        double gvp[3] = {0, 0, 0};
        gvp[2] += gJ[0] * (-fxp / (vz * vz));
        gvp[0] += gJ[2] * (-fxp / (vz * vz));
        gvp[2] += gJ[2] * (2 * fxp * vx / (vz * vz * vz));
        gvp[2] += gJ[4] * (-fyp / (vz * vz));
        gvp[1] += gJ[5] * (-fyp / (vz * vz));
        gvp[2] += gJ[5] * (2 * fyp * vy / (vz * vz * vz));
        for (int d = 0; d < 3; ++d)
            for (int r = 0; r < 3; ++r) gm[d] += f.VM[r * 4 + d] * gvp[r];

        // Sig = M M^T, M = R S
        double gM[9];
        for (int r = 0; r < 3; ++r)
            for (int cc = 0; cc < 3; ++cc) {
                double acc = 0;
                for (int k = 0; k < 3; ++k) acc += (gSig[r * 3 + k] + gSig[k * 3 + r]) * f.M[k * 3 + cc];
                gM[r * 3 + cc] = acc;
            }
        double gR[9];
        for (int r = 0; r < 3; ++r)
            for (int cc = 0; cc < 3; ++cc) gR[r * 3 + cc] = gM[r * 3 + cc] * f.s[cc];
        for (int cc = 0; cc < 3; ++cc) {
            double acc = 0;
            for (int r = 0; r < 3; ++r) acc += gM[r * 3 + cc] * f.R[r * 3 + cc];
            gs[cc] = acc * f.s[cc];  // d s / d log_s = s
        }
        const double x = f.q[0], y = f.q[1], z = f.q[2], qw = f.q[3];
        gq[0] = gR[1] * 2 * y + gR[2] * 2 * z + gR[3] * 2 * y + gR[4] * (-4 * x) + gR[5] * (-2 * qw) +
                gR[6] * 2 * z + gR[7] * 2 * qw + gR[8] * (-4 * x);
        gq[1] = gR[0] * (-4 * y) + gR[1] * 2 * x + gR[2] * 2 * qw + gR[3] * 2 * x + gR[5] * 2 * z +
                gR[6] * (-2 * qw) + gR[7] * 2 * z + gR[8] * (-4 * y);
        gq[2] = gR[0] * (-4 * z) + gR[1] * (-2 * qw) + gR[2] * 2 * x + gR[3] * 2 * qw + gR[4] * (-4 * z) +
                gR[5] * 2 * y + gR[6] * 2 * x + gR[7] * 2 * y;
        gq[3] = gR[1] * (-2 * z) + gR[2] * 2 * y + gR[3] * 2 * z + gR[5] * (-2 * x) + gR[6] * (-2 * y) +
                gR[7] * 2 * x;
    }
}

}  // extern "C"
