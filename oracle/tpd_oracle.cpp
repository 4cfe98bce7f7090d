// tpd_oracle.cpp — CPU oracle for the Gaussian-splatting hot path.
//
// TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
// bench's CPU-baseline leg, never by the product library. See tpd_oracle.h for
// what each function restates and for the parity status ("parity unpinned" for
// the shader maths: the Slang path cannot run here and the reference has no
// golden vectors).
//
// Build: g++ -O2 -fopenmp -ffp-contract=off (no -ffast-math). The FP32 path must
// not contract a*b+c into fma: it is the operation-order transcription.
#include "tpd_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint32_t BLOCK = 16;          // BLOCK_X = BLOCK_Y (splat.slang:8-9)
constexpr uint32_t WORKGROUP = 256;     // WORKGROUP_SIZE (splat.slang:7)

// SH constants (splat/common.slang:3-20). Converted to T from the decimal text.
constexpr double SH_C0 = 0.28209479177387814;
constexpr double SH_C1 = 0.4886025119029199;
constexpr double SH_C2[5] = {1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
                             -1.0925484305920792, 0.5462742152960396};
constexpr double SH_C3[7] = {-0.5900435899266435, 2.890611442640554, -0.4570457994644658,
                             0.3731763325901154, -0.4570457994644658, 1.445305721320277,
                             -0.5900435899266435};

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// max() as a non-NaN-propagating maximum, like fmaxf.
template <typename T> inline T tmax(T a, T b) { return std::fmax(a, b); }
template <typename T> inline T tmin(T a, T b) { return std::fmin(a, b); }

// (int) conversion of the shaders, truncation toward zero, saturated to the int
// range (out-of-range conversion is undefined in SPIR-V and C++).
template <typename T> inline int trunc_int(T v) {
    if (!(v == v)) return 0;
    if (v >= T(2147483520.0)) return 2147483647;
    if (v <= T(-2147483520.0)) return -2147483647 - 1;
    return (int)v;
}

// C[i][j] = ((A[i][0]B[0][j] + A[i][1]B[1][j]) + A[i][2]B[2][j]) (+ A[i][3]B[3][j])
template <typename T, int D> inline void matmul(const T* A, const T* B, T* C) {
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
            T acc = A[i * D + 0] * B[0 * D + j];
            for (int k = 1; k < D; ++k) acc = acc + A[i * D + k] * B[k * D + j];
            C[i * D + j] = acc;
        }
}
template <typename T, int D> inline void transpose(const T* A, T* B) {
    for (int i = 0; i < D; ++i) for (int j = 0; j < D; ++j) B[j * D + i] = A[i * D + j];
}

// Input of one Gaussian in arithmetic type T (record fields after activation).
template <typename T> struct GIn {
    T pos[3]; T opacity; T quat[4]; T scale[4]; T sh[48];
};

template <typename T> struct GOut {
    T color[3]; uint32_t tiles; T px, py, depth, radius; T conic[3]; T opacity;
    uint32_t rect[4];
    bool visible;
    bool fragile;  // f64 only: a decision lies near its threshold
};

template <typename T> struct Cam {
    T V[16]; T P[16]; T focal[2]; uint32_t W, H;
};

template <typename T> Cam<T> make_cam(const orc_camera* c) {
    Cam<T> k;
    for (int i = 0; i < 16; ++i) { k.V[i] = T(c->view[i]); k.P[i] = T(c->projview[i]); }
    k.focal[0] = T(c->focal[0]); k.focal[1] = T(c->focal[1]);
    k.W = c->width; k.H = c->height;
    return k;
}

// evaluateSphericalHarmonics (splat/common.slang:35-80), left-to-right order.
template <typename T>
void eval_sh(const T* sh, const T dir[3], uint32_t degree, int band3_compat, T out[3]) {
    auto feat = [&](int idx, int c) { return sh[(idx - 1) + c * 15 + 3]; };
    T res[3];
    for (int c = 0; c < 3; ++c) res[c] = T(SH_C0) * sh[c];
    if (degree > 0) {
        const T x = dir[0], y = dir[1], z = dir[2];
        for (int c = 0; c < 3; ++c)
            res[c] = res[c] - (T(SH_C1) * y) * feat(1, c) + (T(SH_C1) * z) * feat(2, c) -
                     (T(SH_C1) * x) * feat(3, c);
        if (degree > 1) {
            const T xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, zx = z * x;
            for (int c = 0; c < 3; ++c)
                res[c] = res[c] + (T(SH_C2[0]) * xy) * feat(4, c) + (T(SH_C2[1]) * yz) * feat(5, c) +
                         (T(SH_C2[2]) * (T(2.0) * zz - xx - yy)) * feat(6, c) +
                         (T(SH_C2[3]) * zx) * feat(7, c) + (T(SH_C2[4]) * (xx - yy)) * feat(8, c);
            if (degree > 2) {
                for (int c = 0; c < 3; ++c) {
                    T r = res[c] + ((T(SH_C3[0]) * y) * (T(3.0) * xx - yy)) * feat(9, c) +
                          ((T(SH_C3[1]) * xy) * z) * feat(10, c) +
                          ((T(SH_C3[2]) * y) * (T(4.0) * zz - xx - yy)) * feat(11, c);
                    const T s12 = (T(SH_C3[3]) * z) * (T(2.0) * zz - T(3.0) * xx - T(3.0) * yy);
                    if (band3_compat) r = r + s12 + feat(12, c);  // common.slang:69 as written
                    else r = r + s12 * feat(12, c);
                    r = r + ((T(SH_C3[4]) * x) * (T(4.0) * zz - xx - yy)) * feat(13, c) +
                        ((T(SH_C3[5]) * z) * (xx - yy)) * feat(14, c) +
                        ((T(SH_C3[6]) * x) * (xx - T(3.0) * yy)) * feat(15, c);
                    res[c] = r;
                }
            }
        }
    }
    for (int c = 0; c < 3; ++c) out[c] = tmax(res[c] + T(0.5), T(0));
}

// Fragility windows (f64 only).
constexpr double kCullRel = 1e-5;   // relative window on culling comparisons
constexpr double kTileWin = 2e-4;   // window, in tile units, on a rect boundary
constexpr double kCeilRel = 1e-5;   // relative window on the radius ceil

inline bool near_int_boundary(double v, double grid) {
    // (int)v clamped to [0, grid]: only integer crossings in [1, grid] matter.
    if (v < 1.0 - kTileWin || v > grid + kTileWin) return false;
    double r = std::round(v);
    return r >= 1.0 && std::fabs(v - r) < kTileWin;
}

// project() (project.slang:33-90) with passFrustumClipping, computeCovariance,
// projectCovariance, computeJacobian, ndc2pix, getBoundingRect, SH colour.
template <typename T>
GOut<T> project_one(const GIn<T>& g, const T* model, const Cam<T>& cam, uint32_t degree,
                    int band3_compat) {
    GOut<T> o{};
    o.visible = false;
    o.fragile = false;
    const bool f64 = sizeof(T) == 8;
    const T* mean = g.pos;
    // passFrustumClipping (common.slang:98-119)
    T VM[16], PM[16];
    matmul<T, 4>(cam.V, model, VM);
    T vp[3];
    for (int i = 0; i < 3; ++i)
        vp[i] = VM[i * 4 + 0] * mean[0] + VM[i * 4 + 1] * mean[1] + VM[i * 4 + 2] * mean[2] +
                VM[i * 4 + 3] * T(1.0);
    if (f64 && std::fabs((double)vp[2]) < kCullRel) o.fragile = true;
    if (vp[2] <= T(0.0)) return o;
    matmul<T, 4>(cam.P, model, PM);
    T cp[4];
    for (int i = 0; i < 4; ++i)
        cp[i] = PM[i * 4 + 0] * mean[0] + PM[i * 4 + 1] * mean[1] + PM[i * 4 + 2] * mean[2] +
                PM[i * 4 + 3] * T(1.0);
    if (f64) {
        const double w = std::fabs((double)cp[3]) + 1e-30, win = kCullRel * w;
        if (std::fabs(cp[0] - 1.3 * cp[3]) < win || std::fabs(cp[0] + 1.3 * cp[3]) < win ||
            std::fabs(cp[1] - 1.3 * cp[3]) < win || std::fabs(cp[1] + 1.3 * cp[3]) < win ||
            std::fabs((double)cp[2]) < win || std::fabs(cp[2] - cp[3]) < win)
            o.fragile = true;
    }
    const T k13 = T(1.3f);
    if (cp[0] < -k13 * cp[3] || cp[0] > k13 * cp[3]) return o;
    if (cp[1] < -k13 * cp[3] || cp[1] > k13 * cp[3]) return o;
    if (cp[2] < T(0) || cp[2] > cp[3]) return o;
    const T inv_w = T(1.0) / cp[3];
    const T pp[3] = {cp[0] * inv_w, cp[1] * inv_w, cp[2] * inv_w};

    // focal = 0.5 * imageSize * focalNDC (project.slang:55)
    const T fxy[2] = {(T(0.5) * T(cam.W)) * cam.focal[0], (T(0.5) * T(cam.H)) * cam.focal[1]};

    // computeCovariance (volume.slang:20-41)
    const T* q = g.quat; const T* s = g.scale;
    const T S[9] = {s[0] * s[3], T(0), T(0), T(0), s[1] * s[3], T(0), T(0), T(0), s[2] * s[3]};
    const T x = q[0], y = q[1], z = q[2], w = q[3];
    const T R[9] = {
        T(1.0) - T(2.0) * (y * y + z * z), T(2.0) * (x * y - w * z), T(2.0) * (x * z + w * y),
        T(2.0) * (x * y + w * z), T(1.0) - T(2.0) * (x * x + z * z), T(2.0) * (y * z - w * x),
        T(2.0) * (x * z - w * y), T(2.0) * (y * z + w * x), T(1.0) - T(2.0) * (x * x + y * y)};
    T sigma[9], sigmaT[9], cov3[9];
    matmul<T, 3>(R, S, sigma);
    transpose<T, 3>(sigma, sigmaT);
    matmul<T, 3>(sigma, sigmaT, cov3);

    // projectCovariance + computeJacobian (volume.slang:44-63)
    const T W3[9] = {cam.V[0], cam.V[1], cam.V[2], cam.V[4], cam.V[5], cam.V[6],
                     cam.V[8], cam.V[9], cam.V[10]};
    const T f[2] = {fxy[0] / vp[2], fxy[1] / vp[2]};
    const T t[2] = {vp[0] / vp[2], vp[1] / vp[2]};
    const T J[9] = {f[0], T(0), -f[0] * t[0], T(0), f[1], -f[1] * t[1], T(0), T(0), T(0)};
    T Tm[9], TmT[9], inner[9], cov2[9];
    matmul<T, 3>(J, W3, Tm);
    transpose<T, 3>(Tm, TmT);
    matmul<T, 3>(cov3, TmT, inner);
    matmul<T, 3>(Tm, inner, cov2);

    // low-pass + inverse (project.slang:60-66)
    const T cov[3] = {cov2[0] + T(0.3f), cov2[3], cov2[4] + T(0.3f)};
    const T det = cov[0] * cov[2] - cov[1] * cov[1];
    if (det == T(0.0)) return o;
    const T det_inv = T(1.0) / det;
    const T conic[3] = {cov[2] * det_inv, -cov[1] * det_inv, cov[0] * det_inv};

    // extent (project.slang:69-72)
    const T mid = T(0.5) * (cov[0] + cov[2]);
    const T lambda1 = mid + std::sqrt(tmax(T(0.1f), mid * mid - det));
    const T lambda2 = mid - std::sqrt(tmax(T(0.1f), mid * mid - det));
    const T rarg = T(3.0) * std::sqrt(tmax(lambda1, lambda2));
    const T radius = std::ceil(rarg);
    if (f64) {
        const double rr = std::round((double)rarg);
        if (std::fabs(rarg - rr) < kCeilRel * std::max(1.0, (double)rarg)) o.fragile = true;
    }

    // ndc2pix (volume.slang:3-8)
    const T img[2] = {((pp[0] + T(1.0)) * T(cam.W) - T(1.0)) * T(0.5),
                      ((pp[1] + T(1.0)) * T(cam.H) - T(1.0)) * T(0.5)};
    // getBoundingRect (volume.slang:12-17) with getComputeGrid (common.slang:83-85)
    const uint32_t gx = (cam.W + BLOCK - 1) / BLOCK, gy = (cam.H + BLOCK - 1) / BLOCK;
    // p + r + BLOCK - 1: ((p + r) + 16) - 1, rounded after each operation as written
    const T bx = T(BLOCK);
    const T v0 = (img[0] - radius) / bx, v1 = (img[1] - radius) / bx;
    const T v2 = (img[0] + radius + bx - T(1)) / bx, v3 = (img[1] + radius + bx - T(1)) / bx;
    auto clampi = [](int v, uint32_t g) -> uint32_t {
        int m = std::max(0, v);
        return std::min(g, (uint32_t)m);
    };
    uint32_t rect[4] = {clampi(trunc_int(v0), gx), clampi(trunc_int(v1), gy),
                        clampi(trunc_int(v2), gx), clampi(trunc_int(v3), gy)};
    if (f64) {
        if (near_int_boundary(v0, gx) || near_int_boundary(v1, gy) ||
            near_int_boundary(v2, gx) || near_int_boundary(v3, gy))
            o.fragile = true;
    }
    const uint32_t touched = (rect[2] - rect[0]) * (rect[3] - rect[1]);
    if (touched == 0) return o;

    // direction from the camera position (common.slang:88-92), pre-model mean (project.slang:82)
    T campos[3];
    for (int i = 0; i < 3; ++i)
        campos[i] = -(cam.V[0 * 4 + i] * cam.V[0 * 4 + 3] + cam.V[1 * 4 + i] * cam.V[1 * 4 + 3] +
                      cam.V[2 * 4 + i] * cam.V[2 * 4 + 3]);
    T d[3] = {mean[0] - campos[0], mean[1] - campos[1], mean[2] - campos[2]};
    const T len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const T dir[3] = {d[0] / len, d[1] / len, d[2] / len};
    eval_sh<T>(g.sh, dir, degree, band3_compat, o.color);

    o.tiles = touched;
    o.px = img[0]; o.py = img[1]; o.depth = vp[2]; o.radius = radius;
    o.conic[0] = conic[0]; o.conic[1] = conic[1]; o.conic[2] = conic[2];
    o.opacity = g.opacity;
    std::memcpy(o.rect, rect, sizeof(rect));
    o.visible = true;
    return o;
}

template <typename T> GIn<T> load_rec(const float* r) {
    GIn<T> g;
    for (int i = 0; i < 3; ++i) g.pos[i] = T(r[i]);
    g.opacity = T(r[3]);
    for (int i = 0; i < 4; ++i) { g.quat[i] = T(r[4 + i]); g.scale[i] = T(r[8 + i]); }
    for (int i = 0; i < 48; ++i) g.sh[i] = T(r[12 + i]);
    return g;
}

template <typename T> void model_of(const uint32_t* ent_idx, const float* transforms, uint32_t i,
                                    T* M) {
    if (!transforms) {
        for (int k = 0; k < 16; ++k) M[k] = T((k % 5) == 0 ? 1 : 0);
        return;
    }
    const uint32_t e = ent_idx ? ent_idx[i] : 0;
    for (int k = 0; k < 16; ++k) M[k] = T(transforms[(size_t)e * 16 + k]);
}

}  // namespace

extern "C" {

void orc_preprocess_f32(const float* recs, uint32_t n, const uint32_t* ent_idx,
                        const float* transforms, const orc_camera* cam, uint32_t sh_degree,
                        int band3_compat, uint32_t* out) {
    const Cam<float> c = make_cam<float>(cam);
    const uint32_t deg = std::min<uint32_t>(sh_degree, 3);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        float M[16];
        model_of<float>(ent_idx, transforms, (uint32_t)i, M);
        const GOut<float> o = project_one<float>(load_rec<float>(recs + i * ORC_REC_FLOATS), M, c,
                                                 deg, band3_compat);
        uint32_t* s = out + i * ORC_SPLAT_WORDS;
        std::memset(s, 0, ORC_SPLAT_WORDS * 4);
        if (!o.visible) continue;
        s[0] = fbits(o.color[0]); s[1] = fbits(o.color[1]); s[2] = fbits(o.color[2]);
        s[3] = o.tiles;
        s[4] = fbits(o.px); s[5] = fbits(o.py); s[6] = fbits(o.depth); s[7] = fbits(o.radius);
        s[8] = fbits(o.conic[0]); s[9] = fbits(o.conic[1]); s[10] = fbits(o.conic[2]);
        s[11] = fbits(o.opacity);
    }
}

void orc_preprocess_f64(const float* recs, uint32_t n, const uint32_t* ent_idx,
                        const float* transforms, const orc_camera* cam, uint32_t sh_degree,
                        int band3_compat, double* out_splat, uint32_t* out_rect, uint8_t* fragile) {
    const Cam<double> c = make_cam<double>(cam);
    const uint32_t deg = std::min<uint32_t>(sh_degree, 3);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        double M[16];
        model_of<double>(ent_idx, transforms, (uint32_t)i, M);
        const GOut<double> o = project_one<double>(load_rec<double>(recs + i * ORC_REC_FLOATS), M,
                                                   c, deg, band3_compat);
        double* s = out_splat + i * ORC_SPLAT_WORDS;
        for (int k = 0; k < ORC_SPLAT_WORDS; ++k) s[k] = 0.0;
        if (out_rect) for (int k = 0; k < 4; ++k) out_rect[i * 4 + k] = o.visible ? o.rect[k] : 0;
        if (fragile) fragile[i] = o.fragile ? 1 : 0;
        if (!o.visible) continue;
        s[0] = o.color[0]; s[1] = o.color[1]; s[2] = o.color[2]; s[3] = (double)o.tiles;
        s[4] = o.px; s[5] = o.py; s[6] = o.depth; s[7] = o.radius;
        s[8] = o.conic[0]; s[9] = o.conic[1]; s[10] = o.conic[2]; s[11] = o.opacity;
    }
}

// prefix.slang:40-158 computes an in-place exclusive scan of Splat.tiles and the
// total; the restatement is the sequential definition of the same result.
uint64_t orc_scan_tiles(const uint32_t* splats, uint32_t n, uint32_t* offsets) {
    uint64_t acc = 0;
    for (uint32_t i = 0; i < n; ++i) {
        offsets[i] = (uint32_t)acc;
        acc += splats[(size_t)i * ORC_SPLAT_WORDS + 3];
    }
    return acc;
}

// keygen.slang:23-53: for each Gaussian with radius > 0, keys over its tile rect,
// row-major, key = (tile << 32) | bits(viewZ), value = Gaussian index.
void orc_keygen(const uint32_t* splats, const uint32_t* offsets, uint32_t n, uint32_t width,
                uint32_t height, uint64_t* keys, uint32_t* vals) {
    const uint32_t gx = (width + BLOCK - 1) / BLOCK, gy = (height + BLOCK - 1) / BLOCK;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const uint32_t* s = splats + i * ORC_SPLAT_WORDS;
        const float radius = bitsf(s[7]);
        if (radius <= 0.0f) continue;
        const float px = bitsf(s[4]), py = bitsf(s[5]);
        const float v0 = (px - radius) / 16.0f, v1 = (py - radius) / 16.0f;
        const float v2 = (px + radius + 16.0f - 1.0f) / 16.0f, v3 = (py + radius + 16.0f - 1.0f) / 16.0f;
        auto clampi = [](int v, uint32_t g) -> uint32_t { return std::min(g, (uint32_t)std::max(0, v)); };
        const uint32_t x0 = clampi(trunc_int(v0), gx), y0 = clampi(trunc_int(v1), gy);
        const uint32_t x1 = clampi(trunc_int(v2), gx), y1 = clampi(trunc_int(v3), gy);
        uint32_t off = offsets[i];
        for (uint32_t y = y0; y < y1; ++y)
            for (uint32_t x = x0; x < x1; ++x) {
                keys[off] = ((uint64_t)(y * gx + x) << 32) | (uint64_t)s[6];
                vals[off] = (uint32_t)i;
                ++off;
            }
    }
}

void orc_stable_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t k) {
    std::vector<uint64_t> idx(k);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return keys[a] < keys[b]; });
    std::vector<uint64_t> k2(k);
    std::vector<uint32_t> v2(k);
    for (uint64_t i = 0; i < k; ++i) { k2[i] = keys[idx[i]]; v2[i] = vals[idx[i]]; }
    std::memcpy(keys, k2.data(), k * 8);
    std::memcpy(vals, v2.data(), k * 4);
}

// GaussianEngine.h:234-245: binary search for the bit length.
uint32_t orc_higher_msb(uint32_t n) {
    uint32_t msb = 16, step = 16;
    while (step > 1) {
        step /= 2;
        if (n >> msb) msb += step; else msb -= step;
    }
    if (n >> msb) msb++;
    return msb;
}

uint32_t orc_radix_pass_count(uint32_t width, uint32_t height) {
    const uint32_t tx = (width + BLOCK - 1) / BLOCK, ty = (height + BLOCK - 1) / BLOCK;
    const uint32_t bits = orc_higher_msb(tx * ty) + 32;
    return (bits + 1) / 2;
}

// The four radix-*.slang dispatches of one pass, per 256-key block:
//  shuffle  (radix-shuffle.slang:39-151): stable split by the 2-bit digit into
//           temp[begin .. begin+256), per-block digit counts s0..s3 (padding
//           keys are UINT64_MAX, digit 3, and are not written);
//  prefixA/B (radix-prefixA/B.slang): exclusive scan over blocks of the counts
//           and the global digit totals;
//  mapping  (radix-mapping.slang:40-117): each block copies its digit chunks to
//           totals(d) + blockPrefix(b, d) + i.
void orc_radix4_sort(uint64_t* keys, uint32_t* vals, uint64_t k, uint32_t passes, int threads) {
    if (k == 0) return;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const uint64_t nb = (k + WORKGROUP - 1) / WORKGROUP;
    std::vector<uint64_t> tk(k);
    std::vector<uint32_t> tv(k);
    std::vector<uint32_t> cnt(nb * 4), pre(nb * 4);
    for (uint32_t pass = 0; pass < passes; ++pass) {
        const uint32_t shift = 2 * pass;
        // shuffle
#pragma omp parallel for schedule(static)
        for (int64_t b = 0; b < (int64_t)nb; ++b) {
            const uint64_t begin = (uint64_t)b * WORKGROUP;
            const uint64_t end = std::min<uint64_t>(begin + WORKGROUP, k);
            uint32_t c[4] = {0, 0, 0, 0};
            for (uint64_t i = begin; i < end; ++i) c[(keys[i] >> shift) & 3]++;
            c[3] += (uint32_t)(begin + WORKGROUP - end);  // padding keys are digit 3
            uint32_t o[4] = {0, c[0], c[0] + c[1], c[0] + c[1] + c[2]};
            for (uint64_t i = begin; i < end; ++i) {
                const uint32_t d = (keys[i] >> shift) & 3;
                const uint64_t dst = begin + o[d]++;
                tk[dst] = keys[i];
                tv[dst] = vals[i];
            }
            for (int d = 0; d < 4; ++d) cnt[b * 4 + d] = c[d];
        }
        // prefixA / prefixB: exclusive scan per digit over blocks, totals
        uint64_t tot[4] = {0, 0, 0, 0};
        for (uint64_t b = 0; b < nb; ++b)
            for (int d = 0; d < 4; ++d) { pre[b * 4 + d] = (uint32_t)tot[d]; tot[d] += cnt[b * 4 + d]; }
        const uint64_t base[4] = {0, tot[0], tot[0] + tot[1], tot[0] + tot[1] + tot[2]};
        // mapping
#pragma omp parallel for schedule(static)
        for (int64_t b = 0; b < (int64_t)nb; ++b) {
            const uint64_t begin = (uint64_t)b * WORKGROUP;
            const uint64_t end = std::min<uint64_t>(begin + WORKGROUP, k);
            uint64_t chunk = begin;
            for (int d = 0; d < 4; ++d) {
                uint32_t len = cnt[b * 4 + d];
                if (d == 3) len -= (uint32_t)(begin + WORKGROUP - end);
                const uint64_t dst = base[d] + pre[b * 4 + d];
                for (uint32_t i = 0; i < len; ++i) {
                    keys[dst + i] = tk[chunk + i];
                    vals[dst + i] = tv[chunk + i];
                }
                chunk += len;
            }
        }
    }
}

// range.slang:18-35 after fillBuffer(ranges, 0).
void orc_tile_ranges(const uint64_t* keys, uint64_t k, uint32_t n_tiles, uint32_t* ranges) {
    std::memset(ranges, 0, (size_t)n_tiles * 8);
    for (uint64_t i = 0; i < k; ++i) {
        const uint32_t cur = (uint32_t)(keys[i] >> 32);
        if (i == 0) ranges[cur * 2 + 0] = 0;
        else {
            const uint32_t prev = (uint32_t)(keys[i - 1] >> 32);
            if (cur != prev) { ranges[prev * 2 + 1] = (uint32_t)i; ranges[cur * 2 + 0] = (uint32_t)i; }
        }
        if (i == k - 1) ranges[cur * 2 + 1] = (uint32_t)(i + 1);
    }
}

// blend.slang:24-105, per pixel: front to back over the tile's list.
void orc_blend_f32(const uint32_t* splats, const uint32_t* vals, const uint32_t* ranges,
                   uint32_t width, uint32_t height, float* image, float* final_T,
                   uint32_t* n_contrib, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const uint32_t gx = (width + BLOCK - 1) / BLOCK, gy = (height + BLOCK - 1) / BLOCK;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t tile = 0; tile < (int64_t)gx * gy; ++tile) {
        const uint32_t tx = (uint32_t)(tile % gx), ty = (uint32_t)(tile / gx);
        const uint32_t start = ranges[tile * 2], end = ranges[tile * 2 + 1];
        for (uint32_t ly = 0; ly < BLOCK; ++ly)
            for (uint32_t lx = 0; lx < BLOCK; ++lx) {
                const uint32_t pxl = tx * BLOCK + lx, pyl = ty * BLOCK + ly;
                if (pxl >= width || pyl >= height) continue;
                const float fx = (float)pxl, fy = (float)pyl;
                float T = 1.0f, C[3] = {0, 0, 0};
                uint32_t last = 0;
                for (uint32_t k = start; k < end; ++k) {
                    const uint32_t* s = splats + (size_t)vals[k] * ORC_SPLAT_WORDS;
                    const float dx = bitsf(s[4]) - fx, dy = bitsf(s[5]) - fy;
                    const float cx = bitsf(s[8]), cy = bitsf(s[9]), cz = bitsf(s[10]);
                    const float power = -0.5f * (cx * dx * dx + cz * dy * dy) - cy * dx * dy;
                    if (power > 0.0f) continue;
                    const float alpha = std::fmin(0.99f, bitsf(s[11]) * std::exp(power));
                    if (alpha < 1.0f / 255.0f) continue;
                    if (T * (1.0f - alpha) < 0.0001f) break;
                    for (int c = 0; c < 3; ++c) C[c] = C[c] + bitsf(s[c]) * alpha * T;
                    T = T * (1.0f - alpha);
                    last = k - start + 1;
                }
                const size_t p = (size_t)pyl * width + pxl;
                for (int c = 0; c < 3; ++c) image[p * 3 + c] = C[c];
                if (final_T) final_T[p] = T;
                if (n_contrib) n_contrib[p] = last;
            }
    }
}

void orc_blend_pair_count(const uint32_t* splats, const uint32_t* vals, const uint32_t* ranges,
                          uint32_t width, uint32_t height, uint64_t* evaluated, uint64_t* contributing,
                          int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const uint32_t gx = (width + BLOCK - 1) / BLOCK, gy = (height + BLOCK - 1) / BLOCK;
    uint64_t ev = 0, co = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : ev, co)
    for (int64_t tile = 0; tile < (int64_t)gx * gy; ++tile) {
        const uint32_t tx = (uint32_t)(tile % gx), ty = (uint32_t)(tile / gx);
        const uint32_t start = ranges[tile * 2], end = ranges[tile * 2 + 1];
        for (uint32_t ly = 0; ly < BLOCK; ++ly)
            for (uint32_t lx = 0; lx < BLOCK; ++lx) {
                const uint32_t pxl = tx * BLOCK + lx, pyl = ty * BLOCK + ly;
                if (pxl >= width || pyl >= height) continue;
                const float fx = (float)pxl, fy = (float)pyl;
                float T = 1.0f;
                for (uint32_t k = start; k < end; ++k) {
                    ++ev;
                    const uint32_t* s = splats + (size_t)vals[k] * ORC_SPLAT_WORDS;
                    const float dx = bitsf(s[4]) - fx, dy = bitsf(s[5]) - fy;
                    const float cx = bitsf(s[8]), cy = bitsf(s[9]), cz = bitsf(s[10]);
                    const float power = -0.5f * (cx * dx * dx + cz * dy * dy) - cy * dx * dy;
                    if (power > 0.0f) continue;
                    const float alpha = std::fmin(0.99f, bitsf(s[11]) * std::exp(power));
                    if (alpha < 1.0f / 255.0f) continue;
                    if (T * (1.0f - alpha) < 0.0001f) break;
                    ++co;
                    T = T * (1.0f - alpha);
                }
            }
    }
    *evaluated = ev;
    *contributing = co;
}

// Decision windows for the FP64 blend's fragile flag.
static constexpr double kPowWin = 1e-6, kAlphaRel = 1e-4, kTermRel = 1e-4;

void orc_blend_f64(const double* sp, const uint32_t* vals, const uint32_t* ranges, uint32_t width,
                   uint32_t height, double* image, double* final_T, uint32_t* n_contrib,
                   uint8_t* fragile) {
    const uint32_t gx = (width + BLOCK - 1) / BLOCK, gy = (height + BLOCK - 1) / BLOCK;
    const double a_min = (double)(1.0f / 255.0f);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t tile = 0; tile < (int64_t)gx * gy; ++tile) {
        const uint32_t tx = (uint32_t)(tile % gx), ty = (uint32_t)(tile / gx);
        const uint32_t start = ranges[tile * 2], end = ranges[tile * 2 + 1];
        for (uint32_t ly = 0; ly < BLOCK; ++ly)
            for (uint32_t lx = 0; lx < BLOCK; ++lx) {
                const uint32_t pxl = tx * BLOCK + lx, pyl = ty * BLOCK + ly;
                if (pxl >= width || pyl >= height) continue;
                double T = 1.0, C[3] = {0, 0, 0};
                uint32_t last = 0;
                bool frag = false;
                for (uint32_t k = start; k < end; ++k) {
                    const double* s = sp + (size_t)vals[k] * ORC_SPLAT_WORDS;
                    const double dx = s[4] - pxl, dy = s[5] - pyl;
                    const double power = -0.5 * (s[8] * dx * dx + s[10] * dy * dy) - s[9] * dx * dy;
                    if (std::fabs(power) < kPowWin) frag = true;
                    if (power > 0.0) continue;
                    const double alpha = std::fmin(0.99, s[11] * std::exp(power));
                    if (std::fabs(alpha - a_min) < kAlphaRel * a_min) frag = true;
                    if (alpha < a_min) continue;
                    const double tn = T * (1.0 - alpha);
                    if (std::fabs(tn - 1e-4) < kTermRel * 1e-4) frag = true;
                    if (tn < 1e-4) break;
                    for (int c = 0; c < 3; ++c) C[c] += s[c] * alpha * T;
                    T = tn;
                    last = k - start + 1;
                }
                const size_t p = (size_t)pyl * width + pxl;
                for (int c = 0; c < 3; ++c) image[p * 3 + c] = C[c];
                if (final_T) final_T[p] = T;
                if (n_contrib) n_contrib[p] = last;
                if (fragile) fragile[p] = frag ? 1 : 0;
            }
    }
}

uint64_t orc_frame_f32(const float* recs, uint32_t n, const orc_camera* cam, uint32_t sh_degree,
                       float* image, int threads, uint32_t tile_rows_limit) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    std::vector<uint32_t> splats((size_t)n * ORC_SPLAT_WORDS), offs(n);
    orc_preprocess_f32(recs, n, nullptr, nullptr, cam, sh_degree, 1, splats.data());
    const uint64_t k = orc_scan_tiles(splats.data(), n, offs.data());
    std::vector<uint64_t> keys(k);
    std::vector<uint32_t> vals(k);
    orc_keygen(splats.data(), offs.data(), n, cam->width, cam->height, keys.data(), vals.data());
    orc_radix4_sort(keys.data(), vals.data(), k, orc_radix_pass_count(cam->width, cam->height), threads);
    const uint32_t gx = (cam->width + BLOCK - 1) / BLOCK, gy = (cam->height + BLOCK - 1) / BLOCK;
    std::vector<uint32_t> ranges((size_t)gx * gy * 2);
    orc_tile_ranges(keys.data(), k, gx * gy, ranges.data());
    uint32_t h = cam->height;
    if (tile_rows_limit && tile_rows_limit < gy) h = tile_rows_limit * BLOCK;
    orc_blend_f32(splats.data(), vals.data(), ranges.data(), cam->width, h, image, nullptr, nullptr,
                  threads);
    return k;
}

}  // extern "C"
