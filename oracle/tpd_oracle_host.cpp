// tpd_oracle_host.cpp — the oracle's own inputs: seeded synthetic scenes and
// camera matrices, so that the CPU baselines and checks need nothing from the
// product library.
//
// TEST INFRASTRUCTURE ONLY (see tpd_oracle.h).
//
// Camera maths restates the reference's (paths relative to its project root):
//   Camera::lookAt                     rendering/src/Camera.cpp:3-16
//   PerspectiveCamera projection       extension/src/PerspectiveCamera.cpp:9-23
//   math::mul (mat4 x mat4)            math/include/torpedo/math/mat4.h:256-264
// with the math library's accurate arithmetic: dot products by the Dot2
// algorithm of Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26(6), 2005,
// Algorithm 5.3; vec3.h:239-252, vec4.h:248-264), cross products by Kahan's
// difference of products (common.h:12-17, vec3.h:230-236), vector / scalar as a
// multiply by the reciprocal (vec3.h:210-214). tests/test_golden_host.py pins
// these against the reference's own C++ compiled from its sources.
#include <cmath>
#include <cstring>
#include <random>

#include "tpd_oracle.h"

namespace {

// Dot2: error-free products and sums, errors accumulated separately.
float dot_accurate(const float* a, const float* b, int n) {
    float sum = a[0] * b[0];
    float err = std::fma(a[0], b[0], -sum);
    for (int i = 1; i < n; ++i) {
        const float p = a[i] * b[i];
        const float pe = std::fma(a[i], b[i], -p);
        const float s = sum + p;
        const float bv = s - sum;
        const float se = (sum - (s - bv)) + (p - bv);
        sum = s;
        err = err + (se + pe);
    }
    return sum + err;
}

// a*b - c*d with Kahan's fma correction.
float dop(float a, float b, float c, float d) {
    const float cd = c * d;
    return std::fma(a, b, -cd) + std::fma(-c, d, cd);
}

void unit(float v[3]) {
    const float r = 1.0f / std::sqrt(dot_accurate(v, v, 3));
    for (int k = 0; k < 3; ++k) v[k] *= r;
}

void cross(const float a[3], const float b[3], float o[3]) {
    o[0] = dop(a[1], b[2], a[2], b[1]);
    o[1] = dop(a[2], b[0], a[0], b[2]);
    o[2] = dop(a[0], b[1], a[1], b[0]);
}

}  // namespace

extern "C" {

void orc_look_at(const float eye[3], const float center[3], const float up[3], float view[16]) {
    float f[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
    unit(f);
    float s[3], u[3];
    cross(f, up, s);
    unit(s);
    cross(f, s, u);  // y-down: y = cross(z, x)
    unit(u);
    const float* rows[3] = {s, u, f};
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) view[r * 4 + c] = rows[r][c];
        view[r * 4 + 3] = -dot_accurate(rows[r], eye, 3);
    }
    view[12] = view[13] = view[14] = 0.0f;
    view[15] = 1.0f;
}

void orc_perspective(uint32_t width, uint32_t height, float fov_y_degrees, float near_plane, float far_plane,
                     float proj[16]) {
    std::memset(proj, 0, 16 * sizeof(float));
    const float fy = fov_y_degrees > 0.0f ? 1.0f / std::tan(fov_y_degrees * 3.14159265358979323846f / 180.0f * 0.5f)
                                          : 1.7320508075688772f;
    proj[0] = fy / (float(width) / float(height));
    proj[5] = fy;
    proj[10] = near_plane / (near_plane - far_plane);  // reversed Z: near -> 1, far -> 0
    proj[11] = near_plane * far_plane / (far_plane - near_plane);
    proj[14] = 1.0f;
}

void orc_mat4_mul(const float a[16], const float b[16], float out[16]) {
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            const float col[4] = {b[j], b[4 + j], b[8 + j], b[12 + j]};
            r[i * 4 + j] = dot_accurate(a + 4 * i, col, 4);
        }
    std::memcpy(out, r, sizeof(r));
}

// The seeded synthetic scene of the five workloads: mt19937_64(seed), normals
// drawn in double (std::normal_distribution), per Gaussian in this order:
// mean (3 normals, or 3 uniforms in [-box, box]), log-scale (-4 + 0.5 N),
// quaternion (4 normals, normalised; stored x, y, z, w), opacity logit (N),
// 48 SH coefficients (0.2 N). Records activate them: sigmoid opacity, exp
// scale with modifier 1.
void orc_synthetic_scene(uint64_t seed, uint32_t n, float mean_box, float* records) {
    std::mt19937_64 gen(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    std::uniform_real_distribution<double> ud(-double(mean_box), double(mean_box));
    for (uint32_t i = 0; i < n; ++i) {
        float* r = records + size_t(i) * ORC_REC_FLOATS;
        double v[3];
        for (double& x : v) x = mean_box > 0.0f ? ud(gen) : nd(gen);
        for (int k = 0; k < 3; ++k) r[k] = float(v[k]);
        for (int k = 0; k < 3; ++k) r[8 + k] = float(std::exp(-4.0 + 0.5 * nd(gen)));
        r[11] = 1.0f;
        double q[4], qq = 0.0;
        for (double& x : q) {
            x = nd(gen);
            qq += x * x;
        }
        const double ql = std::sqrt(qq);
        for (int k = 0; k < 4; ++k) r[4 + k] = float(q[k] / ql);
        r[3] = float(1.0 / (1.0 + std::exp(-nd(gen))));
        for (int k = 0; k < 48; ++k) r[12 + k] = float(0.2 * nd(gen));
    }
}

}  // extern "C"
