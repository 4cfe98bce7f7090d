// host_util.cpp — host-side helpers of the C ABI: camera matrices, key width,
// seeded scenes and the PLY reader. No device code.
//
// Camera arithmetic restates the reference's math library so that matrices
// are bit-identical to what the reference computes:
//   dot:   Dot2 of Ogita, Rump and Oishi ("Accurate sum and dot product",
//          SIAM J. Sci. Comput. 2005, Algorithm 5.3): TwoProduct via fma,
//          TwoSum, error terms accumulated as c + (q + r)
//          (reference: math/include/torpedo/math/vec3.h:239-252, vec4.h:248-264)
//   cross: Kahan's difference of products a*b - c*d with an fma error term
//          (reference: math/include/torpedo/math/common.h:12-17, vec3.h:230-236)
//   v / s: v * (1 / s) (reference: vec3.h:210-214)
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/tpdsplat.h"

namespace {

inline void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float z = s - a;
    e = (a - (s - z)) + (b - z);
}

inline void two_prod(float a, float b, float& p, float& e) {
    p = a * b;
    e = std::fma(a, b, -p);
}

float dot2(const float* a, const float* b, int n) {
    float s, c;
    two_prod(a[0], b[0], s, c);
    for (int i = 1; i < n; ++i) {
        float h, r, q;
        two_prod(a[i], b[i], h, r);
        two_sum(s, h, s, q);
        c = c + (q + r);
    }
    return s + c;
}

inline float diff_of_products(float a, float b, float c, float d) {
    const float cd = c * d;
    const float err = std::fma(-c, d, cd);
    const float dop = std::fma(a, b, -cd);
    return dop + err;
}

void cross3(const float* u, const float* v, float* o) {
    o[0] = diff_of_products(u[1], v[2], u[2], v[1]);
    o[1] = diff_of_products(u[2], v[0], u[0], v[2]);
    o[2] = diff_of_products(u[0], v[1], u[1], v[0]);
}

void normalize3(float* v) {
    const float len = std::sqrt(dot2(v, v, 3));
    const float inv = 1.0f / len;
    v[0] *= inv;
    v[1] *= inv;
    v[2] *= inv;
}

constexpr double kC0 = 0.28209479177387814;

}  // namespace

extern "C" {

void tpd_look_at(const float eye[3], const float center[3], const float up[3], float view[16]) {
    float z[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
    normalize3(z);
    float x[3];
    cross3(z, up, x);
    normalize3(x);
    float y[3];
    cross3(z, x, y);
    normalize3(y);
    const float out[16] = {x[0], x[1], x[2], -dot2(x, eye, 3), y[0], y[1], y[2], -dot2(y, eye, 3),
                           z[0], z[1], z[2], -dot2(z, eye, 3), 0.f,  0.f,  0.f,  1.f};
    std::memcpy(view, out, sizeof(out));
}

void tpd_perspective(uint32_t width, uint32_t height, float fov_y_degrees, float near_plane, float far_plane,
                     float proj[16]) {
    const float aspect = static_cast<float>(width) / static_cast<float>(height);
    float fy;
    if (fov_y_degrees > 0.f) {
        const float fov = fov_y_degrees * 3.14159265358979323846f / 180.f;
        fy = 1.f / std::tan(fov * 0.5f);
    } else {
        fy = 1.7320508075688772f;  // sqrt(3): 60 degrees, the constructor's default
    }
    const float fx = fy / aspect;
    const float za = near_plane / (near_plane - far_plane);
    const float zb = near_plane * far_plane / (far_plane - near_plane);
    const float out[16] = {fx, 0.f, 0.f, 0.f, 0.f, fy, 0.f, 0.f, 0.f, 0.f, za, zb, 0.f, 0.f, 1.f, 0.f};
    std::memcpy(proj, out, sizeof(out));
}

void tpd_mat4_mul(const float a[16], const float b[16], float out[16]) {
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            const float col[4] = {b[0 * 4 + j], b[1 * 4 + j], b[2 * 4 + j], b[3 * 4 + j]};
            r[i * 4 + j] = dot2(a + i * 4, col, 4);
        }
    std::memcpy(out, r, sizeof(r));
}

// getHigherMSB (GaussianEngine.h:234-245): a binary search for the bit length
// starting at 16 with steps 8, 4, 2, 1, plus one final correction.
uint32_t tpd_key_bits_for_tiles(uint32_t tiles) {
    uint32_t msb = 16, step = 16;
    while (step > 1) {
        step /= 2;
        msb = (tiles >> msb) ? msb + step : msb - step;
    }
    if (tiles >> msb) ++msb;
    return msb + 32;
}

void tpd_synthetic_scene(uint64_t seed, uint32_t n, float mean_box, float* means, float* log_scales, float* quats,
                         float* opacity_logits, float* sh, void* records) {
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> normal(0.0, 1.0);
    std::uniform_real_distribution<double> box(-double(mean_box), double(mean_box));
    float* rec = static_cast<float*>(records);
    for (uint32_t i = 0; i < n; ++i) {
        double m[3], ls[3], q[4], logit, c[48];
        for (int k = 0; k < 3; ++k) m[k] = mean_box > 0.f ? box(rng) : normal(rng);
        for (int k = 0; k < 3; ++k) ls[k] = -4.0 + 0.5 * normal(rng);
        double qn = 0.0;
        for (int k = 0; k < 4; ++k) {
            q[k] = normal(rng);
            qn += q[k] * q[k];
        }
        qn = std::sqrt(qn);
        for (int k = 0; k < 4; ++k) q[k] /= qn;
        logit = normal(rng);
        for (int k = 0; k < 48; ++k) c[k] = 0.2 * normal(rng);
        if (means) for (int k = 0; k < 3; ++k) means[size_t(i) * 3 + k] = float(m[k]);
        if (log_scales) for (int k = 0; k < 3; ++k) log_scales[size_t(i) * 3 + k] = float(ls[k]);
        if (quats) for (int k = 0; k < 4; ++k) quats[size_t(i) * 4 + k] = float(q[k]);
        if (opacity_logits) opacity_logits[i] = float(logit);
        if (sh) for (int k = 0; k < 48; ++k) sh[size_t(i) * 48 + k] = float(c[k]);
        if (rec) {
            float* r = rec + size_t(i) * 60;
            for (int k = 0; k < 3; ++k) r[k] = float(m[k]);
            r[3] = float(1.0 / (1.0 + std::exp(-logit)));
            for (int k = 0; k < 4; ++k) r[4 + k] = float(q[k]);
            for (int k = 0; k < 3; ++k) r[8 + k] = float(std::exp(ls[k]));
            r[11] = 1.0f;
            for (int k = 0; k < 48; ++k) r[12 + k] = float(c[k]);
        }
    }
}

void tpd_random_points(uint64_t seed, uint32_t n, float radius, const float center[3], float min_scale,
                       float max_scale, float min_opacity, float max_opacity, void* records) {
    std::mt19937 rng(static_cast<uint32_t>(seed));
    std::uniform_real_distribution<float> dpos(-1.0f, 1.0f), dop(min_opacity, max_opacity),
        dscale(min_scale, max_scale), dsh(0.0f, 1.0f);
    const float c0 = float(kC0);
    float* rec = static_cast<float*>(records);
    for (uint32_t i = 0; i < n; ++i) {
        float* r = rec + size_t(i) * 60;
        std::memset(r, 0, 240);
        const float px = dpos(rng), py = dpos(rng), pz = dpos(rng);
        r[0] = px * radius + center[0];
        r[1] = py * radius + center[1];
        r[2] = pz * radius + center[2];
        r[3] = dop(rng);
        r[4] = 0.f; r[5] = 0.f; r[6] = 0.f; r[7] = 1.f;
        const float sx = dscale(rng), sy = dscale(rng), sz = dscale(rng);
        r[8] = sx; r[9] = sy; r[10] = sz; r[11] = 1.f;
        const float cr = dsh(rng), cg = dsh(rng), cb = dsh(rng);
        r[12] = (cr - 0.5f) / c0;  // rgb2sh (GaussianGeometry.h:38-46)
        r[13] = (cg - 0.5f) / c0;
        r[14] = (cb - 0.5f) / c0;
    }
}

// GaussianPoint::fromModel (GaussianGeometry.cpp:59-127): x, y, z; rot_0..3
// stored w first in the file and kept as (x, y, z, w), normalised; scale_0..2
// through exp; opacity through sigmoid; f_dc_0..2 then the f_rest_* that
// follow them, at most 48 floats.
int tpd_load_ply(const char* path, void* records, uint32_t* n_out) {
    if (!path || !n_out) return TPD_ERR_ARG;
    std::ifstream f(path, std::ios::binary);
    if (!f) return TPD_ERR_IO;
    std::string line;
    if (!std::getline(f, line) || line.rfind("ply", 0) != 0) return TPD_ERR_IO;
    bool binary = false, in_vertex = false, vertex_seen = false;
    uint64_t count = 0;
    struct Prop { std::string name; int size; char type; };  // type: f, d, i, u
    std::vector<Prop> props;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ss(line);
        std::string w;
        ss >> w;
        if (w == "format") {
            std::string fmt;
            ss >> fmt;
            if (fmt == "binary_little_endian") binary = true;
            else if (fmt == "ascii") binary = false;
            else return TPD_ERR_IO;
        } else if (w == "element") {
            std::string name;
            ss >> name;
            in_vertex = name == "vertex";
            if (in_vertex) {
                if (vertex_seen) return TPD_ERR_IO;
                vertex_seen = true;
                ss >> count;
            } else if (!vertex_seen) {
                return TPD_ERR_IO;  // elements before the vertices are not supported
            }
        } else if (w == "property" && in_vertex) {
            std::string t, name;
            ss >> t >> name;
            Prop p{name, 4, 'f'};
            if (t == "float" || t == "float32") p = {name, 4, 'f'};
            else if (t == "double" || t == "float64") p = {name, 8, 'd'};
            else if (t == "int" || t == "int32") p = {name, 4, 'i'};
            else if (t == "uint" || t == "uint32") p = {name, 4, 'u'};
            else if (t == "uchar" || t == "uint8") p = {name, 1, 'u'};
            else if (t == "char" || t == "int8") p = {name, 1, 'i'};
            else if (t == "short" || t == "int16") p = {name, 2, 'i'};
            else if (t == "ushort" || t == "uint16") p = {name, 2, 'u'};
            else return TPD_ERR_IO;
            props.push_back(p);
        } else if (w == "end_header") {
            break;
        }
    }
    if (!vertex_seen || count > 0xFFFFFFFFull) return TPD_ERR_IO;
    *n_out = uint32_t(count);
    if (!records) return TPD_OK;

    auto find = [&](const char* name) -> int {
        for (size_t i = 0; i < props.size(); ++i) if (props[i].name == name) return int(i);
        return -1;
    };
    const int ix = find("x"), iy = find("y"), iz = find("z"), iop = find("opacity");
    const int ir[4] = {find("rot_0"), find("rot_1"), find("rot_2"), find("rot_3")};
    const int is[3] = {find("scale_0"), find("scale_1"), find("scale_2")};
    const int idc = find("f_dc_0");
    if (ix < 0 || iy < 0 || iz < 0 || iop < 0 || idc < 0 || ir[0] < 0 || ir[3] < 0 || is[0] < 0 || is[2] < 0)
        return TPD_ERR_IO;
    int n_rest = 0;
    for (const auto& p : props) if (p.name.rfind("f_rest_", 0) == 0) ++n_rest;
    const int n_feat = std::min(3 + n_rest, 48);

    // one record from the properties' values (get(k): property k as a double)
    float* rec = static_cast<float*>(records);
    auto fill = [&](float* r, auto&& get) {
        std::memset(r, 0, 240);
        r[0] = float(get(ix));
        r[1] = float(get(iy));
        r[2] = float(get(iz));
        r[3] = 1.f / (1.f + std::exp(-float(get(iop))));
        float q[4] = {float(get(ir[1])), float(get(ir[2])), float(get(ir[3])), float(get(ir[0]))};
        const float inv = 1.0f / std::sqrt(dot2(q, q, 4));
        for (int k = 0; k < 4; ++k) r[4 + k] = q[k] * inv;
        for (int k = 0; k < 3; ++k) r[8 + k] = std::exp(float(get(is[k])));
        r[11] = 1.f;
        // features: f_dc_0..2 and the properties that follow them, in file order
        for (int k = 0; k < n_feat; ++k) {
            const int pi = idc + k;
            r[12 + k] = pi < int(props.size()) ? float(get(pi)) : 0.f;
        }
    };
    if (binary) {
        // fixed-size vertices: read kBlock of them at a time and decode each
        // property from its offset in the vertex (little-endian, as the
        // format says)
        std::vector<size_t> off(props.size());
        size_t stride = 0;
        for (size_t k = 0; k < props.size(); ++k) {
            off[k] = stride;
            stride += size_t(props[k].size);
        }
        bool all_float = true;  // the usual 3DGS layout: every property a float32
        for (const auto& p : props) all_float = all_float && p.type == 'f';
        // vertices [j0, j1) of a block that starts at vertex v0
        auto decode = [&](const unsigned char* block, uint64_t v0, uint64_t j0, uint64_t j1) {
            for (uint64_t j = j0; j < j1; ++j) {
                const unsigned char* vp = block + j * stride;
                float* r = rec + (v0 + j) * 60;
                if (all_float) {
                    fill(r, [&](int k) -> double {
                        float t;
                        std::memcpy(&t, vp + 4 * size_t(k), 4);
                        return t;
                    });
                    continue;
                }
                fill(r, [&](int k) -> double {
                    const unsigned char* b = vp + off[k];
                    switch (props[k].type) {
                        case 'f': { float t; std::memcpy(&t, b, 4); return t; }
                        case 'd': { double t; std::memcpy(&t, b, 8); return t; }
                        case 'i':
                            if (props[k].size == 4) { int32_t t; std::memcpy(&t, b, 4); return t; }
                            if (props[k].size == 2) { int16_t t; std::memcpy(&t, b, 2); return t; }
                            return static_cast<int8_t>(b[0]);
                        default:
                            if (props[k].size == 4) { uint32_t t; std::memcpy(&t, b, 4); return t; }
                            if (props[k].size == 2) { uint16_t t; std::memcpy(&t, b, 2); return t; }
                            return b[0];
                    }
                });
            }
        };
        // blocks of kBlock vertices, each decoded by up to kThreadsMax host
        // threads (records are independent: the result does not depend on
        // the split)
        constexpr uint64_t kBlock = 1u << 17;
        constexpr unsigned kThreadsMax = 16;
        const unsigned hw = std::max(1u, std::min(kThreadsMax, std::thread::hardware_concurrency()));
        std::vector<unsigned char> block;
        for (uint64_t v0 = 0; v0 < count; v0 += kBlock) {
            const uint64_t nv = std::min(kBlock, count - v0);
            block.resize(nv * stride);
            if (!f.read(reinterpret_cast<char*>(block.data()), std::streamsize(nv * stride))) return TPD_ERR_IO;
            const unsigned nt = unsigned(std::min<uint64_t>(hw, (nv + 4095) / 4096));
            if (nt <= 1) {
                decode(block.data(), v0, 0, nv);
                continue;
            }
            std::vector<std::thread> pool;
            pool.reserve(nt - 1);
            for (unsigned t = 1; t < nt; ++t)
                pool.emplace_back(decode, block.data(), v0, nv * t / nt, nv * (t + 1) / nt);
            decode(block.data(), v0, 0, nv / nt);
            for (auto& th : pool) th.join();
        }
    } else {
        std::vector<double> vals(props.size());
        for (uint64_t v = 0; v < count; ++v) {
            for (size_t k = 0; k < props.size(); ++k)
                if (!(f >> vals[k])) return TPD_ERR_IO;
            fill(rec + v * 60, [&](int k) { return vals[k]; });
        }
    }
    return TPD_OK;
}

}  // extern "C"
