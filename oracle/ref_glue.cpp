// ref_glue.cpp — C entry points over the reference's own host C++, compiled
// from the reference sources by oracle/build_ref.py into oracle/_ref/.
// TEST INFRASTRUCTURE ONLY: used to generate the golden fixtures in
// tests/golden/ (camera matrices, pass counts, PLY records).
//
// Reference code called (paths relative to the reference project root):
//   tpd::PerspectiveCamera  torpedo/extension/src/PerspectiveCamera.cpp
//   tpd::Camera::lookAt     torpedo/rendering/src/Camera.cpp
//   tpd::math::mul          torpedo/math/include/torpedo/math/mat4.h:256-264
//   GaussianPoint::fromModel torpedo/volumetric/src/GaussianGeometry.cpp:59-127
//   GaussianEngine::getHigherMSB torpedo/volumetric/include/torpedo/volumetric/GaussianEngine.h:234-245
//     (its body alone, extracted by build_ref.py into a generated file)
#include <torpedo/extension/PerspectiveCamera.h>
#include <torpedo/volumetric/GaussianGeometry.h>

#include "seeded_random_device.h"

#include <cstdint>
#include <cstring>

uint32_t ref_higher_msb_impl(uint32_t n);  // generated from GaussianEngine.h

namespace {
unsigned int g_random_seed = 0;
int g_arg_probe = 0;
int arg_probe_next() { return g_arg_probe++; }
int arg_probe_first(int a, int) { return a; }
}  // namespace

// The seed GaussianPoint::random draws from std::random_device (see
// seeded_random_device.h).
unsigned int std::tpd_seeded_random_device::operator()() const { return g_random_seed; }

extern "C" {

// updateCameraBuffer (GaussianEngine.cpp:764-775) packing: view, proj*view, (P00, P11).
void ref_camera(const float eye[3], const float center[3], const float up[3], uint32_t w, uint32_t h, float fov_deg,
                float near_plane, float far_plane, float view[16], float proj[16], float projview[16], float focal[2]) {
    tpd::PerspectiveCamera cam(w, h);
    cam.setNear(near_plane);
    cam.setFar(far_plane);
    if (fov_deg > 0.f) cam.setVerticalFov(fov_deg);  // refreshes the projection with near / far
    cam.lookAt({eye[0], eye[1], eye[2]}, {center[0], center[1], center[2]}, {up[0], up[1], up[2]});
    std::memcpy(view, cam.getViewMatrixData(), 64);
    std::memcpy(proj, cam.getProjectionData(), 64);
    auto projection = tpd::mat4{cam.getProjectionData()};
    focal[0] = projection[0, 0];
    focal[1] = projection[1, 1];
    projection = tpd::math::mul(projection, cam.getViewMatrix());
    std::memcpy(projview, projection.data_ptr(), 64);
}

void ref_mat4_mul(const float a[16], const float b[16], float out[16]) {
    const auto r = tpd::math::mul(tpd::mat4{a}, tpd::mat4{b});
    std::memcpy(out, r.data_ptr(), 64);
}

uint32_t ref_higher_msb(uint32_t n) { return ref_higher_msb_impl(n); }

uint32_t ref_gaussian_point_size() { return sizeof(tpd::GaussianPoint); }

// fromModel: returns the count; fills records (n x 60 floats) when not NULL.
uint32_t ref_from_model(const char* path, float* records, uint32_t cap) {
    const auto pts = tpd::GaussianPoint::fromModel(path);
    const uint32_t n = static_cast<uint32_t>(pts.size());
    if (records) std::memcpy(records, pts.data(), sizeof(tpd::GaussianPoint) * std::min(n, cap));
    return n;
}

// GaussianPoint::random (GaussianGeometry.cpp:8-32) with its std::mt19937
// seeded by `seed`: n records.
void ref_random_points(uint32_t seed, uint32_t n, float radius, const float center[3], float min_scale,
                       float max_scale, float min_opacity, float max_opacity, float* records) {
    g_random_seed = seed;
    const auto pts = tpd::GaussianPoint::random(n, radius, {center[0], center[1], center[2]}, min_scale, max_scale,
                                                min_opacity, max_opacity);
    std::memcpy(records, pts.data(), sizeof(tpd::GaussianPoint) * n);
}

// 1 when this build evaluates function arguments right to left (g++ does for
// rgb2sh(dist_sh(rng), dist_sh(rng), dist_sh(rng)), GaussianGeometry.cpp:29;
// clang, the reference's compiler, left to right).
int ref_args_right_to_left() {
    g_arg_probe = 0;
    return arg_probe_first(arg_probe_next(), arg_probe_next()) == 1 ? 1 : 0;
}

}  // extern "C"
