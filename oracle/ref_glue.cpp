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

#include <cstdint>
#include <cstring>

uint32_t ref_higher_msb_impl(uint32_t n);  // generated from GaussianEngine.h

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

}  // extern "C"
