/*
 * tpdsplat.hpp — C++ face of libtpdsplat, shaped like the reference's
 * tpd::GaussianEngine (volumetric/include/torpedo/volumetric/GaussianEngine.h:15-27)
 * so a renderer keeps its compile / getTransformHost().transform /
 * rasterFrame calls. Header-only over the C ABI in tpdsplat.h; errors become
 * exceptions here (tpdsplat::Error, a std::runtime_error, as the reference
 * throws), never across the library boundary.
 *
 * Differences from the reference class, by design:
 *  - compile() takes the point array (and an optional per-point entity index)
 *    that the reference pulls out of its entt Scene with
 *    Scene::dataAll<GaussianPoint>() and buildEntityMap<GaussianPoint>();
 *  - TransformHost::transform takes the entity's index (its value in that
 *    entity map) instead of an entt handle;
 *  - draw() has no swapchain: readImageRGBA8 / readImageRGB copy the image to
 *    host memory (or device memory with the *_device forms of tpd_read_image).
 */
#ifndef TPDSPLAT_HPP
#define TPDSPLAT_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "tpdsplat.h"

namespace tpdsplat {

/* The reference's 240-byte record (GaussianGeometry.h:10-18), opacity and
 * scale already activated as GaussianPoint::fromModel / random leave them. */
struct GaussianPoint {
    float position[3];
    float opacity;
    float quaternion[4];  // x, y, z, w
    float scale[4];       // x, y, z, w = modifier
    float sh[48];
};
static_assert(sizeof(GaussianPoint) == 240, "GaussianPoint must stay 240 bytes");

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const noexcept { return code_; }

private:
    int code_;
};

inline void check(int code, const tpd_engine* e, const char* call) {
    if (code == TPD_OK) return;
    std::string msg = std::string(call) + ": " + tpd_status_string(code);
    const char* detail = e ? tpd_last_error(e) : nullptr;
    if (detail && *detail) msg += std::string(" (") + detail + ")";
    throw Error(code, msg);
}

/* A camera as the reference's Camera / PerspectiveCamera hold it: row-major
 * world->view matrix, projection, and the image size. */
struct Camera {
    float view[16];
    float projection[16];
    uint32_t width;
    uint32_t height;

    /* Camera::lookAt + PerspectiveCamera with the reference's arithmetic. */
    static Camera lookAt(const float eye[3], const float center[3], const float up[3], uint32_t width,
                         uint32_t height, float fovYDegrees = 60.0f, float nearPlane = 0.2f, float farPlane = 100.0f) {
        Camera c{};
        tpd_look_at(eye, center, up, c.view);
        tpd_perspective(width, height, fovYDegrees, nearPlane, farPlane, c.projection);
        c.width = width;
        c.height = height;
        return c;
    }
};

class GaussianEngine;

class TransformHost {
public:
    explicit TransformHost(tpd_engine* e) : e_(e) {}
    /* Model matrix (row-major) of an entity: moves the means of its points. */
    void transform(uint32_t entity, const float model[16]) const {
        check(tpd_set_transform(e_, entity, model), e_, "tpd_set_transform");
    }

private:
    tpd_engine* e_;
};

class GaussianEngine {
public:
    struct Settings {
        uint32_t sphericalHarmonicsDegree{3};
        bool band3Compat{true};   // SH band-3 term as splat/common.slang:69 writes it
        int device{0};
        void* stream{nullptr};    // cudaStream_t; nullptr: the engine makes its own
        [[nodiscard]] static constexpr Settings getDefault() { return {}; }
    };

    explicit GaussianEngine(const Settings& settings = Settings::getDefault()) { create(settings); }
    ~GaussianEngine() { tpd_destroy(e_); }
    GaussianEngine(const GaussianEngine&) = delete;
    GaussianEngine& operator=(const GaussianEngine&) = delete;

    /* Uploads the points (host memory; free them afterwards). entityIndex:
     * one entry per point, < entities; empty = all entity 0. */
    void compile(const std::vector<GaussianPoint>& points, const Settings& settings = Settings::getDefault(),
                 const std::vector<uint32_t>& entityIndex = {}, uint32_t entities = 1) {
        if (settings.sphericalHarmonicsDegree != settings_.sphericalHarmonicsDegree ||
            settings.band3Compat != settings_.band3Compat) {
            tpd_destroy(e_);
            Settings s = settings;
            s.device = settings_.device;
            s.stream = settings_.stream;
            create(s);
        }
        if (!entityIndex.empty() && entityIndex.size() != points.size())
            throw Error(TPD_ERR_ARG, "entityIndex must have one entry per point");
        check(tpd_compile(e_, points.data(), uint32_t(points.size()), entityIndex.empty() ? nullptr : entityIndex.data(),
                          entities),
              e_, "tpd_compile");
    }

    [[nodiscard]] const std::unique_ptr<TransformHost>& getTransformHost() const noexcept { return transforms_; }

    /* Renders one frame; returns when it is done, like rasterFrame. */
    tpd_frame_stats rasterFrame(const Camera& camera) {
        check(tpd_set_camera(e_, camera.view, camera.projection, camera.width, camera.height), e_, "tpd_set_camera");
        tpd_frame_stats st{};
        check(tpd_raster_frame(e_, &st), e_, "tpd_raster_frame");
        width_ = camera.width;
        height_ = camera.height;
        return st;
    }

    /* Pipelined rendering: renders `camera` and copies the RGBA8 image into
     * dst (pinned host memory, width * height * 4 bytes) without waiting; at
     * most two renders may be outstanding. waitRender() waits for the oldest
     * and returns its stats; dst must stay untouched until then. */
    void renderAsync(const Camera& camera, uint8_t* dst) {
        check(tpd_set_camera(e_, camera.view, camera.projection, camera.width, camera.height), e_, "tpd_set_camera");
        check(tpd_render_async(e_, dst, TPD_IMAGE_RGBA8, 0), e_, "tpd_render_async");
    }

    tpd_frame_stats waitRender() {
        tpd_frame_stats st{};
        check(tpd_wait_render(e_, &st), e_, "tpd_wait_render");
        return st;
    }

    /* The draw() step without a swapchain: the last frame as RGBA8 (alpha 255). */
    std::vector<uint8_t> readImageRGBA8() const {
        std::vector<uint8_t> out(size_t(width_) * height_ * 4);
        check(tpd_read_image(e_, out.data(), TPD_IMAGE_RGBA8, 0), e_, "tpd_read_image");
        return out;
    }

    /* The last frame as H x W x 3 floats. */
    std::vector<float> readImageRGB() const {
        std::vector<float> out(size_t(width_) * height_ * 3);
        check(tpd_read_image(e_, out.data(), TPD_IMAGE_RGB32F, 0), e_, "tpd_read_image");
        return out;
    }

    tpd_engine* handle() const noexcept { return e_; }

private:
    void create(const Settings& settings) {
        tpd_settings s;
        tpd_settings_init(&s);
        s.sh_degree = settings.sphericalHarmonicsDegree;
        s.band3_compat = settings.band3Compat ? 1u : 0u;
        s.device = settings.device;
        s.stream = settings.stream;
        tpd_engine* e = nullptr;
        check(tpd_create(&s, &e), nullptr, "tpd_create");
        e_ = e;
        settings_ = settings;
        transforms_ = std::make_unique<TransformHost>(e_);
    }

    tpd_engine* e_ = nullptr;
    Settings settings_{};
    std::unique_ptr<TransformHost> transforms_;
    uint32_t width_ = 0, height_ = 0;
};

}  // namespace tpdsplat

#endif  // TPDSPLAT_HPP
