// Renders the seeded 10,000-Gaussian scene at 256x256 through the C++ wrapper
// (include/tpdsplat.hpp) and writes the RGB32F image to argv[1]. Used by
// tests/test_cpp_wrapper.py, which compares it with the Python binding's frame.
#include <cstdio>
#include <vector>

#include "tpdsplat.hpp"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s out.f32\n", argv[0]);
        return 2;
    }
    try {
        const uint32_t n = 10000;
        std::vector<tpdsplat::GaussianPoint> points(n);
        tpd_synthetic_scene(0, n, 0.0f, nullptr, nullptr, nullptr, nullptr, nullptr, points.data());
        tpdsplat::GaussianEngine engine;
        engine.compile(points);  // the caller's points may be freed from here on
        const float eye[3] = {0.0f, 0.0f, -5.0f}, center[3] = {0.0f, 0.0f, 0.0f}, up[3] = {0.0f, -1.0f, 0.0f};
        const auto camera = tpdsplat::Camera::lookAt(eye, center, up, 256, 256);
        const float identity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        engine.getTransformHost()->transform(0, identity);
        const tpd_frame_stats st = engine.rasterFrame(camera);
        const std::vector<float> rgb = engine.readImageRGB();
        // the same frame through the pipelined calls must give the same RGBA8 image
        const std::vector<uint8_t> rgba = engine.readImageRGBA8();
        std::vector<uint8_t> piped(rgba.size());
        engine.renderAsync(camera, piped.data());
        engine.waitRender();
        if (piped != rgba) {
            std::fprintf(stderr, "pipelined frame differs\n");
            return 4;
        }
        FILE* f = std::fopen(argv[1], "wb");
        if (!f || std::fwrite(rgb.data(), sizeof(float), rgb.size(), f) != rgb.size()) return 3;
        std::fclose(f);
        std::printf("keys %llu visible %u\n", static_cast<unsigned long long>(st.keys), st.visible);
    } catch (const tpdsplat::Error& e) {
        std::fprintf(stderr, "tpdsplat error %d: %s\n", e.code(), e.what());
        return 1;
    }
    return 0;
}
