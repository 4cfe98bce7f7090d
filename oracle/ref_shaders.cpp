// ref_shaders.cpp — runs the reference's own compute shaders on the CPU:
// their Slang source, translated token by token into C++ by
// oracle/slang_to_cpp.py (generated into oracle/_ref/gen/), executed with the
// workgroup model of oracle/slang_cpu.h, dispatched in the order and with
// the sizes that GaussianEngine::rasterFrame records them
// (volumetric/src/GaussianEngine.cpp:621-712, recordSplat :777-791,
// recordBlend :806-863, pass count updateRadixPassCount :351-357):
//   project    ceil(N/256) workgroups of SUBGROUP_SIZE (32) invocations
//   prefix     ceil(N/256) x 128
//   keygen     ceil(N/256) x 256
//   per radix pass p < (getHigherMSB(tiles) + 33) / 2 with blocks = ceil(K/256):
//     radix-shuffle blocks x 128, radix-prefixA and -prefixB
//     ceil(blocks/256) x 128 each, radix-mapping blocks x 256
//   ranges zero-filled, range blocks x 256
//   blend      tilesX x tilesY workgroups of 16 x 16
//
// TEST INFRASTRUCTURE ONLY: built into oracle/_ref/libtpdref.so (git-ignored)
// where the reference tree is present, and used by tests/golden/make_golden.py
// to record golden vectors of the reference's own shader maths.
#include <cstdint>
#include <cstring>
#include <vector>

#include "slang_cpu.h"

namespace slangcpu {
namespace sh_project {
#include "project.inc"
}
namespace sh_prefix {
#include "prefix.inc"
}
namespace sh_keygen {
#include "keygen.inc"
}
namespace sh_shuffle {
#include "radix_shuffle.inc"
}
namespace sh_prefix_a {
#include "radix_prefixA.inc"
}
namespace sh_prefix_b {
#include "radix_prefixB.inc"
}
namespace sh_mapping {
#include "radix_mapping.inc"
}
namespace sh_range {
#include "range.inc"
}
namespace sh_blend {
#include "blend.inc"
}
}  // namespace slangcpu

using namespace slangcpu;

namespace {

constexpr uint32_t kWorkgroup = 256;  // WORKGROUP_SIZE (splat.slang:7)
constexpr uint32_t kBlock = 16;       // BLOCK_X = BLOCK_Y

// getHigherMSB (GaussianEngine.h:234-245) is the engine's, built from the
// reference header by oracle/build_ref.py (gen_higher_msb.cpp).
}  // namespace
uint32_t ref_higher_msb_impl(uint32_t n);

struct RefFrame {
    uint32_t n = 0, width = 0, height = 0;
    std::vector<sh_project::Splat> splats_projected;  // after project
    std::vector<uint32_t> offsets;                      // Splat.tiles after prefix (exclusive scan)
    std::vector<uint64_t> keys;
    std::vector<uint32_t> vals;
    std::vector<uint32_t> ranges;  // tiles x 2
    std::vector<float4> image;
    uint64_t K = 0;
    uint64_t oob = 0;
    uint32_t passes = 0;
};

extern "C" {

// Renders one frame of n 240-byte records through the reference shaders.
// transforms: n_ent row-major model matrices (NULL: one identity);
// transform_index: per record (NULL: all 0). Returns a frame handle.
RefFrame* ref_frame_run(const float* records, uint32_t n, const uint32_t* transform_index, const float* transforms,
                        uint32_t n_ent, const float view[16], const float projview[16], const float focal[2],
                        uint32_t width, uint32_t height, uint32_t sh_degree) {
    auto* f = new RefFrame();
    f->n = n;
    f->width = width;
    f->height = height;
    const uint64_t oob0 = oob_accesses();

    // ---- resources shared across passes (the engine's buffers)
    std::vector<sh_project::Gaussian> gaussians(n);
    static_assert(sizeof(sh_project::Gaussian) == 240 && sizeof(sh_project::Splat) == 48, "reference layouts");
    if (n) std::memcpy(gaussians.data(), records, size_t(n) * 240);
    std::vector<sh_project::Splat> splats(n);
    std::vector<float> identity = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    const float* mats = transforms ? transforms : identity.data();
    const uint32_t ents = transforms ? (n_ent ? n_ent : 1) : 1;
    std::vector<TransformHandle> handles(ents);
    for (uint32_t e = 0; e < ents; ++e) handles[e].m = mats + size_t(e) * 16;
    std::vector<uint32_t> tindex(n, 0u);
    if (transform_index && n) std::memcpy(tindex.data(), transform_index, size_t(n) * 4);
    std::vector<float4> texels(size_t(width) * height, float4(0.f, 0.f, 0.f, 0.f));
    sh_project::Camera cam{};
    for (int r = 0; r < 4; ++r) {
        cam.viewMatrix[r] = float4(view[4 * r], view[4 * r + 1], view[4 * r + 2], view[4 * r + 3]);
        cam.projMatrix[r] = float4(projview[4 * r], projview[4 * r + 1], projview[4 * r + 2], projview[4 * r + 3]);
    }
    cam.focalNDC = float2(focal[0], focal[1]);
    auto bind_image = [&](WTexture2D& img) {
        img.width = width;
        img.height = height;
        img.texels = texels.data();
    };
    const uint32_t wgs = (n + kWorkgroup - 1) / kWorkgroup;

    // ---- project (recordSplat)
    {
        namespace S = sh_project;
        S::info = S::RasterInfo{n, sh_degree, 0, 0};
        bind_image(S::outputImage);
        static_cast<S::Camera&>(S::camera) = cam;
        S::gaussians.bind(gaussians.data(), n);
        S::splats.bind(splats.data(), n);
        S::transforms.bind(handles.data(), handles.size());
        S::transformIndices.bind(tindex.data(), n);
        dispatch(uint3(wgs, 1, 1), S::numthreads(), S::entry);
    }
    f->splats_projected = splats;

    // ---- prefix: in-place exclusive scan of Splat.tiles, total to tilesRendered
    std::vector<uint32_t> tiles_rendered(1, 0u), partition_count(1, 0u), partition_desc(wgs + 1, 0u);
    {
        namespace S = sh_prefix;
        S::info = S::RasterInfo{n, sh_degree, 0, 0};
        S::splats.bind(reinterpret_cast<S::Splat*>(splats.data()), n);
        S::tilesRendered.bind(tiles_rendered.data(), 1);
        S::partitionCount.bind(partition_count.data(), 1);
        S::partitionDescriptors.bind(partition_desc.data(), partition_desc.size());
        dispatch(uint3(wgs, 1, 1), S::numthreads(), S::entry);
    }
    f->offsets.resize(n);
    for (uint32_t i = 0; i < n; ++i) f->offsets[i] = splats[i].tiles;
    const uint32_t K = n ? tiles_rendered[0] : 0u;
    f->K = K;

    // ---- keygen
    std::vector<uint64_t> keys(K), temp_keys(K);
    std::vector<uint32_t> vals(K), temp_vals(K);
    const uint32_t blocks = (K + kWorkgroup - 1) / kWorkgroup;
    if (n) {
        namespace S = sh_keygen;
        S::info = S::RasterInfo{n, sh_degree, K, 0};
        bind_image(S::outputImage);
        S::splats.bind(reinterpret_cast<S::Splat*>(splats.data()), n);
        S::splatKeys.bind(keys.data(), K);
        S::splatIndices.bind(vals.data(), K);
        dispatch(uint3(wgs, 1, 1), S::numthreads(), S::entry);
    }

    // ---- radix passes (updateRadixPassCount: (getHigherMSB(tiles) + 32 + 1) / 2)
    const uint32_t tiles_x = (width + kBlock - 1) / kBlock, tiles_y = (height + kBlock - 1) / kBlock;
    const uint32_t passes = (ref_higher_msb_impl(tiles_x * tiles_y) + 32 + 1) / 2;
    f->passes = passes;
    std::vector<uint64_t> prefix_a(blocks + 1, 0ull), prefix_b(blocks + 1, 0ull);
    const uint32_t scan_wgs = (blocks + kWorkgroup - 1) / kWorkgroup;
    std::vector<uint32_t> count_a(1, 0u), count_b(1, 0u), global_sums(3, 0u);
    std::vector<uint64_t> desc_a(scan_wgs + 1, 0ull), desc_b(scan_wgs + 1, 0ull);
    for (uint32_t p = 0; p < passes && K > 0; ++p) {
        {
            namespace S = sh_shuffle;
            S::info = S::RasterInfo{n, sh_degree, K, p};
            S::splatKeys.bind(keys.data(), K);
            S::splatIndices.bind(vals.data(), K);
            S::globalPrefixA.bind(prefix_a.data(), blocks);
            S::globalPrefixB.bind(prefix_b.data(), blocks);
            S::tempKeys.bind(temp_keys.data(), K);
            S::tempVals.bind(temp_vals.data(), K);
            dispatch(uint3(blocks, 1, 1), S::numthreads(), S::entry);
        }
        {
            namespace S = sh_prefix_a;
            S::info = S::RasterInfo{n, sh_degree, K, p};
            S::globalPrefixes.bind(prefix_a.data(), blocks);
            S::blockCount.bind(count_a.data(), 1);
            S::blockDescriptors.bind(desc_a.data(), desc_a.size());
            S::globalSums.bind(global_sums.data(), 3);
            dispatch(uint3(scan_wgs, 1, 1), S::numthreads(), S::entry);
        }
        {
            namespace S = sh_prefix_b;
            S::info = S::RasterInfo{n, sh_degree, K, p};
            S::globalPrefixes.bind(prefix_b.data(), blocks);
            S::blockCount.bind(count_b.data(), 1);
            S::blockDescriptors.bind(desc_b.data(), desc_b.size());
            S::globalSums.bind(global_sums.data(), 3);
            dispatch(uint3(scan_wgs, 1, 1), S::numthreads(), S::entry);
        }
        {
            namespace S = sh_mapping;
            S::info = S::RasterInfo{n, sh_degree, K, p};
            S::splatKeys.bind(keys.data(), K);
            S::splatIndices.bind(vals.data(), K);
            S::globalPrefixA.bind(prefix_a.data(), blocks);
            S::globalPrefixB.bind(prefix_b.data(), blocks);
            S::tempKeys.bind(temp_keys.data(), K);
            S::tempVals.bind(temp_vals.data(), K);
            S::globalSums.bind(global_sums.data(), 3);
            dispatch(uint3(blocks, 1, 1), S::numthreads(), S::entry);
        }
    }

    // ---- ranges (fillBuffer 0, then range.slang)
    std::vector<uint2> ranges(size_t(tiles_x) * tiles_y, uint2(0u, 0u));
    {
        namespace S = sh_range;
        S::info = S::RasterInfo{n, sh_degree, K, 0};
        S::splatKeys.bind(keys.data(), K);
        S::ranges.bind(ranges.data(), ranges.size());
        dispatch(uint3(blocks, 1, 1), S::numthreads(), S::entry);
    }

    // ---- blend
    {
        namespace S = sh_blend;
        bind_image(S::outputImage);
        S::splats.bind(reinterpret_cast<S::Splat*>(splats.data()), n);
        S::splatIndices.bind(vals.data(), K);
        S::ranges.bind(ranges.data(), ranges.size());
        dispatch(uint3(tiles_x, tiles_y, 1), S::numthreads(), S::entry);
    }

    f->keys = std::move(keys);
    f->vals = std::move(vals);
    f->ranges.resize(ranges.size() * 2);
    for (size_t t = 0; t < ranges.size(); ++t) {
        f->ranges[2 * t] = ranges[t].x;
        f->ranges[2 * t + 1] = ranges[t].y;
    }
    f->image = std::move(texels);
    f->oob = oob_accesses() - oob0;
    return f;
}

uint64_t ref_frame_keys(const RefFrame* f) { return f->K; }
uint64_t ref_frame_oob(const RefFrame* f) { return f->oob; }
uint32_t ref_frame_passes(const RefFrame* f) { return f->passes; }

// Copies the frame's results: splats (n x 12 words, after project), offsets
// (n, after prefix), keys / vals (K, sorted), ranges (tiles x 2), image
// (height x width x 4 floats, what blend stored). Any pointer may be NULL.
void ref_frame_copy(const RefFrame* f, uint32_t* splats, uint32_t* offsets, uint64_t* keys, uint32_t* vals,
                    uint32_t* ranges, float* image) {
    if (splats && f->n) std::memcpy(splats, f->splats_projected.data(), size_t(f->n) * 48);
    if (offsets && f->n) std::memcpy(offsets, f->offsets.data(), size_t(f->n) * 4);
    if (keys && f->K) std::memcpy(keys, f->keys.data(), f->K * 8);
    if (vals && f->K) std::memcpy(vals, f->vals.data(), f->K * 4);
    if (ranges && !f->ranges.empty()) std::memcpy(ranges, f->ranges.data(), f->ranges.size() * 4);
    if (image && !f->image.empty()) std::memcpy(image, f->image.data(), f->image.size() * 16);
}

void ref_frame_free(RefFrame* f) { delete f; }

}  // extern "C"
