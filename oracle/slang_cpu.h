// slang_cpu.h — the small part of Slang's compute-shader language that the
// reference's Gaussian shaders use, as C++20, so that their own source text
// (translated token by token by oracle/slang_to_cpp.py) runs on the CPU.
//
// TEST INFRASTRUCTURE ONLY: it builds the checker oracle/_ref/libtpdref.so,
// which records golden vectors from the reference's shaders; the product
// never uses it.
//
// Semantics, each chosen to be the shader's as written:
//  - float arithmetic is IEEE single precision, rounded after every
//    operation, no contraction (built with -ffp-contract=off); unsuffixed
//    literals are floats (the translator appends f).
//  - vectors and matrices are row-major; mul(A, B) accumulates
//    sum_k A[i][k] B[k][j] for k = 0, 1, ... left to right, mul(M, v) the same
//    with v as a column; dot adds x, y, z, w products left to right.
//  - normalize(v) = v / sqrt(dot(v, v)) per component; sqrt, exp and ceil are
//    the C library's single-precision functions.
//  - (int) of a float truncates toward zero and saturates (NaN -> 0).
//  - min / max of floats return the non-NaN operand (fmin / fmax); of an
//    unsigned and a signed integer, the signed one is converted first.
//  - a workgroup's invocations are fibers of one host thread that meet at
//    GroupMemoryBarrierWithGroupSync; an invocation that returns leaves the
//    barriers of its workgroup. Workgroups start in the order of their index
//    and run concurrently on the host's cores (see dispatch below).
//  - buffers check every index: an access past the end reads 0 and drops the
//    write (robust buffer access) and is counted in oob_accesses().
#pragma once

#include <ucontext.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>
#include <vector>

namespace slangcpu {

using uint = uint32_t;

// ---------------------------------------------------------------- vectors

struct uint2 {
    uint x, y;
    uint2() = default;
    constexpr uint2(uint a, uint b) : x(a), y(b) {}
    uint& operator[](int i) { return i == 0 ? x : y; }
    uint operator[](int i) const { return i == 0 ? x : y; }
};
struct uint3 {
    uint x, y, z;
    uint3() = default;
    constexpr uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    uint2 xy() const { return uint2(x, y); }
};
inline uint2 operator+(uint2 a, uint2 b) { return uint2(a.x + b.x, a.y + b.y); }

struct float2 {
    float x, y;
    float2() = default;
    constexpr float2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};
struct float3 {
    float x, y, z;
    float3() = default;
    constexpr float3(float a, float b, float c) : x(a), y(b), z(c) {}
    float2 xy() const { return float2(x, y); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct float4 {
    float x, y, z, w;
    float4() = default;
    constexpr float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    constexpr float4(float3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    constexpr float4(float2 v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    float2 xy() const { return float2(x, y); }
    float3 xyz() const { return float3(x, y, z); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
static_assert(sizeof(float3) == 12 && sizeof(float4) == 16, "tight vector layouts, as in the shader structs");

inline float2 to_float(uint2 v) { return float2(float(v.x), float(v.y)); }

inline float2 operator+(float2 a, float2 b) { return float2(a.x + b.x, a.y + b.y); }
inline float2 operator-(float2 a, float2 b) { return float2(a.x - b.x, a.y - b.y); }
inline float2 operator*(float2 a, float2 b) { return float2(a.x * b.x, a.y * b.y); }
inline float2 operator+(float2 a, float s) { return float2(a.x + s, a.y + s); }
inline float2 operator-(float2 a, float s) { return float2(a.x - s, a.y - s); }
inline float2 operator*(float2 a, float s) { return float2(a.x * s, a.y * s); }
inline float2 operator/(float2 a, float s) { return float2(a.x / s, a.y / s); }
inline float2 operator*(float s, float2 a) { return float2(s * a.x, s * a.y); }
inline float2 operator*(float2 a, uint2 b) { return a * to_float(b); }
inline float2 operator*(float s, uint2 b) { return s * to_float(b); }

inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator+(float3 a, float s) { return float3(a.x + s, a.y + s, a.z + s); }
inline float3 operator+(float s, float3 a) { return float3(s + a.x, s + a.y, s + a.z); }
inline float3 operator-(float3 a, float s) { return float3(a.x - s, a.y - s, a.z - s); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
inline float3& operator+=(float3& a, float3 b) { return a = a + b; }
inline float3& operator+=(float3& a, float s) { return a = a + s; }

// ---------------------------------------------------------------- matrices (row-major)

struct float2x2 {
    float2 r[2];
    float2& operator[](int i) { return r[i]; }
    const float2& operator[](int i) const { return r[i]; }
};
struct float3x3 {
    float3 r[3];
    float3x3() = default;
    float3x3(float a, float b, float c, float d, float e, float f, float g, float h, float i)
        : r{float3(a, b, c), float3(d, e, f), float3(g, h, i)} {}
    float3& operator[](int i) { return r[i]; }
    const float3& operator[](int i) const { return r[i]; }
    explicit operator float2x2() const { return float2x2{{float2(r[0].x, r[0].y), float2(r[1].x, r[1].y)}}; }
};
struct float4x4 {
    float4 r[4];
    float4x4() = default;
    float4x4(float4 a, float4 b, float4 c, float4 d) : r{a, b, c, d} {}
    float4& operator[](int i) { return r[i]; }
    const float4& operator[](int i) const { return r[i]; }
    explicit operator float3x3() const {
        return float3x3(r[0].x, r[0].y, r[0].z, r[1].x, r[1].y, r[1].z, r[2].x, r[2].y, r[2].z);
    }
};

inline float3x3 mul(const float3x3& A, const float3x3& B) {
    float3x3 C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
    return C;
}
inline float3 mul(const float3x3& A, float3 v) {
    return float3(A[0].x * v.x + A[0].y * v.y + A[0].z * v.z, A[1].x * v.x + A[1].y * v.y + A[1].z * v.z,
                  A[2].x * v.x + A[2].y * v.y + A[2].z * v.z);
}
inline float4x4 mul(const float4x4& A, const float4x4& B) {
    float4x4 C;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j] + A[i][3] * B[3][j];
    return C;
}
inline float4 mul(const float4x4& A, float4 v) {
    float4 o;
    for (int i = 0; i < 4; ++i) o[i] = A[i].x * v.x + A[i].y * v.y + A[i].z * v.z + A[i].w * v.w;
    return o;
}
inline float3x3 transpose(const float3x3& A) {
    float3x3 T;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[j][i] = A[i][j];
    return T;
}

// ---------------------------------------------------------------- intrinsics

inline float sqrt(float x) { return std::sqrt(x); }
inline float exp(float x) { return std::exp(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float3 max(float3 a, float s) { return float3(max(a.x, s), max(a.y, s), max(a.z, s)); }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline uint min(uint a, int b) { return min(a, uint(b)); }
inline uint max(uint a, int b) { return max(a, uint(b)); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 normalize(float3 v) { return v / sqrt(dot(v, v)); }

// (int) conversion: truncation toward zero, saturated.
inline int to_int(float v) {
    if (!(v == v)) return 0;
    if (v >= 2147483520.0f) return std::numeric_limits<int>::max();
    if (v <= -2147483648.0f) return std::numeric_limits<int>::min();
    return int(v);
}

template <typename To, typename From>
inline To reinterpret(From v) {
    static_assert(sizeof(To) == sizeof(From), "reinterpret keeps the size");
    To t;
    std::memcpy(&t, &v, sizeof(To));
    return t;
}

template <typename T>
inline const T& nonuniform(const T& v) { return v; }

// ---------------------------------------------------------------- resources

inline std::atomic<uint64_t>& oob_counter() {
    static std::atomic<uint64_t> n{0};
    return n;
}
inline uint64_t oob_accesses() { return oob_counter().load(); }

template <typename T>
struct StructuredBuffer {
    T* data = nullptr;
    size_t count = 0;
    void bind(T* p, size_t n) {
        data = p;
        count = n;
    }
    T& operator[](size_t i) const {
        if (i < count) return data[i];
        oob_counter().fetch_add(1);
        thread_local T dummy;
        std::memset(static_cast<void*>(&dummy), 0, sizeof(T));
        return dummy;
    }
};
template <typename T>
using RWStructuredBuffer = StructuredBuffer<T>;

template <typename T>
struct ConstantBuffer : T {};

// A bindless model-matrix handle: four float4 rows.
struct TransformHandle {
    const float* m = nullptr;
    std::array<float4, 4> operator*() const {
        return {float4(m[0], m[1], m[2], m[3]), float4(m[4], m[5], m[6], m[7]), float4(m[8], m[9], m[10], m[11]),
                float4(m[12], m[13], m[14], m[15])};
    }
};

// The render target: width x height float4 texels (the shader stores (C, 1)).
struct WTexture2D {
    uint width = 0, height = 0;
    float4* texels = nullptr;
    void GetDimensions(uint, uint& w, uint& h, uint& mips) const {
        w = width;
        h = height;
        mips = 1;
    }
    void Store(uint2 p, float4 v) const {
        if (p.x < width && p.y < height) texels[size_t(p.y) * width + p.x] = v;
        else oob_counter().fetch_add(1);
    }
};

// ---------------------------------------------------------------- atomics

inline void InterlockedAdd(uint& dst, uint v) { std::atomic_ref<uint>(dst).fetch_add(v); }
inline void InterlockedAdd(uint& dst, uint v, uint& orig) { orig = std::atomic_ref<uint>(dst).fetch_add(v); }
inline void InterlockedExchange(uint& dst, uint v) { std::atomic_ref<uint>(dst).exchange(v); }
inline void InterlockedExchange(uint64_t& dst, uint64_t v) { std::atomic_ref<uint64_t>(dst).exchange(v); }
inline void InterlockedCompareExchange(uint& dst, uint cmp, uint v, uint& orig) {
    uint expected = cmp;
    std::atomic_ref<uint>(dst).compare_exchange_strong(expected, v);
    orig = expected;
}
inline void InterlockedCompareExchange(uint64_t& dst, uint64_t cmp, uint64_t v, uint64_t& orig) {
    uint64_t expected = cmp;
    std::atomic_ref<uint64_t>(dst).compare_exchange_strong(expected, v);
    orig = expected;
}

// ---------------------------------------------------------------- workgroups
//
// A workgroup runs on one host thread: its invocations are fibers (ucontext)
// that the thread switches between, and GroupMemoryBarrierWithGroupSync
// switches out of the calling invocation. The thread resumes every
// unfinished invocation in turn; since invocations give up control only at
// barriers (or by returning), one pass over them brings every live
// invocation to the same barrier, which is a barrier's meaning. Groupshared
// variables are thread_local, so each workgroup has its own.
//
// The workgroups of a dispatch start in the order of their index and run
// concurrently on the host's cores; a workgroup, once started, runs to
// completion, so a decoupled look-back (whose partitions are numbered by an
// atomic counter at the start of each workgroup) always waits on running
// workgroups only.

struct FiberGroup {
    ucontext_t sched{};
    std::vector<ucontext_t> ctx;
    std::vector<std::vector<char>> stacks;
    std::vector<uint8_t> done;
    uint32_t current = 0;
    uint3 gid{0, 0, 0}, wg{1, 1, 1};
    const std::function<void(uint3, uint3, uint3)>* entry = nullptr;
};

inline FiberGroup*& current_group() {
    thread_local FiberGroup* g = nullptr;
    return g;
}

inline void GroupMemoryBarrierWithGroupSync() {
    FiberGroup* g = current_group();
    swapcontext(&g->ctx[g->current], &g->sched);
}

inline void fiber_main() {
    FiberGroup* g = current_group();
    const uint32_t t = g->current;
    const uint3 gtid(t % g->wg.x, (t / g->wg.x) % g->wg.y, t / (g->wg.x * g->wg.y));
    const uint3 dtid(g->gid.x * g->wg.x + gtid.x, g->gid.y * g->wg.y + gtid.y, g->gid.z * g->wg.z + gtid.z);
    (*g->entry)(gtid, g->gid, dtid);
    g->done[t] = 1;  // returning resumes the scheduler (uc_link)
}

// Runs entry(group thread id, group id, dispatch thread id) for every
// invocation of groups.x x groups.y x groups.z workgroups of size wg.
inline void dispatch(uint3 groups, uint3 wg, const std::function<void(uint3, uint3, uint3)>& entry) {
    constexpr size_t kStack = 64 * 1024;
    const uint64_t ngroups = uint64_t(groups.x) * groups.y * groups.z;
    const uint32_t nthreads = wg.x * wg.y * wg.z;
    if (ngroups == 0 || nthreads == 0) return;
    std::atomic<uint64_t> next{0};
    const uint32_t workers = uint32_t(std::min<uint64_t>(ngroups, std::max(1u, std::thread::hardware_concurrency())));
    auto worker = [&] {
        FiberGroup fg;
        fg.ctx.resize(nthreads);
        fg.stacks.assign(nthreads, std::vector<char>(kStack));
        fg.done.assign(nthreads, 0);
        fg.wg = wg;
        fg.entry = &entry;
        current_group() = &fg;
        for (uint64_t g = next.fetch_add(1); g < ngroups; g = next.fetch_add(1)) {
            fg.gid = uint3(uint(g % groups.x), uint((g / groups.x) % groups.y), uint(g / (uint64_t(groups.x) * groups.y)));
            for (uint32_t t = 0; t < nthreads; ++t) {
                getcontext(&fg.ctx[t]);
                fg.ctx[t].uc_stack.ss_sp = fg.stacks[t].data();
                fg.ctx[t].uc_stack.ss_size = kStack;
                fg.ctx[t].uc_link = &fg.sched;
                makecontext(&fg.ctx[t], fiber_main, 0);
                fg.done[t] = 0;
            }
            for (uint32_t live = nthreads; live > 0;) {
                for (uint32_t t = 0; t < nthreads; ++t) {
                    if (fg.done[t]) continue;
                    fg.current = t;
                    swapcontext(&fg.sched, &fg.ctx[t]);
                    if (fg.done[t]) --live;
                }
            }
        }
        current_group() = nullptr;
    };
    std::vector<std::thread> pool;
    for (uint32_t w = 1; w < workers; ++w) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
}

}  // namespace slangcpu
