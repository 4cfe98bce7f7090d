// scan_static.cu — tpd_scan_tiles_static: the tile-count scan of
// tpd_scan_tiles with its scratch (control block + look-back descriptors) in
// a fixed array in this library's device memory, so a call allocates nothing
// and needs no workspace from the caller.
//
// Who needs it: a host that cannot hand out device memory at the point where
// it scans — a renderer whose device memory is all held by its own arena or
// by another framework's caching allocator, or a per-frame loop that must not
// call cudaMalloc/cudaFree because either can wait for the whole device to go
// idle and so stalls every stream in flight.
//
// Limits, in the caller's terms:
//  - n <= TPD_SCAN_STATIC_MAX_SPLATS; larger n is rejected with
//    TPD_ERR_CAPACITY before anything is enqueued.
//  - The first call on each device (with that device current) looks up the
//    scratch's address; that lookup can load this library's device code, so
//    make the first call before any stream capture begins.
//  - There is one scratch per device. Two calls on one device whose work
//    overlaps (different streams without ordering, or different threads)
//    share it and race; order them on one stream.
//  - Nothing has to start at zero: every call clears the descriptors and the
//    control block's counters on the stream before the scan runs.
//  - The address is looked up in the device's primary context (the one the
//    runtime uses by default) and kept for the life of the process: calls
//    from another driver context, or after cudaDeviceReset, are not
//    supported.
//  - A look-back wait that runs out leaves wrong offsets; the status output
//    reports it (TPD_DEVSTAT_LOOKBACK_TIMEOUT).
#include <cstdint>
#include <mutex>

#include "../../include/tpdsplat.h"
#include "tpd_common.cuh"
#include "tpd_kernels.h"

using namespace tpd;

namespace {

constexpr uint32_t kStaticScanTile = 1024;  // splats per look-back partition of the scan kernel
constexpr size_t kCtlBytes = 256 * ((sizeof(FrameCtl) + 255) / 256);
constexpr size_t kDescEntries = size_t(TPD_SCAN_STATIC_MAX_SPLATS) / kStaticScanTile + 2;
constexpr size_t kScratchBytes = kCtlBytes + kDescEntries * sizeof(uint64_t);
constexpr uint32_t kStaticSpin = 1u << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scan_scratch[kScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Address of this device's scratch; looked up once per device.
int scratch_for_current_device(unsigned char** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return TPD_ERR_DEVICE;
    if (dev < 0 || dev >= kMaxDevices) return TPD_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scan_scratch) != cudaSuccess || !p) return TPD_ERR_DEVICE;
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return TPD_OK;
}

}  // namespace

extern "C" {

int tpd_scan_tiles_static(const void* splats, uint32_t n, uint32_t* offsets, uint32_t* total, uint32_t* status,
                          void* stream) {
    if (!total) return TPD_ERR_ARG;
    if (n > 0 && (!splats || !offsets)) return TPD_ERR_ARG;
    if (n > TPD_SCAN_STATIC_MAX_SPLATS) return TPD_ERR_CAPACITY;
    unsigned char* scratch = nullptr;
    const int rc = scratch_for_current_device(&scratch);
    if (rc != TPD_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    FrameCtl* ctl = reinterpret_cast<FrameCtl*>(scratch);
    uint64_t* desc = reinterpret_cast<uint64_t*>(scratch + kCtlBytes);
    const size_t entries = size_t(n) / kStaticScanTile + 2;
    if (cudaMemsetAsync(desc, 0, entries * sizeof(uint64_t), s) != cudaSuccess) return TPD_ERR_DEVICE;
    launch_sort_begin(ctl, 0, s);
    launch_scan_tiles(static_cast<const Splat*>(splats), n, offsets, desc, ctl, kStaticSpin,
                      test_never_publish_standalone(), s);
    if (cudaMemcpyAsync(total, &ctl->total_keys, 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return TPD_ERR_DEVICE;
    if (status && cudaMemcpyAsync(status, &ctl->status, 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return TPD_ERR_DEVICE;
    return cudaGetLastError() == cudaSuccess ? TPD_OK : TPD_ERR_DEVICE;
}

}  // extern "C"
