// The FP64 integrand with no device allocation: scratch in a static array.
//
// Who needs it: callers that must not let this library allocate device
// memory. A process that hands nearly all of HBM to the Green tables (the
// 12x12, degree-192 tables alone take about 100 GB) or to a pool allocator
// it manages itself cannot have a library take memory behind its back, and a
// driver whose allocations all go through its own allocator has no way to
// account for memory a library takes with cudaMalloc. Such callers bind their
// tables with cdet_bind_device_table and call cdet_integrand_device_noalloc.
//
// The scratch is one file-scope __device__ array of kNoAllocScratchBytes.
// Every GPU that loads this library holds it until the process exits. In
// host code the array's name is only a host-side stand-in, never a device
// address: the device address comes from cudaGetSymbolAddress, looked up once
// per device (with that device current) by the first call on that device and
// cached for the life of the process. The cache assumes that the device's
// primary context lives as long as the process (no cudaDeviceReset in
// between). The first call should come before any stream capture.
//
// How the array is divided: the batch's own regions (Green matrices, shifted
// diagonals, the subset array a and, where the CDet uses it, dp) come first;
// what is left goes to the per-warp regions of the minors kernel (its
// workspace, where it does not run from shared memory, and the LU-fallback
// scratch), up to the warps the kernel can use. A batch that leaves room for
// fewer than eight warps is refused. Largest batches this allows (they do
// not depend on the GPU): 1,824 configurations of order 10, 928 of order 12,
// 448 of order 13, 224 of order 14 and 32 of order 15; none above order 15
// (cdet_gb300.h has the full table). A batch near its limit runs the minors
// on few warps: smaller batches leave room for more.
//
// Every call shares the array and leaves its contents behind. Nothing in it
// needs to start at zero: each region is written before it is read within a
// call (the per-configuration status output is reset by a memset). Calls
// whose kernels overlap on the GPU (different streams, or different host
// threads on one device without ordering) race on the array; issue them on
// one stream, or order them.
#include "cdet_gb300.h"
#include "cdet_kernels.cuh"

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>

namespace cdet {
int run_fp64_on_scratch(cdet_context* ctx, const double* vertices, const int32_t* orders, int64_t batch,
                        int max_order, double* values, int32_t* status, void* scratch, size_t ws_warps,
                        ScratchRegions regions, cudaStream_t stream);
int context_two_spins(cdet_context* ctx, bool* two_spins);
int fail_with(int code, const char* message);
int context_device(const cdet_context* ctx);
int context_sm_count(const cdet_context* ctx);
}  // namespace cdet

namespace {

constexpr size_t kNoAllocScratchBytes = size_t{64} << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;
constexpr size_t kMinWarps = 8;  // one block of the shared-memory minors kernel

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (== device).
int scratch_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return cdet::fail_with(CDET_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[device]) {
        void* ptr = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (err != cudaSuccess || !ptr) {
            const std::string msg = std::string("cudaGetSymbolAddress(no-allocation scratch): ") +
                                    cudaGetErrorString(err);
            return cdet::fail_with(CDET_ERR_CUDA, msg.c_str());
        }
        g_scratch_address[device] = ptr;
    }
    *out = g_scratch_address[device];
    return CDET_OK;
}

}  // namespace

extern "C" int cdet_integrand_device_noalloc(cdet_context* ctx, const double* vertices,
                                             const int32_t* orders, int64_t batch, int max_order,
                                             double* values, int32_t* status, void* stream) {
    if (!ctx) return cdet::fail_with(CDET_ERR_INVALID, "null context");
    if (max_order < 1 || max_order > cdet::kMaxOrder)
        return cdet::fail_with(CDET_ERR_INVALID, "The replica integrand is defined only for order >= 1 (max 24 here)");
    if (batch < 0) return cdet::fail_with(CDET_ERR_INVALID, "batch must be non-negative");
    if (batch == 0) return CDET_OK;
    if (!vertices || !orders || !values || !status) return cdet::fail_with(CDET_ERR_INVALID, "null buffer");
    bool two_spins = true;
    int rc = cdet::context_two_spins(ctx, &two_spins);
    if (rc != CDET_OK) return rc;
    // only the regions this batch's kernels touch
    cdet::ScratchRegions regions;
    regions.minors_workspace = cdet::minors_use_global_workspace(max_order, two_spins);
    regions.dp_lanes = cdet::fp64_single_order_uses_dp_lanes(max_order);
    const size_t fixed = cdet::scratch_bytes(batch, max_order, 0, regions);
    const size_t per_warp = cdet::scratch_bytes(batch, max_order, 1, regions) - fixed;
    // the warps the minors kernel can use: 32 per SM from the global
    // workspace, one block of at most kMinorsMaxWarps per SM from shared memory
    const size_t sms = static_cast<size_t>(std::max(1, cdet::context_sm_count(ctx)));
    const size_t useful = sms * (regions.minors_workspace ? 32 : cdet::kMinorsMaxWarps);
    const size_t room = fixed < kNoAllocScratchBytes ? (kNoAllocScratchBytes - fixed) / per_warp : 0;
    const size_t ws_warps = std::min(useful, room);
    if (ws_warps < kMinWarps) {
        char msg[320];
        std::snprintf(msg, sizeof(msg),
                      "cdet_integrand_device_noalloc: %lld configurations of order <= %d need %zu bytes of "
                      "scratch, more than its fixed %zu; split the batch",
                      static_cast<long long>(batch), max_order, fixed + kMinWarps * per_warp, kNoAllocScratchBytes);
        return cdet::fail_with(CDET_ERR_INVALID, msg);
    }
    int previous = 0;
    cudaGetDevice(&previous);
    const int device = cdet::context_device(ctx);
    if (previous != device) cudaSetDevice(device);
    void* scratch = nullptr;
    rc = scratch_address(device, &scratch);
    if (rc == CDET_OK)
        rc = cdet::run_fp64_on_scratch(ctx, vertices, orders, batch, max_order, values, status, scratch, ws_warps,
                                       regions, static_cast<cudaStream_t>(stream));
    if (previous != device) cudaSetDevice(previous);
    return rc;
}
