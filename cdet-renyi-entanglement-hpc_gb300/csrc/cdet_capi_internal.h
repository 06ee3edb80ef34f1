// Host-side state shared by the C ABI's translation units (cdet_capi.cu and
// the MCMCMC runtime, cdet_mcmcmc_host.cu): the context and the helpers the
// runtime calls. Not part of the public interface.
#pragma once

#include "cdet_gb300.h"
#include "cdet_kernels.cuh"

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

namespace capi {

struct TableSlot {
    cdet::TableDev dev{};
    void* owned = nullptr;  // device allocation made by cdet_upload_table
    int alias_of = -1;      // kind this slot shares, or -1
    bool ready = false;
};

// bf16 slices of one branch of one table (split assembly)
struct SlicedBranch {
    void* mem = nullptr;  // slices followed by exponents
    const uint16_t* slices = nullptr;
    const int32_t* exponents = nullptr;
    const uint64_t* level_rows = nullptr;  // rows reaching each accumulator level, per sub-block
    const uint8_t* leads = nullptr;        // first nonzero slice per K step
    const uint32_t* key_costs = nullptr;   // estimated tile time per sub-block
    size_t blocks = 0;
};

}  // namespace capi

struct cdet_context {
    int device = 0;
    int sm_count = 0;
    cdet_runtime_scalars scalars{};
    size_t coeff_count = 0, corner_count = 0;
    capi::TableSlot tables[4];
    // scratch
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    int64_t scratch_batch = 0;
    int scratch_order = 0;
    size_t ws_warps = 0;
    bool scratch_dd = false;  // the scratch holds the double-double lane region
    // staging for the host-buffer entry points
    void* staging = nullptr;
    size_t staging_bytes = 0;
    uint64_t calls = 0, fallbacks = 0;
    int last_launches = 0;
    // split assembly
    int assembly = CDET_ASSEMBLY_FP64;
    int all_subsets_form = CDET_FORM_AUTO;
    // all-subsets CDet form measured fastest, per (order, fused, floor(log2 batch))
    std::map<std::tuple<int, int, int>, int> form_tuned;
    // single-top post-assembly form: fixed (cdet_set_integrand_form) or measured
    // per (order, fused, floor(log2 batch)) under CDET_INTEGRAND_AUTO
    int integrand_form = CDET_INTEGRAND_AUTO;
    cdet::QueueShape queue_shape{};
    std::map<std::tuple<int, int, int>, std::pair<int, cdet::QueueShape>> integrand_tuned;
    // INTEGRAND_REAL (CDET_INTEGRAND_REAL_*) and the double-double mode's scalars
    int integrand_real = CDET_INTEGRAND_REAL_DOUBLE;
    cdet::DDPair dd_shift[2]{}, dd_threshold{}, dd_u{}, dd_beta{}, dd_tol{}, dd_fpm_shift{};
    std::map<std::pair<const double*, size_t>, capi::SlicedBranch> sliced;  // (coeffs, blocks) -> slices
    void* split_scratch = nullptr;
    size_t split_scratch_bytes = 0;
    int32_t* split_error = nullptr;  // device flag of the last split evaluation
    // measurement hooks
    bool profiling = false;
    std::vector<cdet::KernelEvents> pending;  // recorded, not yet read
    std::vector<cdet::KernelEvents> spare;    // read, reusable
    int64_t pending_launches = 0;
    // bumped whenever a device buffer that launches capture changes (scratch,
    // split scratch, tables, slices): CUDA graphs of older launches are stale
    uint64_t generation = 0;
};

namespace capi {

class DeviceGuard {
public:
    explicit DeviceGuard(int device) {
        cudaGetDevice(&previous_);
        if (previous_ != device) cudaSetDevice(device);
        device_ = device;
    }
    ~DeviceGuard() {
        if (previous_ != device_) cudaSetDevice(previous_);
    }

private:
    int previous_ = 0, device_ = 0;
};

// Records the message for cdet_last_error and returns the code.
int fail(int code, const std::string& message);
int cuda_fail(cudaError_t err, const char* what);

// The table a kind resolves to (following aliases), or null before upload.
const cdet::TableDev* resolve(const cdet_context* ctx, int kind);

// Launches one evaluation of the context's assembly on `stream` (device
// buffers; all_subsets = 1: the 2^max_order subset values of each envelope).
// Asynchronous once the context's scratch holds the batch. With `reuse` the
// Green matrices go to the caller's buffers and pairs of retained vertices are
// copied from the previous evaluation's (the MCMCMC step).
int run(cdet_context* ctx, const double* vertices, const int32_t* orders, int64_t batch, int max_order,
        int all_subsets, double* values, int32_t* status, cudaStream_t stream, bool assembly_only = false,
        const cdet::GreenReuse* reuse = nullptr);

}  // namespace capi
