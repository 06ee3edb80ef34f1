// Kernel argument blocks and launchers shared by the C-ABI translation units.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace cdet {

constexpr int kMaxOrder = 24;  // largest order (envelope) any kernel accepts

// Status bits per configuration (the reference throws or counts instead).
constexpr int32_t kStatusNonFinite = 1;    // "Value is not finite" (integrand_replica_randomly_sampled.h:543-545)
constexpr int32_t kStatusFpmFallback = 2;  // whole-matrix LU fallback ran (fast_principle_minors.h:180-186)
constexpr int32_t kStatusBadInput = 4;     // order out of range or a vertex coordinate the decode rejects

// IntegrandRuntimeScalars<double> (integrand_replica_randomly_sampled.h:41-51).
struct Scalars {
    int32_t n1, n2, nu, nv;
    double beta, u, branch_eps, scale, diag_up_shift, diag_down_shift;
    double tol_fpm, fpm_shift, z_eps0, z_safety;
};

// One PiecewiseChebyshevTable<double> resident in HBM.
struct TableDev {
    const double* upper;
    const double* lower;
    const double* upper_corners;
    const double* lower_corners;
};

struct DDPair {
    double hi, lo;
};

// Device scratch of one evaluation: per configuration the Green matrices of
// both table sets and spins, their shifted diagonals, and the subset arrays
// a[mask] and dp[mask] of the CDet recursion laid out lane-interleaved for
// 32-configuration groups.
struct Scratch {
    double* green;      // [batch][2 sets][2 spins][max_order^2]
    double* diag;       // [batch][2][2][max_order]
    double* a_int;      // [groups][2][2^max_order][32]
    double* dp_int;     // [groups][2][2^max_order][32]
    double* ws_global;  // per-warp minors workspace when it does not fit shared memory
    double* lu_scratch; // per-lane LU fallback scratch, [warps][32][max_order^2]
    size_t ws_warps;    // warps the global workspace holds
    int32_t* slot_of;   // [batch] order-sorted slot of each configuration (single-order FP64 CDet)
    int32_t* config_at; // [batch] configuration in each slot
    uint32_t* order_count;  // [64] counting-sort buckets
    double* dd_lanes;   // double-double lane form: a [groups][2][2^max_order][32] and dp of the
                        // masks holding vertex 0 [groups][2][2^(max_order-1)][32], (hi, lo) pairs
};

// Per-warp workspace of the minors recursion (mat2pm), in elements of the
// arithmetic type: the matrix, two Schur-complement lists, the pivots'
// inverses and factors, and the shifted minors of each spin.
struct WsLayout {
    int list;      // elements per Schur-complement list
    size_t a, old_list, new_list, aux, shifted_up, shifted_down, total;
    int arena = 0;  // > 0: the compact form (compact_minors_layout), doubles per spin's arena
};

// ---- compact workspace of the FP64 warp recursion (orders <= 10) ----------
// The shifted minors of an order-n matrix fill [0, 2^n) level by level (level
// l writes [2^(l+1), 2^(l+2)) after its Schur complements), so the level
// lists can share one arena with them: list L_k (2^k matrices of (n-k)^2)
// sits low, at 2^(k+1) (only minors below that are written while it lives),
// or high, ending at the arena's end, alternating so that a level's two lists
// never meet. L_{n-2}, read while the last level writes [2^(n-1), 2^n), is
// high; the last level's 1 x 1 children go straight to the minors.
constexpr int kCompactMaxOrder = 10;
__host__ __device__ inline int compact_list_doubles(int n, int k) { return (1 << k) * (n - k) * (n - k); }
__host__ __device__ inline bool compact_list_high(int n, int k) { return ((n - 2 - k) & 1) == 0; }
__host__ __device__ inline int compact_list_offset(int n, int k, int arena) {
    return compact_list_high(n, k) ? arena - compact_list_doubles(n, k) : (1 << (k + 1));
}
// Doubles an order-n arena needs: the minors, each level's two lists apart,
// each high list above the minors written before it is last read.
__host__ __device__ inline int compact_arena_doubles(int n) {
    int t = 1 << n;
    for (int k = 0; k + 2 < n; ++k) {  // level k holds L_k and L_{k+1}
        const int lo = compact_list_high(n, k) ? k + 1 : k;
        t = max(t, (1 << (lo + 1)) + compact_list_doubles(n, k) + compact_list_doubles(n, k + 1));
    }
    for (int k = 0; k + 1 < n; ++k)
        if (compact_list_high(n, k))
            t = max(t, (k == n - 2 ? (1 << n) : (1 << (k + 1))) + compact_list_doubles(n, k));
    return t;
}

// The compact workspace of a batch of orders up to nmax (<= 10) in shared
// memory: one arena per spin (the spin-up minors at its start, the spin-down
// ones one arena later), after the matrix A when with_a (the double-double
// form widens A into it; the FP64 form reads A from the Green matrices). The
// arena is at least 2^(nmax+1) elements, so that after the minors its
// elements from 2^nmax on hold the recursion arrays of the forms that run the
// CDet on the same warp (old_list: dp, new_list: a of the even masks).
__host__ __device__ inline WsLayout compact_minors_layout(int nmax, bool two_spins, bool with_a = false) {
    WsLayout l{};
    int arena = compact_arena_doubles(nmax);
    if (arena < (2 << nmax)) arena = 2 << nmax;
    arena = (arena + 1) & ~1;
    const size_t base = with_a ? (static_cast<size_t>(nmax) * nmax + 1) & ~static_cast<size_t>(1) : 0;
    l.arena = arena;
    l.list = 0;
    l.a = 0;
    l.aux = 0;
    l.shifted_up = base;
    l.shifted_down = base + static_cast<size_t>(arena);
    l.old_list = base + (static_cast<size_t>(1) << nmax);
    l.new_list = l.old_list + (static_cast<size_t>(1) << (nmax - 1));
    l.total = base + static_cast<size_t>(arena) * (two_spins ? 2 : 1);
    return l;
}

// two_spins = false when both sets evaluate one spin only (up and down tables
// and shifts identical): the spin-down minors then need no space. with_aux =
// false leaves out the pivots' inverses and factors (aux): the FP64 warp
// recursion keeps them in its lists, only the chunked recursion of orders
// 11..14 and the double-double one need the region.
__host__ __device__ inline WsLayout ws_layout(int nmax, bool two_spins = true, bool with_aux = true) {
    WsLayout l;
    size_t list = static_cast<size_t>(nmax) * nmax;
    for (int level = 0; level < nmax - 1; ++level) {
        const size_t ns = static_cast<size_t>(nmax - level - 1);
        const size_t cand = (static_cast<size_t>(1) << (level + 1)) * ns * ns;
        if (cand > list) list = cand;
    }
    l.list = static_cast<int>(list);
    const size_t subsets = static_cast<size_t>(1) << nmax;
    auto even = [](size_t x) { return (x + 1) & ~static_cast<size_t>(1); };
    l.a = 0;
    l.old_list = even(static_cast<size_t>(nmax) * nmax);
    l.new_list = l.old_list + even(list);
    l.aux = l.new_list + even(list);
    l.shifted_up = l.aux + (with_aux ? even(subsets / 2 + 2) : 0);
    l.shifted_down = l.shifted_up + subsets;
    l.total = two_spins ? l.shifted_down + subsets : l.shifted_down;
    return l;
}

constexpr uint32_t kQueueHeadIndex = 48;  // the queue head's uint32 slot in Scratch::order_count

// all-subsets CDet work layouts, the values of the C ABI's CDET_FORM_*
constexpr int kFormAuto = 0, kFormLane = 1, kFormWarp = 2;
constexpr int kAllWarpMaxOrder = 11;  // the warp form holds a and dp of one set in shared memory

// How a single-top batch runs after its Green matrices (the values of the C
// ABI's CDET_INTEGRAND_*): staged (minors kernel, global a array, CDet
// kernel) or the persistent queue kernel (minors and CDet of a configuration
// on one warp or a pair of warps, configurations taken from order-sorted
// slots). Both give the same values bit for bit.
constexpr int kIntegrandAuto = 0, kIntegrandStaged = 1, kIntegrandQueue = 2;
constexpr int kQueueMaxOrder = 10;  // the queue form keeps a configuration's workspace in shared memory
constexpr int kQueueMaxWarps = 12;  // warps per block of the queue kernel (384 threads)
constexpr int kMinorsMaxWarps = 12;  // warps per block (one block per SM) of the shared-memory minors kernel
struct QueueShape {
    int warps_per_sm = 0;  // resident warps per SM (0: as many as the shared memory holds)
    int pair = 0;          // 1: two warps per configuration (one per set)
    int grab = 1;          // slots a warp (pair) takes per queue pop
};

struct Problem {
    Scalars s;
    TableDev up[2], down[2];  // set 0 = twisted (r=2), set 1 = ordinary (r=1)
    int same_spin[2];         // up/down tables and diagonal shifts identical: compute spin up only
    const double* vertices;   // [batch][max_order][4]: tau, x, y, replica in [0,1)
    const int32_t* orders;    // [batch] (single-order mode); ignored for all-subsets
    int64_t batch;
    int max_order;
    int all_subsets;          // 0: one value per configuration; 1: 2^max_order values
    int fused_cdet;           // 1: CDet pair updates as FMAs (split assembly); 0: the reference's
                              // separately rounded multiply, subtract and add
    int all_subsets_form;     // kFormAuto / kFormLane / kFormWarp (CDET_FORM_*, cdet_set_all_subsets_form)
    int sorted;               // set by the launcher: minors and the lane CDet work in order-sorted slots
    int integrand_form;       // kIntegrandStaged or kIntegrandQueue (single-top batches of order <= 10)
    QueueShape queue;         // launch shape of the queue form
    // Green-pair reuse (all-subsets batches of MCMCMC chains): when reuse_mask
    // is set, configuration c's first popcount(reuse_mask[c]) vertices are the
    // vertices of the previous evaluation selected by that mask, in increasing
    // order, and the Green entries (and shifted diagonals) of pairs of them are
    // copied from reuse_green / reuse_diag (the previous evaluation's layout)
    // instead of evaluated: the same values, since an entry depends only on its
    // two vertices (integrand_replica_randomly_sampled.h:57-86, 664-696)
    const double* reuse_green;
    const double* reuse_diag;
    const uint64_t* reuse_mask;
    // INTEGRAND_REAL=double_double with VECTOR_REAL=double
    // (cdet_integrand_evaluator.h:431-465): the Green matrices as in the FP64
    // form, then minors, CDet and the order-1 branch in the reference's
    // DoubleDouble arithmetic (integrand_replica_randomly_sampled.h:486-546)
    int dd_mode;
    int raw_diag;             // the assembly stores the unshifted diagonal Green values in diag
    DDPair dd_shift[2];       // IntegrandRuntimeScalars<DoubleDouble> diagonal_up_shift, diagonal_down_shift
    DDPair dd_threshold;      // ZTRANSFORM_EPSILON0 * ZTRANSFORM_SAFETY_FACTOR in DoubleDouble
    DDPair dd_u, dd_beta;     // DoubleDouble(U), DoubleDouble(beta)
    DDPair dd_tol, dd_fpm_shift;  // DoubleDouble(TOL_FPM), DoubleDouble(FPM_GLOBAL_SHIFT)
    DDPair pref_dd[2][kMaxOrder + 1];   // cdet_order_prefactor<DoubleDouble>, [set][order]
    double pref_ld[2][kMaxOrder + 1];   // cdet_order_prefactor<double> (host long double)
    double* values;
    int32_t* status;
};

// This evaluation's Green matrices and diagonals in caller-owned buffers
// (replacing the scratch's), and the previous evaluation's with the masks of
// retained vertices: Green-pair reuse of the MCMCMC step (Problem::reuse_*).
struct GreenReuse {
    double* green;              // [batch][2][2][max_order^2]
    double* diag;               // [batch][2][2][max_order]
    const double* prev_green;   // the previous evaluation's, same layout
    const double* prev_diag;
    const uint64_t* mask;       // [batch] or null (no reuse this evaluation)
};

#ifdef __CUDACC__
// Index of the i-th lowest set bit of m (i < popcount(m)).
__device__ __forceinline__ int nth_set_bit(uint64_t m, int i) {
    for (int t = 0; t < i; ++t) m &= m - 1;
    return __ffsll(static_cast<long long>(m)) - 1;
}

// Green-pair reuse of entry (i, j) of one table set of configuration c (order
// n): when both vertices were retained from the previous evaluation, copies
// both spins' entries (and the shifted diagonals when i == j) from it and
// returns true. A copy equals a fresh evaluation bit for bit: the same two
// vertices, the same operations.
__device__ __forceinline__ bool copy_reused_pair(const Problem& p, double* green, double* diag, int64_t c, int set,
                                                 int i, int j, int n) {
    if (!p.reuse_mask) return false;
    const uint64_t kept = __ldg(p.reuse_mask + c);
    const int k = __popcll(kept);
    if (i >= k || j >= k) return false;
    const int oi = nth_set_bit(kept, i);
    const int oj = i == j ? oi : nth_set_bit(kept, j);
    const int nmax = p.max_order;
    const int64_t per_set = static_cast<int64_t>(nmax) * nmax;
    const int64_t mslot = (c * 2 + set) * 2;
    green[mslot * per_set + i * n + j] = __ldg(p.reuse_green + mslot * per_set + oi * n + oj);
    green[(mslot + 1) * per_set + i * n + j] = __ldg(p.reuse_green + (mslot + 1) * per_set + oi * n + oj);
    if (i == j) {
        diag[mslot * nmax + i] = __ldg(p.reuse_diag + mslot * nmax + oi);
        diag[(mslot + 1) * nmax + i] = __ldg(p.reuse_diag + (mslot + 1) * nmax + oi);
    }
    return true;
}
#endif

// Optional events bracketing the stages of one evaluation: [0] start,
// [1] assembly prep done (descriptors and sort of the split form; equal to
// [0] for the FP64 form), [2] assembly done, [3] minors done, [4] CDet done.
struct KernelEvents {
    cudaEvent_t marks[5];
};

// Split-precision assembly plan: the sliced coefficient blocks of every table
// the two sets use, grouped in segments (one per table and branch) whose
// blocks are numbered consecutively from segment_base.
struct SplitPlan {
    int segments;
    uint32_t segment_base[9];       // ascending; [segments] = total blocks
    const uint16_t* slices[8];      // bf16 slices of the segment's blocks
    const int32_t* exponents[8];    // binary exponent of each block
    const uint8_t* leads[8];        // first nonzero slice of each K step of each sub-block row
    const uint64_t* level_rows[8];  // per sub-block: rows reaching each accumulator level (a byte per level)
    const uint32_t* key_costs[8];   // per sub-block: the estimated time of one of its tiles (relative clocks)
    int records_per_set[2];         // 1 when up and down share one table, else 2
    int segment_of[2][2][2];        // [set][record][0 upper, 1 lower] -> segment
    int spin_mask[2][2];            // [set][record] -> spins the record writes
    uint32_t nblocks;               // sub-blocks over all segments (the keys of the lookup sort)
    int nrb, nkc;                   // sub-blocks of a coefficient block: row chunks x column chunks of 128
    int ksteps_last;                // K steps of the last column chunk (the others have 8)
};

// Sub-blocks of nu x nv coefficients, K steps of the last column chunk, and
// the slice bytes of `blocks` blocks (each sub-block 128 rows x its K steps).
void split_geometry(int nu, int nv, int* nrb, int* nkc, int* ksteps_last);
size_t split_slices_bytes(int nu, int nv, size_t blocks);
// bytes of the per-K-step leads of `blocks` blocks (one byte per K step of each row chunk)
size_t split_leads_bytes(int nu, int nv, size_t blocks);
// bytes of the per-sub-block level rows of `blocks` blocks (8 per sub-block)
size_t split_level_rows_bytes(int nu, int nv, size_t blocks);
// Slices `blocks` coefficient blocks and estimates each sub-block's tile
// time (key_costs, one uint32 per sub-block, used to balance the assembly's
// per-CTA tile ranges).
cudaError_t launch_slice_table(const double* coeffs, int nu, int nv, size_t blocks, uint16_t* slices,
                               int32_t* exponents, uint8_t* leads, uint64_t* level_rows, uint32_t* key_costs,
                               cudaStream_t stream);
size_t split_scratch_bytes(int64_t batch, int max_order, const SplitPlan& plan);
// Bytes of the split assembly's status region: its error flag (int32 at
// byte 0) and counters (uint64 at byte 8: the accumulator columns its
// tcgen05.mma instructions wrote, each 2 x 128 x 16 flops of issued tensor
// work; at byte 16: coefficient-slice bytes streamed from global memory).
constexpr size_t kSplitStatusBytes = 32;
// Largest CHEB_NU / CHEB_NV the split assembly takes (sub-blocks of 128 x 128).
constexpr int kSplitMaxDegree = 256;
cudaError_t launch_split_assembly(const Problem& p, const Scratch& w, const SplitPlan& plan, void* scratch,
                                  size_t scratch_bytes, int sm_count, int32_t** error_flag_out,
                                  cudaStream_t stream, const KernelEvents* events);

cudaError_t launch_fp64_assembly_only(const Problem& p, const Scratch& scratch, cudaStream_t stream);
size_t minors_workspace_doubles(int max_order);
// Whether the minors kernel keeps its per-warp workspace in global memory
// (orders whose workspace does not fit four warps' worth of shared memory).
bool minors_use_global_workspace(int max_order, bool two_spins);
// Whether the FP64 form's CDet of a single-order batch (not all-subsets)
// keeps dp in the lane-interleaved global array.
bool fp64_single_order_uses_dp_lanes(int max_order);
// Which optional regions a scratch carve holds: the global minors workspace
// and the lane-interleaved dp array of the lane-per-configuration CDet. Both
// default to present; a caller with a fixed budget leaves out what its
// launches do not touch.
struct ScratchRegions {
    bool minors_workspace = true;
    bool dp_lanes = true;
    bool dd_lanes = false;  // the double-double integrand's lane-interleaved a and dp
};
size_t scratch_bytes(int64_t batch, int max_order, size_t ws_warps, ScratchRegions regions = {});
void carve_scratch(void* base, int64_t batch, int max_order, size_t ws_warps, Scratch* out,
                   ScratchRegions regions = {});
// assembly = true launches the FP64 Green-matrix assembly first; false
// expects the Green matrices already in scratch (split-precision assembly).
// One MCMCMC step for a batch of chains (uniform or histogram seed kernel),
// after the all-subset integrand of every chain's envelope.
constexpr int kMcmcmcMaxEnvelope = 24;
struct McmcmcStepArgs {
    int64_t chains;
    int envelope, order_min, order_max;
    int warmup;                     // 1: count the chosen order for the lambda adaptation
    double inv_binom[kMcmcmcMaxEnvelope + 1];
    const double* values;           // [chains][2^envelope] all-subset integrands
    const int32_t* integrand_status;
    const double* vertices;         // [chains][envelope][4]
    double* next_vertices;
    const double* lambdas;          // [chains][envelope + 1]
    uint64_t* mt;                   // [312][chains]
    int32_t* mt_index;              // [chains]
    uint64_t* counts;               // [chains][envelope + 1] warmup block counts
    int32_t* error;                 // [chains]: 0, 1 (integrand not finite), 2 (normalisation), 3 (seed density)
    // per-step outputs at ring row r = *ring_row (0 when ring_row is null):
    // chosen_out[r][chains], norm_out[r][chains], signal_out[r][chains][envelope + 1]
    const int64_t* ring_row;
    uint64_t* chosen_out;           // or null
    uint64_t* retained_out;         // or null: [chains] the chosen mask whose vertices lead next_vertices
                                    // (0 when the chain made no step), read by the next evaluation's
                                    // Green-pair reuse
    double* norm_out;               // or null
    double* signal_out;             // or null
    // histogram seed kernel when tau_bins > 0: row probabilities and their
    // CDFs (tau [bins][bins], space [N1 N2][N1 N2], replica [2][2]) and the
    // conditional generation probabilities scratch [chains][2^envelope]
    int tau_bins, n1, n2;
    const double *tau_prob, *space_prob, *replica_prob;
    const double *tau_cdf, *space_cdf, *replica_cdf;
    double* cprob;
};
cudaError_t launch_mcmcmc_init(int64_t chains, int envelope, const uint64_t* seeds, uint64_t* mt, int32_t* mt_index,
                               double* vertices, cudaStream_t stream);
// Launches the step: for small batches one warp-per-chain kernel; otherwise
// one thread-per-chain kernel, preceded for the histogram seed kernel by the
// warp-per-chain conditional probabilities. *kernels = the kernels launched.
cudaError_t launch_mcmcmc_step(const McmcmcStepArgs& args, cudaStream_t stream, int* kernels);
// Smallest all-subsets batch for which the FP64 CDet runs one lane per
// configuration; smaller batches run one warp per configuration.
int all_subsets_lane_form_min_batch(int sm_count);
// *row = (*row + 1) % rows, after a step (one thread)
cudaError_t launch_mcmcmc_advance_row(int64_t* row, int64_t rows, cudaStream_t stream);

// Order-1 diagonal observable: items[3 * N1 * N2] scratch, out[3] = {twisted -
// 2 ordinary, twisted, ordinary}; tables in kind order (twisted up, twisted
// down, ordinary up, ordinary down).
cudaError_t launch_diagonal_order1(const TableDev* const tables[4], int n1, int n2, int nu, int nv, double beta,
                                   double u, double alpha_up, double alpha_down, double* items, double* out,
                                   cudaStream_t stream);

cudaError_t launch_fp64_integrand(const Problem& p, const Scratch& scratch, int sm_count,
                                  cudaStream_t stream, const KernelEvents* events, bool assembly = true);
// Whether launch_fp64_integrand sorts the batch by order first (three more
// kernels: the lane CDet of a single-order batch, and the queue form).
bool sorts_orders(const Problem& p);
// Whether the batch runs the queue form (p.integrand_form and the orders it supports).
bool uses_queue_form(const Problem& p);
// The double-double integrand after the FP64 assembly (orders <= kDDMaxOrder,
// single-top batches): one persistent kernel over the order-sorted slots
// (the sort already launched), its workspace in shared memory.
constexpr int kDDMaxOrder = 10;
constexpr int kDDMaxWarps = 8;  // warps per block of the double-double minors and warp-form kernels
cudaError_t launch_integrand_dd(const Problem& p, const Scratch& scratch, int sm_count, cudaStream_t stream);
// The post-assembly stages alone (sort, minors, CDet, or the queue kernel),
// on Green matrices already in scratch: what the autotuner times.
cudaError_t launch_post_assembly(const Problem& p, const Scratch& scratch, int sm_count, cudaStream_t stream);
// Grid of the queue form for this problem: warps per block, blocks, shared bytes per block.
void queue_launch_shape(const Problem& p, const Scratch& scratch, int sm_count, int* warps_per_block, int* blocks,
                        size_t* smem);

}  // namespace cdet
