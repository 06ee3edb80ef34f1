// C ABI of the GB300 CDet integrand (declared in include/cdet_gb300.h).
//
// Host side: context and table bookkeeping, the order prefactors (computed on
// the host exactly as the reference does), device scratch, and the launch of
// the FP64 kernels in cdet_kernels.cu. The host compiler runs with
// -ffp-contract=off so the double-double prefactor arithmetic below rounds
// every operation separately, as the reference's DoubleDouble does.
#include "cdet_capi_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <utility>
#include <vector>

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace capi {

int fail(int code, const std::string& message) {
    g_last_error = message;
    return code;
}

int cuda_fail(cudaError_t err, const char* what) {
    return fail(CDET_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

}  // namespace capi

using capi::cuda_fail;
using capi::DeviceGuard;
using capi::fail;
using capi::SlicedBranch;
using capi::TableSlot;

namespace {


// DoubleDouble (utility/types.h:30-182), host side.
struct HostDD {
    double hi, lo;
};
double h_two_sum(double a, double b, double& e) {
    const double s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
    return s;
}
double h_quick_two_sum(double a, double b, double& e) {
    const double s = a + b;
    e = b - (s - a);
    return s;
}
HostDD h_add(HostDD x, HostDD y) {
    double s2, t2;
    double s1 = h_two_sum(x.hi, y.hi, s2);
    const double t1 = h_two_sum(x.lo, y.lo, t2);
    s2 += t1;
    s1 = h_quick_two_sum(s1, s2, s2);
    s2 += t2;
    HostDD r;
    r.hi = h_quick_two_sum(s1, s2, r.lo);
    return r;
}
HostDD h_mul(HostDD x, HostDD y) {
    const double p = x.hi * y.hi;
    double e = std::fma(x.hi, y.hi, -p);
    e += x.hi * y.lo + x.lo * y.hi + x.lo * y.lo;
    HostDD r;
    r.hi = h_quick_two_sum(p, e, r.lo);
    return r;
}
HostDD h_div(HostDD x, HostDD y) {
    const double q1 = x.hi / y.hi;
    const HostDD prod = h_mul(HostDD{q1, 0.0}, y);
    const HostDD r = h_add(x, HostDD{-prod.hi, -prod.lo});
    const double q2 = (r.hi + r.lo) / y.hi;
    HostDD q = h_add(HostDD{q1, 0.0}, HostDD{q2, 0.0});
    const double s = q.hi + q.lo;
    q.lo = q.lo - (s - q.hi);
    q.hi = s;
    return q;
}

// cdet_order_prefactor<DoubleDouble> (integrand_replica_randomly_sampled.h:155-159):
// (-r)^n / (n! N1 N2); (-r)^n is exact for r in {1, 2}.
HostDD prefactor_dd(int order, int n1, int n2, int r) {
    double power = 1.0;
    for (int i = 0; i < order; ++i) power *= -static_cast<double>(r);
    HostDD factorial{1.0, 0.0};
    for (int i = 1; i <= order; ++i) factorial = h_mul(factorial, HostDD{static_cast<double>(i), 0.0});
    const HostDD den = h_mul(h_mul(factorial, HostDD{static_cast<double>(n1), 0.0}),
                             HostDD{static_cast<double>(n2), 0.0});
    return h_div(HostDD{power, 0.0}, den);
}

// cdet_order_prefactor<double> (:160-170), in the host's long double.
double prefactor_ld(int order, int n1, int n2, int r) {
    long double num = 1.0L;
    for (int i = 0; i < order; ++i) num *= -static_cast<long double>(r);
    long double den = static_cast<long double>(n1) * static_cast<long double>(n2);
    for (int i = 2; i <= order; ++i) den *= static_cast<long double>(i);
    return static_cast<double>(num / den);
}

}  // namespace


namespace {

const cdet::TableDev* resolve(const cdet_context* ctx, int kind) {
    const TableSlot& slot = ctx->tables[kind];
    if (slot.alias_of >= 0) return resolve(ctx, slot.alias_of);
    return slot.ready ? &slot.dev : nullptr;
}

bool valid_kind(int kind) { return kind >= 0 && kind < 4; }

size_t expected_coeffs(const cdet_runtime_scalars& s) {
    const size_t sites = static_cast<size_t>(s.n1) * s.n2;
    return 4 * sites * sites * static_cast<size_t>(s.cheb_nu) * s.cheb_nv;
}
size_t expected_corners(const cdet_runtime_scalars& s) {
    const size_t sites = static_cast<size_t>(s.n1) * s.n2;
    return 4 * sites * sites;
}

void release_slot(TableSlot& slot) {
    if (slot.owned) cudaFree(slot.owned);
    slot = TableSlot{};
}

// Drops the cached split slices of a slot's coefficients before the slot is
// replaced: a new table may be allocated at the same device address.
void forget_slices(cdet_context* ctx, const TableSlot& slot) {
    ++ctx->generation;  // the slot is about to be replaced
    if (!slot.ready) return;
    for (auto it = ctx->sliced.begin(); it != ctx->sliced.end();) {
        if (it->first.first == slot.dev.upper || it->first.first == slot.dev.lower) {
            cudaFree(it->second.mem);
            it = ctx->sliced.erase(it);
        } else {
            ++it;
        }
    }
}

// The optional regions the context's scratch holds.
cdet::ScratchRegions scratch_regions(const cdet_context* ctx) {
    cdet::ScratchRegions r;
    r.dd_lanes = ctx->scratch_dd;
    return r;
}

int ensure_scratch(cdet_context* ctx, int64_t batch, int max_order) {
    const bool dd = ctx->integrand_real == CDET_INTEGRAND_REAL_DOUBLE_DOUBLE;
    if (ctx->scratch && batch <= ctx->scratch_batch && max_order <= ctx->scratch_order && (!dd || ctx->scratch_dd))
        return CDET_OK;
    const int64_t new_batch = batch > ctx->scratch_batch ? batch : ctx->scratch_batch;
    const int new_order = max_order > ctx->scratch_order ? max_order : ctx->scratch_order;
    // minors warps with a global workspace (orders whose workspace does not
    // fit shared memory): up to 32 per SM, as many as 4 GiB of workspace holds
    // (at least eight, the largest block of the minors kernel, which runs
    // no more warps than the workspace has)
    const size_t per_warp = (cdet::minors_workspace_doubles(new_order) +
                             static_cast<size_t>(32) * new_order * new_order) * sizeof(double);
    size_t ws_warps = static_cast<size_t>(ctx->sm_count) * 32;
    const size_t ws_cap = (size_t{4} << 30) / per_warp;
    if (ws_warps > ws_cap) ws_warps = ws_cap;
    if (ws_warps < 8) ws_warps = 8;
    cdet::ScratchRegions regions;
    regions.dd_lanes = dd || ctx->scratch_dd;
    const size_t bytes = cdet::scratch_bytes(new_batch, new_order, ws_warps, regions);
    if (ctx->scratch) {
        cudaDeviceSynchronize();
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
    }
    cudaError_t err = cudaMalloc(&ctx->scratch, bytes);
    if (err != cudaSuccess) {
        ctx->scratch_batch = 0;
        ctx->scratch_order = 0;
        ctx->scratch_dd = false;
        return cuda_fail(err, "cudaMalloc(scratch)");
    }
    ++ctx->generation;
    ctx->scratch_bytes = bytes;
    ctx->scratch_batch = new_batch;
    ctx->scratch_order = new_order;
    ctx->ws_warps = ws_warps;
    ctx->scratch_dd = regions.dd_lanes;
    return CDET_OK;
}

int build_problem(cdet_context* ctx, const double* vertices, const int32_t* orders,
                  int64_t batch, int max_order, int all_subsets, double* values,
                  int32_t* status, cdet::Problem* p) {
    const cdet_runtime_scalars& s = ctx->scalars;
    p->s = cdet::Scalars{s.n1, s.n2, s.cheb_nu, s.cheb_nv, s.beta, s.u, s.branch_eps, s.scale,
                         s.diag_up_shift, s.diag_down_shift, s.tol_fpm, s.fpm_shift, s.z_eps0,
                         s.z_safety};
    const int kinds[2][2] = {{CDET_TWISTED_UP, CDET_TWISTED_DOWN},
                             {CDET_ORDINARY_UP, CDET_ORDINARY_DOWN}};
    for (int set = 0; set < 2; ++set) {
        const cdet::TableDev* up = resolve(ctx, kinds[set][0]);
        const cdet::TableDev* down = resolve(ctx, kinds[set][1]);
        if (!up || !down) return fail(CDET_ERR_STATE, "Green-function tables have not been uploaded");
        p->up[set] = *up;
        p->down[set] = *down;
        p->same_spin[set] = (up->upper == down->upper && up->lower == down->lower &&
                             up->upper_corners == down->upper_corners &&
                             up->lower_corners == down->lower_corners &&
                             s.diag_up_shift == s.diag_down_shift)
                                ? 1
                                : 0;
    }
    p->vertices = vertices;
    p->orders = orders;
    p->batch = batch;
    p->max_order = max_order;
    p->all_subsets = all_subsets;
    p->fused_cdet = ctx->assembly == CDET_ASSEMBLY_SPLIT_BF16 ? 1 : 0;
    p->all_subsets_form = ctx->all_subsets_form;
    p->sorted = 0;
    p->integrand_form = cdet::kIntegrandStaged;
    p->queue = cdet::QueueShape{};
    p->reuse_green = nullptr;
    p->reuse_diag = nullptr;
    p->reuse_mask = nullptr;
    p->dd_mode = ctx->integrand_real == CDET_INTEGRAND_REAL_DOUBLE_DOUBLE ? 1 : 0;
    p->raw_diag = p->dd_mode;
    p->dd_shift[0] = ctx->dd_shift[0];
    p->dd_shift[1] = ctx->dd_shift[1];
    p->dd_threshold = ctx->dd_threshold;
    p->dd_u = ctx->dd_u;
    p->dd_beta = ctx->dd_beta;
    p->dd_tol = ctx->dd_tol;
    p->dd_fpm_shift = ctx->dd_fpm_shift;
    for (int set = 0; set < 2; ++set) {
        const int r = set == 0 ? 2 : 1;
        for (int n = 0; n <= cdet::kMaxOrder; ++n) {
            const HostDD dd = n >= 1 ? prefactor_dd(n, s.n1, s.n2, r) : HostDD{0.0, 0.0};
            p->pref_dd[set][n] = cdet::DDPair{dd.hi, dd.lo};
            p->pref_ld[set][n] = n >= 2 ? prefactor_ld(n, s.n1, s.n2, r) : 0.0;
        }
    }
    p->values = values;
    p->status = status;
    return CDET_OK;
}

int slice_branch(cdet_context* ctx, const double* coeffs, size_t blocks, SlicedBranch** out) {
    auto key = std::make_pair(coeffs, blocks);
    auto it = ctx->sliced.find(key);
    if (it != ctx->sliced.end()) {
        *out = &it->second;
        return CDET_OK;
    }
    const cdet_runtime_scalars& s = ctx->scalars;
    // slices, then the level rows (8-byte aligned), the exponents and the K-step leads
    const size_t sbytes = cdet::split_slices_bytes(s.cheb_nu, s.cheb_nv, blocks);
    const size_t rbytes = cdet::split_level_rows_bytes(s.cheb_nu, s.cheb_nv, blocks);
    const size_t lbytes = cdet::split_leads_bytes(s.cheb_nu, s.cheb_nv, blocks);
    // then the sub-blocks' tile costs (4-byte aligned)
    int nrb = 0, nkc = 0, ksteps_last = 0;
    cdet::split_geometry(s.cheb_nu, s.cheb_nv, &nrb, &nkc, &ksteps_last);
    const size_t cost_at = (sbytes + rbytes + blocks * sizeof(int32_t) + lbytes + 15) & ~static_cast<size_t>(15);
    const size_t cbytes = blocks * static_cast<size_t>(nrb) * nkc * sizeof(uint32_t);
    SlicedBranch b;
    cudaError_t err = cudaMalloc(&b.mem, cost_at + cbytes + 256);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc(split slices)");
    char* base = static_cast<char*>(b.mem);
    b.slices = reinterpret_cast<const uint16_t*>(base);
    b.level_rows = reinterpret_cast<const uint64_t*>(base + sbytes);
    b.exponents = reinterpret_cast<const int32_t*>(base + sbytes + rbytes);
    b.leads = reinterpret_cast<const uint8_t*>(base + sbytes + rbytes + blocks * sizeof(int32_t));
    b.key_costs = reinterpret_cast<const uint32_t*>(base + cost_at);
    b.blocks = blocks;
    err = cdet::launch_slice_table(coeffs, s.cheb_nu, s.cheb_nv, blocks, const_cast<uint16_t*>(b.slices),
                                   const_cast<int32_t*>(b.exponents), const_cast<uint8_t*>(b.leads),
                                   const_cast<uint64_t*>(b.level_rows), const_cast<uint32_t*>(b.key_costs), nullptr);
    if (err == cudaSuccess) err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        cudaFree(b.mem);
        return cuda_fail(err, "slicing the tables");
    }
    ++ctx->generation;
    auto res = ctx->sliced.emplace(key, b);
    *out = &res.first->second;
    return CDET_OK;
}

// The segments of the split assembly: per set, one record per distinct
// up/down table, and per record the two branches.
int build_split_plan(cdet_context* ctx, cdet::SplitPlan* plan) {
    const cdet_runtime_scalars& s = ctx->scalars;
    if (s.cheb_nu > cdet::kSplitMaxDegree || s.cheb_nv > cdet::kSplitMaxDegree)
        return fail(CDET_ERR_INVALID, "split assembly needs CHEB_NU and CHEB_NV <= 256");
    *plan = cdet::SplitPlan{};
    cdet::split_geometry(s.cheb_nu, s.cheb_nv, &plan->nrb, &plan->nkc, &plan->ksteps_last);
    const size_t nsub = static_cast<size_t>(plan->nrb) * plan->nkc;
    const size_t sites2 = static_cast<size_t>(s.n1) * s.n2 * s.n1 * s.n2;
    const int kinds[2][2] = {{CDET_TWISTED_UP, CDET_TWISTED_DOWN}, {CDET_ORDINARY_UP, CDET_ORDINARY_DOWN}};
    uint32_t base = 0;
    int seg = 0;
    for (int set = 0; set < 2; ++set) {
        const cdet::TableDev* up = resolve(ctx, kinds[set][0]);
        const cdet::TableDev* down = resolve(ctx, kinds[set][1]);
        if (!up || !down) return fail(CDET_ERR_STATE, "Green-function tables have not been uploaded");
        const bool shared = up->upper == down->upper && up->lower == down->lower;
        const cdet::TableDev* recs[2] = {up, down};
        plan->records_per_set[set] = shared ? 1 : 2;
        const size_t blocks = set == 0 ? 4 * sites2 : sites2;  // ordinary: replica (0,0) only
        for (int r = 0; r < plan->records_per_set[set]; ++r) {
            plan->spin_mask[set][r] = shared ? 3 : (1 << r);
            for (int br = 0; br < 2; ++br) {
                SlicedBranch* sb = nullptr;
                const int rc = slice_branch(ctx, br == 0 ? recs[r]->upper : recs[r]->lower, blocks, &sb);
                if (rc != CDET_OK) return rc;
                plan->segment_base[seg] = base;
                plan->slices[seg] = sb->slices;
                plan->exponents[seg] = sb->exponents;
                plan->leads[seg] = sb->leads;
                plan->level_rows[seg] = sb->level_rows;
                plan->key_costs[seg] = sb->key_costs;
                plan->segment_of[set][r][br] = seg;
                base += static_cast<uint32_t>(blocks * nsub);
                ++seg;
            }
        }
    }
    plan->segments = seg;
    plan->segment_base[seg] = base;
    plan->nblocks = base;
    return CDET_OK;
}

// Times the whole evaluation with each all-subsets form (twice each, so that
// neither pays the kernels' first-launch costs alone) and returns the faster.
// Both forms write the same values, so the evaluation's outputs stand.
int tune_all_subsets_form(cdet_context* ctx, cdet::Problem p, const cdet::Scratch& w, cudaStream_t stream,
                          int* best) {
    int rc = CDET_OK;
    if (ctx->assembly == CDET_ASSEMBLY_SPLIT_BF16) {
        // the split path needs its plan and scratch first: run it once in the automatic form
        cdet::SplitPlan plan;
        rc = build_split_plan(ctx, &plan);
        if (rc != CDET_OK) return rc;
        const size_t need = cdet::split_scratch_bytes(p.batch, p.max_order, plan);
        if (need > ctx->split_scratch_bytes) {
            cudaDeviceSynchronize();
            if (ctx->split_scratch) cudaFree(ctx->split_scratch);
            ctx->split_scratch = nullptr;
            ctx->split_scratch_bytes = 0;
            const cudaError_t err = cudaMalloc(&ctx->split_scratch, need);
            ++ctx->generation;
            if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc(split scratch)");
            ctx->split_scratch_bytes = need;
        }
    }
    auto launch = [&](int form) -> cudaError_t {
        p.all_subsets_form = form;
        if (ctx->assembly == CDET_ASSEMBLY_SPLIT_BF16) {
            cdet::SplitPlan plan;
            if (build_split_plan(ctx, &plan) != CDET_OK) return cudaErrorUnknown;
            cudaError_t err = cdet::launch_split_assembly(p, w, plan, ctx->split_scratch, ctx->split_scratch_bytes,
                                                          ctx->sm_count, &ctx->split_error, stream, nullptr);
            if (err != cudaSuccess) return err;
            return cdet::launch_fp64_integrand(p, w, ctx->sm_count, stream, nullptr, false);
        }
        return cdet::launch_fp64_integrand(p, w, ctx->sm_count, stream, nullptr);
    };
    cudaEvent_t ev[3];
    for (cudaEvent_t& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return cuda_fail(cudaGetLastError(), "cudaEventCreate");
    float ms[2] = {0.0f, 0.0f};
    cudaError_t err = cudaSuccess;
    for (int round = 0; round < 2 && err == cudaSuccess; ++round) {
        err = cudaEventRecord(ev[0], stream);
        if (err == cudaSuccess) err = launch(cdet::kFormLane);
        if (err == cudaSuccess) err = cudaEventRecord(ev[1], stream);
        if (err == cudaSuccess) err = launch(cdet::kFormWarp);
        if (err == cudaSuccess) err = cudaEventRecord(ev[2], stream);
        if (err == cudaSuccess) err = cudaEventSynchronize(ev[2]);
        if (err == cudaSuccess && round == 1) {
            err = cudaEventElapsedTime(&ms[0], ev[0], ev[1]);
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms[1], ev[1], ev[2]);
        }
    }
    for (cudaEvent_t& e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return cuda_fail(err, "timing the all-subsets forms");
    *best = ms[1] < ms[0] ? cdet::kFormWarp : cdet::kFormLane;
    return CDET_OK;
}

// Times the post-assembly stages of a single-top batch in every candidate
// form on the Green matrices already in scratch (each candidate twice, the
// second round timed, so none pays first-launch costs alone) and returns the
// fastest. Every form writes the same values and status bits, so the
// evaluation's outputs stand whichever ran last.
int tune_integrand_form(cdet_context* ctx, cdet::Problem p, const cdet::Scratch& w, cudaStream_t stream,
                        std::pair<int, cdet::QueueShape>* best) {
    std::vector<std::pair<int, cdet::QueueShape>> cand;
    cand.push_back({cdet::kIntegrandStaged, cdet::QueueShape{}});
    cdet::QueueShape q;
    q.warps_per_sm = 0, q.pair = 0, q.grab = 1;
    cand.push_back({cdet::kIntegrandQueue, q});  // one warp per configuration, as many as fit
    q.pair = 1;
    cand.push_back({cdet::kIntegrandQueue, q});  // two warps per configuration
    q.pair = 0, q.grab = 4;
    cand.push_back({cdet::kIntegrandQueue, q});  // four slots per pop
    q.grab = 1, q.warps_per_sm = 4;
    cand.push_back({cdet::kIntegrandQueue, q});  // four warps per SM (more L1 per warp)
    std::vector<cudaEvent_t> ev(cand.size() + 1);
    for (cudaEvent_t& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return cuda_fail(cudaGetLastError(), "cudaEventCreate");
    std::vector<float> ms(cand.size(), 0.0f);
    cudaError_t err = cudaSuccess;
    for (int round = 0; round < 2 && err == cudaSuccess; ++round) {
        err = cudaEventRecord(ev[0], stream);
        for (size_t i = 0; i < cand.size() && err == cudaSuccess; ++i) {
            p.integrand_form = cand[i].first;
            p.queue = cand[i].second;
            err = cdet::launch_post_assembly(p, w, ctx->sm_count, stream);
            if (err == cudaSuccess) err = cudaEventRecord(ev[i + 1], stream);
        }
        if (err == cudaSuccess) err = cudaEventSynchronize(ev[cand.size()]);
        for (size_t i = 0; round == 1 && i < cand.size() && err == cudaSuccess; ++i)
            err = cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
    }
    for (cudaEvent_t& e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return cuda_fail(err, "timing the integrand forms");
    size_t k = 0;
    for (size_t i = 1; i < cand.size(); ++i)
        if (ms[i] < ms[k]) k = i;
    *best = cand[k];
    return CDET_OK;
}

int run(cdet_context* ctx, const double* vertices, const int32_t* orders, int64_t batch,
        int max_order, int all_subsets, double* values, int32_t* status, cudaStream_t stream,
        bool assembly_only = false, const cdet::GreenReuse* reuse = nullptr) {
    if (batch < 0) return fail(CDET_ERR_INVALID, "batch must be non-negative");
    if (batch == 0) return CDET_OK;
    if (!vertices || !values || !status || (!all_subsets && !orders))
        return fail(CDET_ERR_INVALID, "null buffer");
    if (ctx->integrand_real == CDET_INTEGRAND_REAL_DOUBLE_DOUBLE && !assembly_only &&
        (all_subsets || max_order > cdet::kDDMaxOrder))
        return fail(CDET_ERR_INVALID, "double-double integrand: single-configuration integrands of order <= 10 only");
    int rc = ensure_scratch(ctx, batch, max_order);
    if (rc != CDET_OK) return rc;
    cdet::Problem p;
    rc = build_problem(ctx, vertices, orders, batch, max_order, all_subsets, values, status, &p);
    if (rc != CDET_OK) return rc;
    cdet::Scratch w;
    cdet::carve_scratch(ctx->scratch, ctx->scratch_batch, ctx->scratch_order, ctx->ws_warps, &w,
                        scratch_regions(ctx));
    // The carve above is for the reserved (batch, order); the kernels index
    // with the call's max_order, which only needs less.
    if (reuse) {
        w.green = reuse->green;
        w.diag = reuse->diag;
        p.reuse_green = reuse->prev_green;
        p.reuse_diag = reuse->prev_diag;
        p.reuse_mask = reuse->mask;
    }
    cudaError_t err = cudaMemsetAsync(status, 0, static_cast<size_t>(batch) * sizeof(int32_t), stream);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMemsetAsync(status)");
    cdet::KernelEvents* events = nullptr;
    if (ctx->profiling && !assembly_only) {
        if (ctx->spare.empty()) {
            cdet::KernelEvents ev{};
            for (cudaEvent_t& e : ev.marks) {
                err = cudaEventCreate(&e);
                if (err != cudaSuccess) return cuda_fail(err, "cudaEventCreate");
            }
            ctx->spare.push_back(ev);
        }
        ctx->pending.push_back(ctx->spare.back());
        ctx->spare.pop_back();
        events = &ctx->pending.back();
    }
    int launches = 3;
    // The all-subsets CDet has two work layouts with identical values; under
    // CDET_FORM_AUTO the first evaluation of each (order, fused, batch size
    // class) outside a stream capture times both and keeps the faster.
    if (p.all_subsets && ctx->all_subsets_form == CDET_FORM_AUTO && !assembly_only && !ctx->profiling &&
        max_order <= cdet::kAllWarpMaxOrder) {
        int log2b = 0;
        while ((int64_t{2} << log2b) <= batch) ++log2b;
        const auto key = std::make_tuple(max_order, p.fused_cdet, log2b);
        auto it = ctx->form_tuned.find(key);
        if (it == ctx->form_tuned.end()) {
            cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(stream, &capture) == cudaSuccess && capture == cudaStreamCaptureStatusNone) {
                int best = cdet::kFormAuto;
                rc = tune_all_subsets_form(ctx, p, w, stream, &best);
                if (rc != CDET_OK) return rc;
                it = ctx->form_tuned.emplace(key, best).first;
            }
        }
        if (it != ctx->form_tuned.end()) p.all_subsets_form = it->second;
    }
    // Single-top batches: the post-assembly form, fixed by
    // cdet_set_integrand_form or, under CDET_INTEGRAND_AUTO, measured once per
    // (order, fused, batch size class) outside a capture (staged until then).
    bool tune_post = false;
    std::tuple<int, int, int> post_key;
    if (p.dd_mode) {
        // the double-double integrand: STAGED = its lane form, QUEUE = its warp
        // form, AUTO = the lane form from one warp of configurations per SM
        p.integrand_form = ctx->integrand_form;
    } else if (!p.all_subsets && !assembly_only && max_order <= cdet::kQueueMaxOrder) {
        if (ctx->integrand_form != CDET_INTEGRAND_AUTO) {
            p.integrand_form = ctx->integrand_form;
            p.queue = ctx->queue_shape;
        } else {
            int log2b = 0;
            while ((int64_t{2} << log2b) <= batch) ++log2b;
            post_key = std::make_tuple(max_order, p.fused_cdet, log2b);
            auto it = ctx->integrand_tuned.find(post_key);
            if (it != ctx->integrand_tuned.end()) {
                p.integrand_form = it->second.first;
                p.queue = it->second.second;
            } else if (!ctx->profiling) {
                cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
                tune_post = cudaStreamIsCapturing(stream, &capture) == cudaSuccess &&
                            capture == cudaStreamCaptureStatusNone;
            }
        }
    }
    auto settle_post_form = [&]() -> int {
        if (!tune_post) return CDET_OK;
        std::pair<int, cdet::QueueShape> best;
        const int trc = tune_integrand_form(ctx, p, w, stream, &best);
        if (trc != CDET_OK) return trc;
        ctx->integrand_tuned.emplace(post_key, best);
        p.integrand_form = best.first;
        p.queue = best.second;
        return CDET_OK;
    };
    if (ctx->assembly == CDET_ASSEMBLY_SPLIT_BF16) {
        cdet::SplitPlan plan;
        rc = build_split_plan(ctx, &plan);
        if (rc != CDET_OK) return rc;
        const size_t need = cdet::split_scratch_bytes(batch, max_order, plan);
        if (need > ctx->split_scratch_bytes) {
            cudaDeviceSynchronize();
            if (ctx->split_scratch) cudaFree(ctx->split_scratch);
            ctx->split_scratch = nullptr;
            ctx->split_scratch_bytes = 0;
            err = cudaMalloc(&ctx->split_scratch, need);
            ++ctx->generation;
            if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc(split scratch)");
            ctx->split_scratch_bytes = need;
        }
        if (events && events->marks[0]) cudaEventRecord(events->marks[0], stream);
        err = cdet::launch_split_assembly(p, w, plan, ctx->split_scratch, ctx->split_scratch_bytes,
                                          ctx->sm_count, &ctx->split_error, stream, events);
        if (err != cudaSuccess) return cuda_fail(err, "split assembly launch");
        if (events && events->marks[2]) cudaEventRecord(events->marks[2], stream);
        if (!assembly_only) {
            rc = settle_post_form();
            if (rc != CDET_OK) return rc;
            err = cdet::launch_fp64_integrand(p, w, ctx->sm_count, stream, events, false);
            if (err != cudaSuccess) return cuda_fail(err, "kernel launch");
            // descriptors, scan, scatter, tiles and per-CTA ranges, tensor assembly + minors,
            // CDet (or the queue kernel, or the double-double kernel)
            launches = 5 + ((cdet::uses_queue_form(p) || p.dd_mode) ? 1 : 2);
        } else {
            launches = 5;
        }
        if (plan.nrb * plan.nkc > 1) ++launches;  // the sub-block combine
    } else if (!assembly_only) {
        if (tune_post) {
            err = cdet::launch_fp64_assembly_only(p, w, stream);
            if (err != cudaSuccess) return cuda_fail(err, "kernel launch");
            rc = settle_post_form();
            if (rc != CDET_OK) return rc;
            err = cdet::launch_post_assembly(p, w, ctx->sm_count, stream);
        } else {
            err = cdet::launch_fp64_integrand(p, w, ctx->sm_count, stream, events);
        }
        if (err != cudaSuccess) return cuda_fail(err, "kernel launch");
        // assembly + minors, CDet (or the queue kernel, or the double-double kernel)
        launches = (cdet::uses_queue_form(p) || p.dd_mode) ? 2 : 3;
        if (p.reuse_mask && p.all_subsets) launches += 2;  // the reuse scan and the copies
    } else {
        launches = 1;
        err = cdet::launch_fp64_assembly_only(p, w, stream);
        if (err != cudaSuccess) return cuda_fail(err, "kernel launch");
    }
    if (!assembly_only && cdet::sorts_orders(p)) launches += 3;  // the order sort of a mixed batch
    ctx->last_launches = launches;  // kernels of this library (the status and bucket resets are memsets)
    if (events) ctx->pending_launches += launches;
    return CDET_OK;
}

int run_host(cdet_context* ctx, const double* vertices, const int32_t* orders, int64_t batch,
             int order_arg, int all_subsets, double* values, int32_t* status) {
    if (batch <= 0) return batch == 0 ? CDET_OK : fail(CDET_ERR_INVALID, "batch must be non-negative");
    if (!vertices || !values || !status || (!all_subsets && !orders))
        return fail(CDET_ERR_INVALID, "null buffer");
    const size_t vbytes = static_cast<size_t>(batch) * order_arg * 4 * sizeof(double);
    const size_t obytes = all_subsets ? 0 : static_cast<size_t>(batch) * sizeof(int32_t);
    const size_t out_count = all_subsets ? static_cast<size_t>(batch) << order_arg : static_cast<size_t>(batch);
    const size_t valbytes = out_count * sizeof(double);
    const size_t sbytes = static_cast<size_t>(batch) * sizeof(int32_t);
    auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    const size_t need = up(vbytes) + up(obytes) + up(valbytes) + up(sbytes);
    if (need > ctx->staging_bytes) {
        if (ctx->staging) cudaFree(ctx->staging);
        ctx->staging = nullptr;
        cudaError_t err = cudaMalloc(&ctx->staging, need);
        if (err != cudaSuccess) {
            ctx->staging_bytes = 0;
            return cuda_fail(err, "cudaMalloc(staging)");
        }
        ctx->staging_bytes = need;
    }
    char* base = static_cast<char*>(ctx->staging);
    double* d_v = reinterpret_cast<double*>(base);
    int32_t* d_o = reinterpret_cast<int32_t*>(base + up(vbytes));
    double* d_val = reinterpret_cast<double*>(base + up(vbytes) + up(obytes));
    int32_t* d_s = reinterpret_cast<int32_t*>(base + up(vbytes) + up(obytes) + up(valbytes));
    cudaStream_t stream = nullptr;
    cudaError_t err = cudaMemcpyAsync(d_v, vertices, vbytes, cudaMemcpyHostToDevice, stream);
    if (err == cudaSuccess && obytes)
        err = cudaMemcpyAsync(d_o, orders, obytes, cudaMemcpyHostToDevice, stream);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMemcpyAsync(H2D)");
    int rc = run(ctx, d_v, all_subsets ? nullptr : d_o, batch, order_arg, all_subsets, d_val, d_s, stream);
    if (rc != CDET_OK) return rc;
    err = cudaMemcpyAsync(values, d_val, valbytes, cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaMemcpyAsync(status, d_s, sbytes, cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) return cuda_fail(err, "evaluation");
    if (ctx->assembly == CDET_ASSEMBLY_SPLIT_BF16 && ctx->split_error) {
        int32_t flag = 0;
        err = cudaMemcpy(&flag, ctx->split_error, sizeof(flag), cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) return cuda_fail(err, "reading the split assembly status");
        if (flag) return fail(CDET_ERR_CUDA, "split assembly: a pipeline wait timed out");
    }
    ctx->calls += static_cast<uint64_t>(batch);
    bool flagged = false;
    for (int64_t c = 0; c < batch; ++c) {
        if (status[c] & CDET_CONFIG_FPM_FALLBACK) ++ctx->fallbacks;
        if (status[c] & (CDET_CONFIG_NONFINITE | CDET_CONFIG_BAD_INPUT)) flagged = true;
    }
    if (flagged) return fail(CDET_ERR_VALUE, "Error (integrand): Value is not finite or input rejected");
    return CDET_OK;
}

}  // namespace

namespace capi {

const cdet::TableDev* resolve(const cdet_context* ctx, int kind) { return ::resolve(ctx, kind); }

int run(cdet_context* ctx, const double* vertices, const int32_t* orders, int64_t batch, int max_order,
        int all_subsets, double* values, int32_t* status, cudaStream_t stream, bool assembly_only,
        const cdet::GreenReuse* reuse) {
    return ::run(ctx, vertices, orders, batch, max_order, all_subsets, values, status, stream, assembly_only,
                 reuse);
}

}  // namespace capi

namespace cdet {

// Runs the FP64 form on scratch memory the caller provides (at least
// scratch_bytes(batch, max_order, ws_warps, regions) bytes), allocating
// nothing and recording no profiling events. Used by the no-allocation entry
// point.
int run_fp64_on_scratch(cdet_context* ctx, const double* vertices, const int32_t* orders, int64_t batch,
                        int max_order, double* values, int32_t* status, void* scratch, size_t ws_warps,
                        ScratchRegions regions, cudaStream_t stream) {
    Problem p;
    int rc = build_problem(ctx, vertices, orders, batch, max_order, 0, values, status, &p);
    if (rc != CDET_OK) return rc;
    p.fused_cdet = 0;  // the FP64 form throughout, whatever assembly the context selects
    p.dd_mode = 0;     // and the FP64 integrand, whatever INTEGRAND_REAL the context selects
    p.raw_diag = 0;
    Scratch w;
    carve_scratch(scratch, batch, max_order, ws_warps, &w, regions);
    cudaError_t err = cudaMemsetAsync(status, 0, static_cast<size_t>(batch) * sizeof(int32_t), stream);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMemsetAsync(status)");
    err = launch_fp64_integrand(p, w, ctx->sm_count, stream, nullptr);
    if (err != cudaSuccess) return cuda_fail(err, "kernel launch");
    ctx->last_launches = 3 + (sorts_orders(p) ? 3 : 0);
    return CDET_OK;
}

// Whether some table set evaluates two spins (distinct up and down tables or
// diagonal shifts); the minors then keep the spin-down minors too.
int context_two_spins(cdet_context* ctx, bool* two_spins) {
    Problem p;
    const int rc = build_problem(ctx, nullptr, nullptr, 0, 1, 0, nullptr, nullptr, &p);
    if (rc != CDET_OK) return rc;
    *two_spins = !(p.same_spin[0] && p.same_spin[1]);
    return CDET_OK;
}

int fail_with(int code, const char* message) { return fail(code, message); }
int context_device(const cdet_context* ctx) { return ctx->device; }
int context_sm_count(const cdet_context* ctx) { return ctx->sm_count; }

}  // namespace cdet

extern "C" {

const char* cdet_last_error(void) { return g_last_error.c_str(); }

int cdet_create(const cdet_runtime_scalars* scalars, int device, cdet_context** out) {
    if (!scalars || !out) return fail(CDET_ERR_INVALID, "null argument");
    *out = nullptr;
    const cdet_runtime_scalars& s = *scalars;
    if (s.n1 < 1 || s.n2 < 1 || s.cheb_nu < 1 || s.cheb_nv < 1)
        return fail(CDET_ERR_INVALID, "lattice extents and Chebyshev sizes must be positive");
    int count = 0;
    cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess) return cuda_fail(err, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return fail(CDET_ERR_INVALID, "no such CUDA device");
    DeviceGuard guard(device);
    cdet_context* ctx = new cdet_context();
    ctx->device = device;
    ctx->scalars = s;
    ctx->coeff_count = expected_coeffs(s);
    ctx->corner_count = expected_corners(s);
    err = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (err != cudaSuccess) {
        delete ctx;
        return cuda_fail(err, "cudaDeviceGetAttribute");
    }
    *out = ctx;
    return CDET_OK;
}

void cdet_destroy(cdet_context* ctx) {
    if (!ctx) return;
    DeviceGuard guard(ctx->device);
    cudaDeviceSynchronize();
    for (auto* list : {&ctx->pending, &ctx->spare})
        for (auto& ev : *list)
            for (cudaEvent_t e : ev.marks) cudaEventDestroy(e);
    for (TableSlot& slot : ctx->tables) release_slot(slot);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->staging) cudaFree(ctx->staging);
    if (ctx->split_scratch) cudaFree(ctx->split_scratch);
    for (auto& kv : ctx->sliced) cudaFree(kv.second.mem);
    delete ctx;
}

int cdet_upload_table(cdet_context* ctx, int kind, const cdet_table_view* t, size_t coeff_count,
                      size_t corner_count) {
    if (!ctx || !t || !valid_kind(kind)) return fail(CDET_ERR_INVALID, "bad argument");
    if (coeff_count != ctx->coeff_count || corner_count != ctx->corner_count)
        return fail(CDET_ERR_INVALID, "table size does not match N1, N2, CHEB_NU, CHEB_NV");
    if (!t->upper_coeffs || !t->lower_coeffs || !t->upper_corners || !t->lower_corners)
        return fail(CDET_ERR_INVALID, "null table array");
    DeviceGuard guard(ctx->device);
    TableSlot& slot = ctx->tables[kind];
    forget_slices(ctx, slot);
    release_slot(slot);
    const size_t cb = coeff_count * sizeof(double), kb = corner_count * sizeof(double);
    void* mem = nullptr;
    cudaError_t err = cudaMalloc(&mem, 2 * cb + 2 * kb);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc(table)");
    char* base = static_cast<char*>(mem);
    const void* src[4] = {t->upper_coeffs, t->lower_coeffs, t->upper_corners, t->lower_corners};
    const size_t off[4] = {0, cb, 2 * cb, 2 * cb + kb};
    const size_t len[4] = {cb, cb, kb, kb};
    for (int k = 0; k < 4; ++k) {
        err = cudaMemcpy(base + off[k], src[k], len[k], cudaMemcpyHostToDevice);
        if (err != cudaSuccess) {
            cudaFree(mem);
            return cuda_fail(err, "cudaMemcpy(table)");
        }
    }
    slot.owned = mem;
    slot.dev = cdet::TableDev{reinterpret_cast<const double*>(base), reinterpret_cast<const double*>(base + cb),
                              reinterpret_cast<const double*>(base + 2 * cb),
                              reinterpret_cast<const double*>(base + 2 * cb + kb)};
    slot.ready = true;
    return CDET_OK;
}

int cdet_bind_device_table(cdet_context* ctx, int kind, const cdet_table_view* t,
                           size_t coeff_count, size_t corner_count) {
    if (!ctx || !t || !valid_kind(kind)) return fail(CDET_ERR_INVALID, "bad argument");
    if (coeff_count != ctx->coeff_count || corner_count != ctx->corner_count)
        return fail(CDET_ERR_INVALID, "table size does not match N1, N2, CHEB_NU, CHEB_NV");
    if (!t->upper_coeffs || !t->lower_coeffs || !t->upper_corners || !t->lower_corners)
        return fail(CDET_ERR_INVALID, "null table array");
    TableSlot& slot = ctx->tables[kind];
    forget_slices(ctx, slot);
    release_slot(slot);
    slot.dev = cdet::TableDev{t->upper_coeffs, t->lower_coeffs, t->upper_corners, t->lower_corners};
    slot.ready = true;
    return CDET_OK;
}

int cdet_alias_table(cdet_context* ctx, int kind, int source_kind) {
    if (!ctx || !valid_kind(kind) || !valid_kind(source_kind) || kind == source_kind)
        return fail(CDET_ERR_INVALID, "bad argument");
    for (int k = source_kind; k >= 0; k = ctx->tables[k].alias_of)
        if (k == kind) return fail(CDET_ERR_INVALID, "alias cycle");
    TableSlot& slot = ctx->tables[kind];
    forget_slices(ctx, slot);
    release_slot(slot);
    slot.alias_of = source_kind;
    return CDET_OK;
}

int cdet_reserve(cdet_context* ctx, int64_t batch, int max_order) {
    if (!ctx || batch < 1 || max_order < 1 || max_order > cdet::kMaxOrder)
        return fail(CDET_ERR_INVALID, "bad argument");
    DeviceGuard guard(ctx->device);
    return ensure_scratch(ctx, batch, max_order);
}

int cdet_integrand_device(cdet_context* ctx, const double* vertices, const int32_t* orders,
                          int64_t batch, int max_order, double* values, int32_t* status,
                          void* stream) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (max_order < 1 || max_order > cdet::kMaxOrder)
        return fail(CDET_ERR_INVALID, "The replica integrand is defined only for order >= 1 (max 24 here)");
    DeviceGuard guard(ctx->device);
    return run(ctx, vertices, orders, batch, max_order, 0, values, status,
               static_cast<cudaStream_t>(stream));
}

int cdet_all_subsets_device(cdet_context* ctx, const double* vertices, int envelope_order,
                            int64_t batch, double* values, int32_t* status, void* stream) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (envelope_order <= 1 || envelope_order > cdet::kMaxOrder)
        return fail(CDET_ERR_INVALID,
                    "The all-subset replica integrand is defined only for envelope order >= 2 (max 24 here)");
    DeviceGuard guard(ctx->device);
    return run(ctx, vertices, nullptr, batch, envelope_order, 1, values, status,
               static_cast<cudaStream_t>(stream));
}

int cdet_integrand_host(cdet_context* ctx, const double* vertices, const int32_t* orders,
                        int64_t batch, int max_order, double* values, int32_t* status) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (max_order < 1 || max_order > cdet::kMaxOrder)
        return fail(CDET_ERR_INVALID, "The replica integrand is defined only for order >= 1 (max 24 here)");
    DeviceGuard guard(ctx->device);
    return run_host(ctx, vertices, orders, batch, max_order, 0, values, status);
}

int cdet_all_subsets_host(cdet_context* ctx, const double* vertices, int envelope_order,
                          int64_t batch, double* values, int32_t* status) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (envelope_order <= 1 || envelope_order > cdet::kMaxOrder)
        return fail(CDET_ERR_INVALID,
                    "The all-subset replica integrand is defined only for envelope order >= 2 (max 24 here)");
    DeviceGuard guard(ctx->device);
    return run_host(ctx, vertices, nullptr, batch, envelope_order, 1, values, status);
}

int cdet_counters(const cdet_context* ctx, uint64_t* integrand_calls, uint64_t* fpm_fallbacks) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (integrand_calls) *integrand_calls = ctx->calls;
    if (fpm_fallbacks) *fpm_fallbacks = ctx->fallbacks;
    return CDET_OK;
}

int cdet_last_launch_count(const cdet_context* ctx) { return ctx ? ctx->last_launches : 0; }

int cdet_all_subsets_form_tuned(const cdet_context* ctx, int max_order, int fused, int64_t batch, int* form) {
    if (!ctx || !form) return fail(CDET_ERR_INVALID, "null argument");
    int log2b = 0;
    while ((int64_t{2} << log2b) <= batch) ++log2b;
    const auto it = ctx->form_tuned.find(std::make_tuple(max_order, fused ? 1 : 0, log2b));
    *form = it == ctx->form_tuned.end() ? CDET_FORM_AUTO : it->second;
    return CDET_OK;
}

int cdet_set_all_subsets_form(cdet_context* ctx, int form) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (form != CDET_FORM_AUTO && form != CDET_FORM_LANE && form != CDET_FORM_WARP)
        return fail(CDET_ERR_INVALID, "unknown all-subsets form");
    static_assert(CDET_FORM_AUTO == cdet::kFormAuto && CDET_FORM_LANE == cdet::kFormLane &&
                      CDET_FORM_WARP == cdet::kFormWarp,
                  "form codes");
    ctx->all_subsets_form = form;
    return CDET_OK;
}

int cdet_set_integrand_form(cdet_context* ctx, int form, int warps_per_sm, int pair, int grab) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    static_assert(CDET_INTEGRAND_AUTO == cdet::kIntegrandAuto && CDET_INTEGRAND_STAGED == cdet::kIntegrandStaged &&
                      CDET_INTEGRAND_QUEUE == cdet::kIntegrandQueue,
                  "integrand form codes");
    if (form != CDET_INTEGRAND_AUTO && form != CDET_INTEGRAND_STAGED && form != CDET_INTEGRAND_QUEUE)
        return fail(CDET_ERR_INVALID, "unknown integrand form");
    if (warps_per_sm < 0 || warps_per_sm > 32 || (pair != 0 && pair != 1) || grab < 1 || grab > 64)
        return fail(CDET_ERR_INVALID, "queue shape: warps_per_sm in 0..32, pair 0 or 1, grab in 1..64");
    ctx->integrand_form = form;
    ctx->queue_shape.warps_per_sm = warps_per_sm;
    ctx->queue_shape.pair = pair;
    ctx->queue_shape.grab = grab;
    return CDET_OK;
}

int cdet_integrand_form_tuned(const cdet_context* ctx, int max_order, int fused, int64_t batch, int* form,
                              int* warps_per_sm, int* pair, int* grab) {
    if (!ctx || !form || !warps_per_sm || !pair || !grab) return fail(CDET_ERR_INVALID, "null argument");
    int log2b = 0;
    while ((int64_t{2} << log2b) <= batch) ++log2b;
    const auto it = ctx->integrand_tuned.find(std::make_tuple(max_order, fused ? 1 : 0, log2b));
    const cdet::QueueShape q = it == ctx->integrand_tuned.end() ? cdet::QueueShape{} : it->second.second;
    *form = it == ctx->integrand_tuned.end() ? CDET_INTEGRAND_AUTO : it->second.first;
    *warps_per_sm = q.warps_per_sm;
    *pair = q.pair;
    *grab = q.grab;
    return CDET_OK;
}

int cdet_set_integrand_real(cdet_context* ctx, int real_type, const cdet_dd_scalars* dd) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (real_type == CDET_INTEGRAND_REAL_DOUBLE) {
        ctx->integrand_real = real_type;
        return CDET_OK;
    }
    if (real_type != CDET_INTEGRAND_REAL_DOUBLE_DOUBLE) return fail(CDET_ERR_INVALID, "unknown INTEGRAND_REAL");
    if (!dd) return fail(CDET_ERR_INVALID, "double-double integrand: null scalars");
    auto h = [](cdet_dd x) { return HostDD{x.hi, x.lo}; };
    auto d = [](HostDD x) { return cdet::DDPair{x.hi, x.lo}; };
    if (dd->u.hi == 0.0 && dd->u.lo == 0.0) return fail(CDET_ERR_INVALID, "U must be non-zero");
    // make_integrand_runtime_scalars<DoubleDouble> (integrand_replica_randomly_sampled.h:98-119):
    // diagonal_up_shift = alpha_down / U, diagonal_down_shift = alpha_up / U
    ctx->dd_shift[0] = d(h_div(h(dd->alpha_down), h(dd->u)));
    ctx->dd_shift[1] = d(h_div(h(dd->alpha_up), h(dd->u)));
    // compute_dp_ztransform's roundoff_threshold = epsilon0 * safety_factor (:251)
    ctx->dd_threshold = d(h_mul(h(dd->z_eps0), h(dd->z_safety)));
    ctx->dd_u = d(h(dd->u));
    ctx->dd_beta = d(h(dd->beta));
    ctx->dd_tol = d(h(dd->tol_fpm));
    ctx->dd_fpm_shift = d(h(dd->fpm_shift));
    ctx->integrand_real = real_type;
    return CDET_OK;
}

int cdet_set_assembly(cdet_context* ctx, int mode) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (mode != CDET_ASSEMBLY_FP64 && mode != CDET_ASSEMBLY_SPLIT_BF16)
        return fail(CDET_ERR_INVALID, "unknown assembly mode");
    if (mode == CDET_ASSEMBLY_SPLIT_BF16 &&
        (ctx->scalars.cheb_nu > cdet::kSplitMaxDegree || ctx->scalars.cheb_nv > cdet::kSplitMaxDegree))
        return fail(CDET_ERR_INVALID, "split assembly needs CHEB_NU and CHEB_NV <= 256");
    if (ctx->assembly != mode) ++ctx->generation;
    ctx->assembly = mode;
    return CDET_OK;
}

int cdet_prepare_split(cdet_context* ctx) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    DeviceGuard guard(ctx->device);
    cdet::SplitPlan plan;
    return build_split_plan(ctx, &plan);
}

int cdet_assemble_device(cdet_context* ctx, const double* vertices, const int32_t* orders,
                         int64_t batch, int max_order, double* green, double* diag,
                         int32_t* status, void* stream) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    if (max_order < 1 || max_order > cdet::kMaxOrder) return fail(CDET_ERR_INVALID, "order out of range");
    if (!green || !diag) return fail(CDET_ERR_INVALID, "null buffer");
    DeviceGuard guard(ctx->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double scratch_dummy = 0.0;
    int rc = run(ctx, vertices, orders, batch, max_order, 0, &scratch_dummy, status, st, true);
    if (rc != CDET_OK) return rc;
    cdet::Scratch w;
    cdet::carve_scratch(ctx->scratch, ctx->scratch_batch, ctx->scratch_order, ctx->ws_warps, &w,
                        scratch_regions(ctx));
    const size_t gbytes = static_cast<size_t>(batch) * 4 * max_order * max_order * sizeof(double);
    const size_t dbytes = static_cast<size_t>(batch) * 4 * max_order * sizeof(double);
    cudaError_t err = cudaMemcpyAsync(green, w.green, gbytes, cudaMemcpyDeviceToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(diag, w.diag, dbytes, cudaMemcpyDeviceToDevice, st);
    if (err != cudaSuccess) return cuda_fail(err, "copying the Green matrices");
    return CDET_OK;
}

int cdet_diagonal_order1_density(cdet_context* ctx, double alpha_up, double alpha_down, double* out) {
    if (!ctx || !out) return fail(CDET_ERR_INVALID, "bad argument");
    DeviceGuard guard(ctx->device);
    const cdet::TableDev* tables[4];
    for (int k = 0; k < 4; ++k) {
        tables[k] = resolve(ctx, k);
        if (!tables[k]) return fail(CDET_ERR_STATE, "Green-function tables have not been uploaded");
    }
    const cdet_runtime_scalars& s = ctx->scalars;
    if (s.u == 0.0) return fail(CDET_ERR_INVALID, "The diagonal observable is undefined for U = 0");
    const int sites = s.n1 * s.n2;
    double* buf = nullptr;
    cudaError_t err = cudaMalloc(&buf, (static_cast<size_t>(3) * sites + 4) * sizeof(double));
    if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc(diagonal observable)");
    double* items = buf + 4;
    err = cdet::launch_diagonal_order1(tables, s.n1, s.n2, s.cheb_nu, s.cheb_nv, s.beta, s.u, alpha_up,
                                       alpha_down, items, buf, nullptr);
    if (err == cudaSuccess) err = cudaMemcpy(out, buf, 3 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (err != cudaSuccess) return cuda_fail(err, "diagonal observable");
    return CDET_OK;
}

int cdet_profile_enable(cdet_context* ctx, int enable) {
    if (!ctx) return fail(CDET_ERR_INVALID, "null context");
    ctx->profiling = enable != 0;
    return CDET_OK;
}

int cdet_profile_read(cdet_context* ctx, double* kernel_ms, int64_t* launches) {
    if (!ctx || !kernel_ms) return fail(CDET_ERR_INVALID, "bad argument");
    DeviceGuard guard(ctx->device);
    for (cdet::KernelEvents& ev : ctx->pending) {
        cudaError_t err = cudaEventSynchronize(ev.marks[4]);
        if (err != cudaSuccess) return cuda_fail(err, "cudaEventSynchronize");
        for (int k = 0; k < 4; ++k) {
            float ms = 0.0f;
            err = cudaEventElapsedTime(&ms, ev.marks[k], ev.marks[k + 1]);
            if (err != cudaSuccess) return cuda_fail(err, "cudaEventElapsedTime");
            kernel_ms[k] += ms;
        }
        ctx->spare.push_back(ev);
    }
    ctx->pending.clear();
    if (launches) *launches += ctx->pending_launches;
    ctx->pending_launches = 0;
    return CDET_OK;
}

int cdet_split_counters(cdet_context* ctx, uint64_t* out) {
    if (!ctx || !out) return fail(CDET_ERR_INVALID, "bad argument");
    out[0] = out[1] = 0;
    if (!ctx->split_error) return CDET_OK;
    DeviceGuard guard(ctx->device);
    const cudaError_t err = cudaMemcpy(out, reinterpret_cast<const char*>(ctx->split_error) + 8, 2 * sizeof(uint64_t),
                                       cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMemcpy(split counters)");
    return CDET_OK;
}

}  // extern "C"

// ------------------------------------------------ chunked table directory --
namespace {

bool read_key_values(const std::filesystem::path& path, std::map<std::string, std::string>& out) {
    std::ifstream in(path);
    if (!in.is_open()) return false;
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '#') continue;
        const size_t pos = line.find('=');
        if (pos == std::string::npos) continue;
        out[line.substr(0, pos)] = line.substr(pos + 1);
    }
    return true;
}

struct TransformJob {
    int kind, branch;  // branch 0 = upper, 1 = lower
    size_t begin, end;
};

int kind_index(const std::string& name) {
    static const char* names[4] = {"twisted_up", "twisted_down", "ordinary_up", "ordinary_down"};
    for (int k = 0; k < 4; ++k)
        if (name == names[k]) return k;
    return -1;
}

const char* kind_name(int k) {
    static const char* names[4] = {"twisted_up", "twisted_down", "ordinary_up", "ordinary_down"};
    return names[k];
}

std::string range_token(size_t begin, size_t end) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%010zu_%010zu", begin, end);
    return buf;
}

}  // namespace

extern "C" int cdet_load_chunks(cdet_context* ctx, const char* dir, double* order1) {
    namespace fs = std::filesystem;
    if (!ctx || !dir) return fail(CDET_ERR_INVALID, "bad argument");
    const fs::path root(dir);
    // ensure_manifest_matches_for_real (chunked_load_data.h:884-906) for the
    // entries this context can check
    std::map<std::string, std::string> manifest;
    if (!read_key_values(root / "manifest.txt", manifest))
        return fail(CDET_ERR_INVALID, "Could not open " + (root / "manifest.txt").string());
    const cdet_runtime_scalars& s = ctx->scalars;
    const size_t sitepairs = ctx->corner_count;
    const size_t nodes = static_cast<size_t>(s.cheb_nu) * s.cheb_nv;
    const std::pair<const char*, std::string> expected[] = {
        {"layout_version", "1"},
        {"N1", std::to_string(s.n1)},
        {"N2", std::to_string(s.n2)},
        {"CHEB_NU", std::to_string(s.cheb_nu)},
        {"CHEB_NV", std::to_string(s.cheb_nv)},
        {"node_count", std::to_string(nodes)},
        {"replica_sitepair_count", std::to_string(sitepairs)},
        {"LOAD_DATA_REAL", "double"},
        {"VECTOR_REAL", "double"},
    };
    for (const auto& [key, value] : expected) {
        auto it = manifest.find(key);
        if (it == manifest.end() || it->second != value)
            return fail(CDET_ERR_INVALID, std::string("Chunk manifest mismatch for ") + key + ": expected " + value +
                                              " but found " + (it == manifest.end() ? "(missing)" : it->second));
    }
    {
        auto it = manifest.find("BETA");
        if (it == manifest.end() || std::strtod(it->second.c_str(), nullptr) != s.beta)
            return fail(CDET_ERR_INVALID, "Chunk manifest mismatch for BETA");
    }
    if (!fs::exists(root / "READY"))
        return fail(CDET_ERR_INVALID, "Chunked load-data directory is missing READY: " + (root / "READY").string());
    // read_chunked_transform_jobs (:510-534)
    std::vector<TransformJob> jobs;
    {
        std::ifstream in(root / "transform_jobs.tsv");
        if (!in.is_open()) return fail(CDET_ERR_INVALID, "Could not open " + (root / "transform_jobs.tsv").string());
        std::string line;
        while (std::getline(in, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::vector<std::string> tok;
            size_t start = 0;
            while (true) {
                const size_t tab = line.find('\t', start);
                tok.push_back(line.substr(start, tab == std::string::npos ? std::string::npos : tab - start));
                if (tab == std::string::npos) break;
                start = tab + 1;
            }
            if (tok.size() < 5) return fail(CDET_ERR_INVALID, "Malformed transform job line: " + line);
            TransformJob j{kind_index(tok[1]), tok[2] == "upper" ? 0 : (tok[2] == "lower" ? 1 : -1),
                           static_cast<size_t>(std::stoull(tok[3])), static_cast<size_t>(std::stoull(tok[4]))};
            if (j.kind < 0 || j.branch < 0 || j.end < j.begin || j.end > sitepairs)
                return fail(CDET_ERR_INVALID, "Malformed transform job line: " + line);
            jobs.push_back(j);
        }
    }
    DeviceGuard guard(ctx->device);
    const size_t cb = ctx->coeff_count * sizeof(double), kb = sitepairs * sizeof(double);
    void* mem[4] = {nullptr, nullptr, nullptr, nullptr};
    char* pinned[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    cudaStream_t stream = nullptr;
    constexpr size_t kStage = size_t{32} << 20;
    int rc = CDET_OK;
    auto cleanup = [&](bool free_tables) {
        if (stream) cudaStreamSynchronize(stream);
        for (int i = 0; i < 2; ++i) {
            if (pinned[i]) cudaFreeHost(pinned[i]);
            if (done[i]) cudaEventDestroy(done[i]);
        }
        if (stream) cudaStreamDestroy(stream);
        if (free_tables)
            for (void* m : mem)
                if (m) cudaFree(m);
    };
    cudaError_t err = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    for (int i = 0; err == cudaSuccess && i < 2; ++i) {
        err = cudaHostAlloc(reinterpret_cast<void**>(&pinned[i]), kStage, cudaHostAllocDefault);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
    }
    for (int k = 0; err == cudaSuccess && k < 4; ++k) {
        err = cudaMalloc(&mem[k], 2 * cb + 2 * kb);
        if (err == cudaSuccess) err = cudaMemsetAsync(mem[k], 0, 2 * cb + 2 * kb, stream);  // uncovered ranges stay 0
    }
    if (err != cudaSuccess) {
        cleanup(true);
        return cuda_fail(err, "allocating the chunked tables");
    }
    int slot_i = 0;
    // one file into device memory through the two pinned buffers
    auto stream_file = [&](const fs::path& path, size_t bytes, char* dst) -> int {
        std::error_code ec;
        const auto size = fs::file_size(path, ec);
        if (ec) return fail(CDET_ERR_INVALID, "Could not stat " + path.string());
        if (static_cast<size_t>(size) != bytes)
            return fail(CDET_ERR_INVALID, "Unexpected file size for " + path.string() + ": expected " +
                                              std::to_string(bytes) + " bytes, got " + std::to_string(size));
        FILE* f = std::fopen(path.string().c_str(), "rb");
        if (!f) return fail(CDET_ERR_INVALID, "Could not open " + path.string());
        while (bytes > 0) {
            const size_t n = bytes < kStage ? bytes : kStage;
            cudaError_t e = cudaEventSynchronize(done[slot_i]);
            if (e != cudaSuccess || std::fread(pinned[slot_i], 1, n, f) != n) {
                std::fclose(f);
                return e != cudaSuccess ? cuda_fail(e, "chunk copy") : fail(CDET_ERR_INVALID, "Short read from " + path.string());
            }
            e = cudaMemcpyAsync(dst, pinned[slot_i], n, cudaMemcpyHostToDevice, stream);
            if (e == cudaSuccess) e = cudaEventRecord(done[slot_i], stream);
            if (e != cudaSuccess) {
                std::fclose(f);
                return cuda_fail(e, "chunk copy");
            }
            dst += n;
            bytes -= n;
            slot_i ^= 1;
        }
        std::fclose(f);
        return CDET_OK;
    };
    // load_coeff_chunks_for_branch (:1372-1392)
    for (const TransformJob& j : jobs) {
        const fs::path path = root / "coeffs" / kind_name(j.kind) / (j.branch == 0 ? "upper" : "lower") /
                              ("sitepairs_" + range_token(j.begin, j.end) + ".bin");
        char* dst = static_cast<char*>(mem[j.kind]) + (j.branch == 0 ? 0 : cb) + j.begin * nodes * sizeof(double);
        rc = stream_file(path, (j.end - j.begin) * nodes * sizeof(double), dst);
        if (rc != CDET_OK) break;
    }
    // load_corner_chunk_for_branch (:1394-1406)
    for (int k = 0; rc == CDET_OK && k < 4; ++k)
        for (int b = 0; rc == CDET_OK && b < 2; ++b) {
            const fs::path path = root / "corners" / kind_name(k) / (b == 0 ? "upper.bin" : "lower.bin");
            rc = stream_file(path, kb, static_cast<char*>(mem[k]) + 2 * cb + b * kb);
        }
    if (rc == CDET_OK) {
        err = cudaStreamSynchronize(stream);
        if (err != cudaSuccess) rc = cuda_fail(err, "chunk copy");
    }
    if (rc != CDET_OK) {
        cleanup(true);
        return rc;
    }
    cleanup(false);
    for (int k = 0; k < 4; ++k) {
        TableSlot& slot = ctx->tables[k];
        forget_slices(ctx, slot);
        release_slot(slot);
        char* base = static_cast<char*>(mem[k]);
        slot.owned = mem[k];
        slot.dev = cdet::TableDev{reinterpret_cast<const double*>(base), reinterpret_cast<const double*>(base + cb),
                                  reinterpret_cast<const double*>(base + 2 * cb),
                                  reinterpret_cast<const double*>(base + 2 * cb + kb)};
        slot.ready = true;
    }
    // read_chunked_diagonal_observable_value (:1320-1329), when present
    if (order1) {
        order1[0] = order1[1] = std::nan("");
        std::map<std::string, std::string> diag;
        if (read_key_values(root / "diagonal_observable.txt", diag)) {
            auto hi = diag.find("order1_hi"), lo = diag.find("order1_lo");
            if (hi == diag.end() || lo == diag.end())
                return fail(CDET_ERR_INVALID, "Malformed " + (root / "diagonal_observable.txt").string());
            order1[0] = std::stod(hi->second);
            order1[1] = std::stod(lo->second);
        }
    }
    return CDET_OK;
}
