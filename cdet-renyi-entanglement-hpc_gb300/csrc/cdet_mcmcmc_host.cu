// MCMCMC chains resident on the GPU: the host runtime of the C ABI's
// cdet_mcmcmc_* entry points (declared in include/cdet_gb300.h). The step
// kernels are in cdet_mcmcmc.cu.
//
// A step is the all-subset integrand of every chain's envelope, the step
// kernel, and a one-thread kernel that advances the row of the step-output
// ring, all on the chains' own stream. After one direct step (which creates
// every buffer the step needs) the three are captured once in a CUDA graph
// per (vertex buffer, warmup) and replayed; a change of the context's
// buffers (its generation) drops the graphs. The ring has two halves of
// ring_steps rows; when a half is full it is copied to pinned host memory and,
// while the GPU runs the next half, host threads fold it into every chain's
// MCMCMCChainResult in long double, as run_single_mcmcmc_chain
// (mcmcmc_sampler.h:1036-1084) does.
#include "cdet_capi_internal.h"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <limits>
#include <random>
#include <string>
#include <thread>
#include <vector>

using namespace capi;

struct cdet_mcmcmc {
    cdet_context* ctx = nullptr;
    cdet_mcmcmc_config cfg{};
    int64_t chains = 0;
    double inv_binom[cdet::kMcmcmcMaxEnvelope + 1] = {};
    void* block = nullptr;
    double* vert[2] = {nullptr, nullptr};
    int cur = 0;
    double* values = nullptr;
    int32_t* istatus = nullptr;
    double* lambdas = nullptr;
    uint64_t* mt = nullptr;
    int32_t* mt_index = nullptr;
    uint64_t* counts = nullptr;
    int32_t* error = nullptr;
    int64_t warmup_done = 0;
    // histogram seed kernel (tau_bins > 0): probabilities, CDFs and the
    // conditional generation probabilities scratch in one allocation
    int tau_bins = 0;
    void* hist_block = nullptr;
    double *tau_prob = nullptr, *space_prob = nullptr, *replica_prob = nullptr;
    double *tau_cdf = nullptr, *space_cdf = nullptr, *replica_cdf = nullptr;
    double* cprob = nullptr;
    // host side: seeds, current lambdas [chains][envelope + 1], results
    std::vector<uint64_t> seeds;
    std::vector<double> host_lambdas;
    std::vector<cdet_mcmcmc_chain_result> results;
    // step-output ring: rows [2 ring_steps][chains] of chosen masks, local
    // normalisations and order signals, a device row counter, and its pinned
    // host copy
    cudaStream_t stream = nullptr;
    int64_t ring_steps = 0;
    void* ring = nullptr;
    int64_t* d_row = nullptr;
    uint64_t* d_chosen = nullptr;
    double* d_norm = nullptr;
    double* d_signal = nullptr;
    void* pinned = nullptr;
    uint64_t* h_chosen = nullptr;
    double* h_norm = nullptr;
    double* h_signal = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr};
    int64_t row = 0;  // host mirror of *d_row
    // CUDA graphs of one step, [vertex buffer][warmup]
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    uint64_t graph_generation = 0;
    uint64_t ready_generation = ~uint64_t{0};
    bool use_graphs = true;
    int launches_per_step = 0;
    int64_t kernel_launches = 0;
    int64_t graph_steps = 0;
    // Green-pair reuse: the Green matrices and diagonals of the evaluation of
    // vert[b] in green2[b] / diag2[b], and per chain the chosen mask whose
    // vertices lead the next vertex buffer (written by the step kernel);
    // zeroed whenever the previous matrices cannot be reused (first step,
    // restored vertices, new tables or buffers, another assembly)
    void* reuse_block = nullptr;
    double* green2[2] = {nullptr, nullptr};
    double* diag2[2] = {nullptr, nullptr};
    uint64_t* retained = nullptr;
    bool green_reuse = true;
    uint64_t reuse_generation = ~uint64_t{0};
};

namespace {

int64_t ring_rows(const cdet_mcmcmc* m) { return 2 * m->ring_steps; }

// RunningStatsLongDouble::add (mcmcmc_sampler.h:36-42): Welford's update
void stats_add(cdet_running_stats& s, long double value) {
    ++s.count;
    const long double delta = value - s.mean;
    s.mean += delta / static_cast<long double>(s.count);
    const long double delta2 = value - s.mean;
    s.m2 += delta * delta2;
}

// RunningStatsLongDouble::stderr (:70-76)
long double stats_stderr(const cdet_running_stats& s) {
    if (s.count < 2) return std::numeric_limits<long double>::quiet_NaN();
    return std::sqrt((s.m2 / static_cast<long double>(s.count - 1)) / static_cast<long double>(s.count));
}

// adapt_mcmcmc_lambdas (mcmcmc_sampler.h:579-600) for every chain with a
// nonzero block (only_pending: the partial last block, :1050-1054), then the
// counts are cleared. Waits for the chains' stream first.
int mcmcmc_adapt(cdet_mcmcmc* m, bool only_pending) {
    const int env = m->cfg.envelope_order;
    const size_t n = static_cast<size_t>(m->chains) * (env + 1);
    std::vector<uint64_t> counts(n);
    std::vector<double>& lambdas = m->host_lambdas;
    cudaError_t err = cudaStreamSynchronize(m->stream);
    if (err == cudaSuccess)
        err = cudaMemcpy(counts.data(), m->counts, n * sizeof(uint64_t), cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC lambda adaptation");
    const int omin = m->cfg.order_min, omax = m->cfg.order_max;
    const int order_count = omax - omin + 1;
    const double target = 1.0 / static_cast<double>(order_count);
    for (int64_t c = 0; c < m->chains; ++c) {
        uint64_t* cc = counts.data() + c * (env + 1);
        double* lam = lambdas.data() + c * (env + 1);
        bool pending = false;
        for (int o = 0; o <= env; ++o) pending |= cc[o] != 0;
        if (only_pending && !pending) continue;
        uint64_t total = 0;
        for (int o = omin; o <= omax; ++o) total += cc[o];
        if (total != 0) {
            for (int o = omin; o <= omax; ++o) {
                const double actual = (static_cast<double>(cc[o]) + 1.0) /
                                      (static_cast<double>(total) + static_cast<double>(order_count));
                lam[o] *= std::exp(m->cfg.lambda_adapt_rate * std::log(target / actual));
            }
        }
        for (int o = 0; o <= env; ++o) cc[o] = 0;
    }
    err = cudaMemcpy(m->counts, counts.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(m->lambdas, lambdas.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC lambda adaptation");
    return CDET_OK;
}

cdet::McmcmcStepArgs step_args(const cdet_mcmcmc* m, int warmup) {
    const int env = m->cfg.envelope_order;
    cdet::McmcmcStepArgs a{};
    a.chains = m->chains;
    a.envelope = env;
    a.order_min = m->cfg.order_min;
    a.order_max = m->cfg.order_max;
    a.warmup = warmup ? 1 : 0;
    for (int o = 0; o <= env; ++o) a.inv_binom[o] = m->inv_binom[o];
    a.values = m->values;
    a.integrand_status = m->istatus;
    a.vertices = m->vert[m->cur];
    a.next_vertices = m->vert[m->cur ^ 1];
    a.lambdas = m->lambdas;
    a.mt = m->mt;
    a.mt_index = m->mt_index;
    a.counts = m->counts;
    a.error = m->error;
    a.ring_row = m->d_row;
    a.chosen_out = m->d_chosen;
    a.retained_out = m->retained;
    a.norm_out = m->d_norm;
    a.signal_out = m->d_signal;
    if (m->tau_bins > 0) {
        a.tau_bins = m->tau_bins;
        a.n1 = m->ctx->scalars.n1;
        a.n2 = m->ctx->scalars.n2;
        a.tau_prob = m->tau_prob;
        a.space_prob = m->space_prob;
        a.replica_prob = m->replica_prob;
        a.tau_cdf = m->tau_cdf;
        a.space_cdf = m->space_cdf;
        a.replica_cdf = m->replica_cdf;
        a.cprob = m->cprob;
    }
    return a;
}

// Enqueues one step (integrand, step kernel, ring row advance) on the
// chains' stream; *launches = the kernels it launches.
int enqueue_step(cdet_mcmcmc* m, int warmup, int* launches) {
    // the Green matrices of this step's vertices go to green2[cur]; pairs of
    // retained vertices are copied from green2[cur ^ 1], the previous step's
    const cdet::GreenReuse reuse{m->green2[m->cur], m->diag2[m->cur], m->green2[m->cur ^ 1], m->diag2[m->cur ^ 1],
                                 m->green_reuse ? m->retained : nullptr};
    int rc = run(m->ctx, m->vert[m->cur], nullptr, m->chains, m->cfg.envelope_order, 1, m->values, m->istatus,
                 m->stream, false, &reuse);
    if (rc != CDET_OK) return rc;
    int step_kernels = 0;
    cudaError_t err = cdet::launch_mcmcmc_step(step_args(m, warmup), m->stream, &step_kernels);
    if (err == cudaSuccess) err = cdet::launch_mcmcmc_advance_row(m->d_row, ring_rows(m), m->stream);
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC step launch");
    *launches = m->ctx->last_launches + step_kernels + 1;
    return CDET_OK;
}

void drop_graphs(cdet_mcmcmc* m) {
    for (auto& per_buffer : m->graph)
        for (cudaGraphExec_t& g : per_buffer)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
}

// One step: a graph replay when a graph of this step is current, otherwise a
// direct launch (capturing the graph first once a direct step has run at the
// context's current generation).
int launch_step(cdet_mcmcmc* m, int warmup) {
    cdet_context* ctx = m->ctx;
    // the previous step's Green matrices came from other tables, buffers or
    // another assembly (each bumps the context's generation): none is reused
    if (m->reuse_generation != ctx->generation) {
        const cudaError_t err = cudaMemsetAsync(m->retained, 0, static_cast<size_t>(m->chains) * 8, m->stream);
        if (err != cudaSuccess) return cuda_fail(err, "MCMCMC Green-pair reuse reset");
        m->reuse_generation = ctx->generation;
    }
    const bool graphs = m->use_graphs && !ctx->profiling;
    if (graphs && m->graph_generation != ctx->generation) {
        drop_graphs(m);
        m->graph_generation = ctx->generation;
    }
    cudaGraphExec_t& g = m->graph[m->cur][warmup ? 1 : 0];
    if (graphs && !g && m->ready_generation == ctx->generation) {
        cudaGraph_t graph = nullptr;
        int launches = 0;
        int rc = CDET_ERR_CUDA;
        cudaError_t err = cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
            rc = enqueue_step(m, warmup, &launches);
            err = cudaStreamEndCapture(m->stream, &graph);
        }
        if (err == cudaSuccess && rc == CDET_OK && graph) err = cudaGraphInstantiate(&g, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (err != cudaSuccess || rc != CDET_OK || !g) {
            // launch directly from now on; the capture enqueued nothing
            g = nullptr;
            m->use_graphs = false;
            cudaGetLastError();
        } else {
            m->launches_per_step = launches;
        }
    }
    if (graphs && g) {
        const cudaError_t err = cudaGraphLaunch(g, m->stream);
        if (err != cudaSuccess) return cuda_fail(err, "MCMCMC step graph launch");
        m->kernel_launches += m->launches_per_step;
        ++m->graph_steps;
    } else {
        int launches = 0;
        const int rc = enqueue_step(m, warmup, &launches);
        if (rc != CDET_OK) return rc;
        m->kernel_launches += launches;
        m->ready_generation = ctx->generation;  // every buffer of the step exists now
    }
    m->cur ^= 1;
    return CDET_OK;
}

// Runs fn(first_chain, end_chain) over the chains on up to the host's
// hardware threads (work = chain-steps to fold).
template <typename F>
void parallel_chains(int64_t chains, int64_t work, F&& fn) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int64_t threads = std::min<int64_t>({static_cast<int64_t>(hw), chains, std::max<int64_t>(1, work / 2048)});
    if (threads <= 1) {
        fn(int64_t{0}, chains);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(threads));
    for (int64_t t = 0; t < threads; ++t) {
        const int64_t a = chains * t / threads, b = chains * (t + 1) / threads;
        pool.emplace_back([&fn, a, b] { fn(a, b); });
    }
    for (std::thread& th : pool) th.join();
}

// Folds ring rows [first_row, first_row + n) (run steps first_step...) of
// the pinned copy into the chain results (run_single_mcmcmc_chain,
// :1036-1084) and the caller's optional outputs.
void fold_rows(cdet_mcmcmc* m, int warmup, int64_t first_row, int64_t n, int64_t first_step, uint64_t* chosen,
               double* norms, double* signal) {
    const int env = m->cfg.envelope_order, e1 = env + 1;
    const int omin = m->cfg.order_min, omax = m->cfg.order_max;
    const int64_t chains = m->chains;
    const long double envelope = static_cast<long double>(env);
    parallel_chains(chains, chains * n, [&](int64_t c0, int64_t c1) {
        for (int64_t c = c0; c < c1; ++c) {
            cdet_mcmcmc_chain_result& r = m->results[static_cast<size_t>(c)];
            const double* lam = m->host_lambdas.data() + c * e1;
            for (int64_t k = 0; k < n; ++k) {
                const int64_t row = first_row + k;
                const uint64_t mask = m->h_chosen[row * chains + c];
                const double* sig = m->h_signal + (row * chains + c) * e1;
                const int64_t step = first_step + k;
                if (chosen) chosen[step * chains + c] = mask;
                if (norms) norms[step * chains + c] = m->h_norm[row * chains + c];
                if (signal) std::memcpy(signal + (step * chains + c) * e1, sig, sizeof(double) * e1);
                if (mask == 0) continue;  // the chain stopped with an error
                const int order = __builtin_popcountll(mask);
                const long double retained = static_cast<long double>(order) / envelope;
                if (warmup) {
                    ++r.warmup_proposed_steps;
                    ++r.warmup_accepted_steps;
                    ++r.warmup_chosen_counts[order];
                    stats_add(r.warmup_retained_fraction_stats, retained);
                } else {
                    ++r.production_proposed_steps;
                    ++r.production_accepted_steps;
                    ++r.production_chosen_counts[order];
                    stats_add(r.production_retained_fraction_stats, retained);
                    for (int o = omin; o <= omax; ++o) stats_add(r.order_signal_stats[o], sig[o] / lam[o]);
                }
            }
        }
    });
}

int chain_errors(cdet_mcmcmc* m) {
    std::vector<int32_t> errors(static_cast<size_t>(m->chains));
    cudaError_t err = cudaMemcpy(errors.data(), m->error, m->chains * 4, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC status");
    for (int64_t c = 0; c < m->chains; ++c) {
        if (errors[c] == 1)
            return fail(CDET_ERR_VALUE, "Error (all-subset integrand): Value is not finite (chain " +
                                            std::to_string(c) + ")");
        if (errors[c] == 2)
            return fail(CDET_ERR_VALUE,
                        "MCMCMC local normalization is zero or non-finite (chain " + std::to_string(c) + ")");
        if (errors[c] == 3)
            return fail(CDET_ERR_VALUE,
                        "MCMCMC seed density is negative or non-finite (chain " + std::to_string(c) + ")");
    }
    if (m->ctx->assembly == CDET_ASSEMBLY_SPLIT_BF16 && m->ctx->split_error) {
        int32_t flag = 0;
        err = cudaMemcpy(&flag, m->ctx->split_error, sizeof(flag), cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) return cuda_fail(err, "reading the split assembly status");
        if (flag) return fail(CDET_ERR_CUDA, "split assembly: a pipeline wait timed out");
    }
    return CDET_OK;
}

void free_chains(cdet_mcmcmc* m) {
    drop_graphs(m);
    for (cudaEvent_t& e : m->copied)
        if (e) cudaEventDestroy(e);
    if (m->stream) cudaStreamDestroy(m->stream);
    if (m->pinned) cudaFreeHost(m->pinned);
    if (m->ring) cudaFree(m->ring);
    if (m->block) cudaFree(m->block);
    if (m->hist_block) cudaFree(m->hist_block);
    if (m->reuse_block) cudaFree(m->reuse_block);
    delete m;
}

}  // namespace

extern "C" {

int cdet_mcmcmc_create(cdet_context* ctx, const cdet_mcmcmc_config* config, int64_t chains, const uint64_t* seeds,
                       const double* lambdas, cdet_mcmcmc** out) {
    if (!ctx || !config || !seeds || !lambdas || !out) return fail(CDET_ERR_INVALID, "null argument");
    const cdet_mcmcmc_config& c = *config;
    // validate_mcmcmc_config (mcmcmc_sampler.h:432-493)
    if (c.order_min < 1) return fail(CDET_ERR_INVALID, "MCMCMC_ORDER_MIN must be at least 1 for the replica integrand");
    if (c.order_max < c.order_min) return fail(CDET_ERR_INVALID, "MCMCMC_ORDER_MAX must be >= MCMCMC_ORDER_MIN");
    if (c.envelope_order <= c.order_max)
        return fail(CDET_ERR_INVALID, "MCMCMC_ENVELOPE_ORDER must be larger than MCMCMC_ORDER_MAX");
    if (c.envelope_order > cdet::kMcmcmcMaxEnvelope)
        return fail(CDET_ERR_INVALID, "MCMCMC_ENVELOPE_ORDER must be <= 24 for the GPU chains");
    if (chains <= 0) return fail(CDET_ERR_INVALID, "MCMCMC_CHAIN_COUNT must be positive");
    if (c.lambda_adapt_interval <= 0) return fail(CDET_ERR_INVALID, "MCMCMC_LAMBDA_ADAPT_INTERVAL must be positive");
    for (int o = c.order_min; o <= c.order_max; ++o)
        if (!(lambdas[o] > 0.0) || !std::isfinite(lambdas[o]))
            return fail(CDET_ERR_INVALID, "MCMCMC_LAMBDAS entries must be positive finite numbers");
    for (int k = 0; k < 4; ++k)
        if (!resolve(ctx, k)) return fail(CDET_ERR_STATE, "Green-function tables have not been uploaded");
    DeviceGuard guard(ctx->device);
    auto* m = new cdet_mcmcmc;
    m->ctx = ctx;
    m->cfg = c;
    m->chains = chains;
    const int env = c.envelope_order;
    const int e1 = env + 1;
    for (int o = c.order_min; o <= c.order_max; ++o) {
        // 1 / binomial_as_double(envelope, order) (:174-185); the binomial is an exact integer here
        uint64_t b = 1;
        const int k = o < env - o ? o : env - o;
        for (int i = 1; i <= k; ++i) b = b * static_cast<uint64_t>(env - k + i) / static_cast<uint64_t>(i);
        m->inv_binom[o] = 1.0 / static_cast<double>(b);
    }
    m->seeds.assign(seeds, seeds + chains);
    m->host_lambdas.resize(static_cast<size_t>(chains) * e1);
    for (int64_t ch = 0; ch < chains; ++ch)
        for (int o = 0; o <= env; ++o) m->host_lambdas[ch * e1 + o] = lambdas[o];
    m->results.assign(static_cast<size_t>(chains), cdet_mcmcmc_chain_result{});
    for (int64_t ch = 0; ch < chains; ++ch) m->results[static_cast<size_t>(ch)].seed = seeds[ch];

    const size_t nv = static_cast<size_t>(chains) * env * 4;
    const size_t nvals = static_cast<size_t>(chains) << env;
    const size_t nl = static_cast<size_t>(chains) * e1;
    const size_t nmt = static_cast<size_t>(chains) * 312;
    auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    const size_t bytes = 2 * up(nv * 8) + up(nvals * 8) + up(chains * 4) + up(nl * 8) + up(nmt * 8) +
                         up(chains * 4) + up(nl * 8) + up(chains * 4) + up(chains * 8);
    // ring halves of up to 256 steps and 16 MiB
    const size_t per_step = static_cast<size_t>(chains) * (2 + e1) * 8;
    m->ring_steps = std::max<int64_t>(1, std::min<int64_t>(256, static_cast<int64_t>((size_t{16} << 20) / per_step)));
    const size_t ring_bytes = up(8) + 2 * static_cast<size_t>(m->ring_steps) * per_step;
    const size_t ng = static_cast<size_t>(chains) * 4 * env * env, nd = static_cast<size_t>(chains) * 4 * env;
    const size_t reuse_bytes = 2 * up(ng * 8) + 2 * up(nd * 8) + up(chains * 8);
    cudaError_t err = cudaMalloc(&m->block, bytes);
    if (err == cudaSuccess) err = cudaMalloc(&m->reuse_block, reuse_bytes);
    if (err == cudaSuccess) err = cudaMalloc(&m->ring, ring_bytes);
    if (err == cudaSuccess) err = cudaMallocHost(&m->pinned, ring_bytes);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    for (cudaEvent_t& e : m->copied)
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (err != cudaSuccess) {
        free_chains(m);
        return cuda_fail(err, "allocating the MCMCMC chains");
    }
    char* p = static_cast<char*>(m->block);
    auto take = [&](size_t b) {
        void* r = p;
        p += up(b);
        return r;
    };
    m->vert[0] = static_cast<double*>(take(nv * 8));
    m->vert[1] = static_cast<double*>(take(nv * 8));
    m->values = static_cast<double*>(take(nvals * 8));
    m->istatus = static_cast<int32_t*>(take(chains * 4));
    m->lambdas = static_cast<double*>(take(nl * 8));
    m->mt = static_cast<uint64_t*>(take(nmt * 8));
    m->mt_index = static_cast<int32_t*>(take(chains * 4));
    m->counts = static_cast<uint64_t*>(take(nl * 8));
    m->error = static_cast<int32_t*>(take(chains * 4));
    uint64_t* dseeds = static_cast<uint64_t*>(take(chains * 8));
    p = static_cast<char*>(m->reuse_block);
    for (int b = 0; b < 2; ++b) m->green2[b] = static_cast<double*>(take(ng * 8));
    for (int b = 0; b < 2; ++b) m->diag2[b] = static_cast<double*>(take(nd * 8));
    m->retained = static_cast<uint64_t*>(take(chains * 8));
    const size_t rows = 2 * static_cast<size_t>(m->ring_steps);
    m->d_row = static_cast<int64_t*>(m->ring);
    m->d_chosen = reinterpret_cast<uint64_t*>(static_cast<char*>(m->ring) + up(8));
    m->d_norm = reinterpret_cast<double*>(m->d_chosen + rows * chains);
    m->d_signal = m->d_norm + rows * chains;
    m->h_chosen = reinterpret_cast<uint64_t*>(static_cast<char*>(m->pinned) + up(8));
    m->h_norm = reinterpret_cast<double*>(m->h_chosen + rows * chains);
    m->h_signal = m->h_norm + rows * chains;
    err = cudaMemcpy(dseeds, seeds, chains * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(m->lambdas, m->host_lambdas.data(), nl * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemset(m->counts, 0, nl * 8);
    if (err == cudaSuccess) err = cudaMemset(m->error, 0, chains * 4);
    if (err == cudaSuccess) err = cudaMemset(m->d_row, 0, 8);
    if (err == cudaSuccess) err = cudaMemset(m->retained, 0, chains * 8);  // the first step reuses nothing
    if (err == cudaSuccess) err = cdet::launch_mcmcmc_init(chains, env, dseeds, m->mt, m->mt_index, m->vert[0], nullptr);
    if (err == cudaSuccess) err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        free_chains(m);
        return cuda_fail(err, "MCMCMC chain initialisation");
    }
    *out = m;
    return CDET_OK;
}

int cdet_mcmcmc_run(cdet_mcmcmc* m, int warmup, int64_t steps, uint64_t* chosen, double* norms, double* signal) {
    if (!m || steps < 0) return fail(CDET_ERR_INVALID, "bad argument");
    if (steps == 0) return CDET_OK;
    DeviceGuard guard(m->ctx->device);
    const int64_t chains = m->chains, e1 = m->cfg.envelope_order + 1, B = m->ring_steps;
    // a half of the ring in flight to the host: its half, first row, rows, first run step
    int pending = -1;
    int64_t pending_row = 0, pending_rows = 0, pending_step = 0;
    int rc = CDET_OK;
    int64_t s = 0;
    while (s < steps && rc == CDET_OK) {
        const int half = static_cast<int>(m->row / B);
        const int64_t first_row = m->row;
        const int64_t n = std::min(steps - s, (half + 1) * B - first_row);
        for (int64_t k = 0; k < n && rc == CDET_OK; ++k) {
            rc = launch_step(m, warmup);
            if (rc == CDET_OK && warmup) {
                ++m->warmup_done;
                if (m->warmup_done % m->cfg.lambda_adapt_interval == 0) rc = mcmcmc_adapt(m, false);
            }
        }
        if (rc != CDET_OK) break;
        cudaError_t err = cudaSuccess;
        const size_t off = static_cast<size_t>(first_row * chains);
        err = cudaMemcpyAsync(m->h_chosen + off, m->d_chosen + off, n * chains * 8, cudaMemcpyDeviceToHost, m->stream);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(m->h_norm + off, m->d_norm + off, n * chains * 8, cudaMemcpyDeviceToHost, m->stream);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(m->h_signal + off * e1, m->d_signal + off * e1, n * chains * e1 * 8,
                                  cudaMemcpyDeviceToHost, m->stream);
        if (err == cudaSuccess) err = cudaEventRecord(m->copied[half], m->stream);
        if (err != cudaSuccess) {
            rc = cuda_fail(err, "MCMCMC step outputs");
            break;
        }
        if (pending >= 0) {
            err = cudaEventSynchronize(m->copied[pending]);
            if (err != cudaSuccess) {
                rc = cuda_fail(err, "MCMCMC step outputs");
                break;
            }
            fold_rows(m, warmup, pending_row, pending_rows, pending_step, chosen, norms, signal);
        }
        pending = half;
        pending_row = first_row;
        pending_rows = n;
        pending_step = s;
        s += n;
        m->row = (first_row + n) % ring_rows(m);
    }
    const cudaError_t err = cudaStreamSynchronize(m->stream);
    if (rc == CDET_OK && err != cudaSuccess) rc = cuda_fail(err, "MCMCMC steps");
    if (rc == CDET_OK && pending >= 0) fold_rows(m, warmup, pending_row, pending_rows, pending_step, chosen, norms, signal);
    if (rc != CDET_OK) {
        // steps launched before the failure advanced the device row: resynchronise
        int64_t device_row = 0;
        if (cudaMemcpy(&device_row, m->d_row, sizeof(device_row), cudaMemcpyDeviceToHost) == cudaSuccess)
            m->row = device_row;
        return rc;
    }
    return chain_errors(m);
}

int cdet_mcmcmc_end_warmup(cdet_mcmcmc* m) {
    if (!m) return fail(CDET_ERR_INVALID, "bad argument");
    DeviceGuard guard(m->ctx->device);
    if (m->warmup_done % m->cfg.lambda_adapt_interval == 0) return CDET_OK;
    return mcmcmc_adapt(m, true);
}

int cdet_mcmcmc_state(const cdet_mcmcmc* m, double* vertices, double* lambdas, uint64_t* rng_state) {
    if (!m) return fail(CDET_ERR_INVALID, "bad argument");
    DeviceGuard guard(m->ctx->device);
    const int env = m->cfg.envelope_order;
    const int64_t chains = m->chains;
    cudaError_t err = cudaDeviceSynchronize();
    if (err == cudaSuccess && vertices)
        err = cudaMemcpy(vertices, m->vert[m->cur], static_cast<size_t>(chains) * env * 4 * 8, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess && lambdas)
        err = cudaMemcpy(lambdas, m->lambdas, static_cast<size_t>(chains) * (env + 1) * 8, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess && rng_state) {
        std::vector<uint64_t> words(static_cast<size_t>(chains) * 312);
        std::vector<int32_t> index(static_cast<size_t>(chains));
        err = cudaMemcpy(words.data(), m->mt, words.size() * 8, cudaMemcpyDeviceToHost);
        if (err == cudaSuccess) err = cudaMemcpy(index.data(), m->mt_index, chains * 4, cudaMemcpyDeviceToHost);
        if (err == cudaSuccess)
            for (int64_t c = 0; c < chains; ++c) {
                for (int i = 0; i < 312; ++i) rng_state[c * 313 + i] = words[static_cast<size_t>(i) * chains + c];
                rng_state[c * 313 + 312] = static_cast<uint64_t>(index[c]);
            }
    }
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC state");
    return CDET_OK;
}

int cdet_mcmcmc_destroy(cdet_mcmcmc* m) {
    if (!m) return CDET_OK;
    DeviceGuard guard(m->ctx->device);
    cudaDeviceSynchronize();
    free_chains(m);
    return CDET_OK;
}

int cdet_mcmcmc_set_green_reuse(cdet_mcmcmc* m, int enable) {
    if (!m) return fail(CDET_ERR_INVALID, "null chains");
    DeviceGuard guard(m->ctx->device);
    cudaError_t err = cudaStreamSynchronize(m->stream);
    if (err == cudaSuccess) err = cudaMemset(m->retained, 0, static_cast<size_t>(m->chains) * 8);
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC Green-pair reuse switch");
    m->green_reuse = enable != 0;
    drop_graphs(m);  // their evaluations were captured with the other setting
    return CDET_OK;
}

int cdet_mcmcmc_launch_count(const cdet_mcmcmc* m, int64_t* launches, int64_t* graph_steps) {
    if (!m) return fail(CDET_ERR_INVALID, "null argument");
    if (launches) *launches = m->kernel_launches;
    if (graph_steps) *graph_steps = m->graph_steps;
    return CDET_OK;
}

int cdet_mcmcmc_set_histogram(cdet_mcmcmc* m, int32_t tau_bins, const double* tau_prob, const double* space_prob,
                              const double* replica_prob) {
    if (!m || !tau_prob || !space_prob || !replica_prob) return fail(CDET_ERR_INVALID, "null argument");
    const int n1 = m->ctx->scalars.n1, n2 = m->ctx->scalars.n2;
    if (tau_bins <= 0 || n1 <= 0 || n2 <= 0) return fail(CDET_ERR_INVALID, "Histogram seed dimensions must be positive");
    const size_t sites = static_cast<size_t>(n1) * n2;
    const size_t nt = static_cast<size_t>(tau_bins) * tau_bins, ns = sites * sites;
    // build_cdfs (mcmcmc_seed.h:190-203): running row sums, the last column set to 1
    auto cdf = [](const double* prob, size_t columns, size_t rows) {
        std::vector<double> out(columns * rows);
        for (size_t r = 0; r < rows; ++r) {
            double cumulative = 0.0;
            for (size_t c = 0; c < columns; ++c) {
                cumulative += prob[r * columns + c];
                out[r * columns + c] = cumulative;
            }
            out[r * columns + columns - 1] = 1.0;
        }
        return out;
    };
    const std::vector<double> tc = cdf(tau_prob, tau_bins, tau_bins), sc = cdf(space_prob, sites, sites),
                              rc = cdf(replica_prob, 2, 2);
    DeviceGuard guard(m->ctx->device);
    auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    const size_t nprob = static_cast<size_t>(m->chains) << m->cfg.envelope_order;
    const size_t bytes = 2 * (up(nt * 8) + up(ns * 8) + up(32)) + up(nprob * 8);
    void* block = nullptr;
    cudaError_t err = cudaMalloc(&block, bytes);
    if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc(MCMCMC histogram seed)");
    char* p = static_cast<char*>(block);
    auto take = [&](size_t b) {
        double* r = reinterpret_cast<double*>(p);
        p += up(b);
        return r;
    };
    double* tp = take(nt * 8);
    double* sp = take(ns * 8);
    double* rp = take(32);
    double* tcd = take(nt * 8);
    double* scd = take(ns * 8);
    double* rcd = take(32);
    double* cprob = take(nprob * 8);
    err = cudaMemcpy(tp, tau_prob, nt * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(sp, space_prob, ns * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(rp, replica_prob, 32, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(tcd, tc.data(), nt * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(scd, sc.data(), ns * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(rcd, rc.data(), 32, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
        cudaFree(block);
        return cuda_fail(err, "MCMCMC histogram seed upload");
    }
    cudaDeviceSynchronize();
    drop_graphs(m);  // graphs of earlier steps use the previous seed kernel
    if (m->hist_block) cudaFree(m->hist_block);
    m->hist_block = block;
    m->tau_bins = tau_bins;
    m->tau_prob = tp;
    m->space_prob = sp;
    m->replica_prob = rp;
    m->tau_cdf = tcd;
    m->space_cdf = scd;
    m->replica_cdf = rcd;
    m->cprob = cprob;
    return CDET_OK;
}

int cdet_mcmcmc_learn_histogram(cdet_context* ctx, const cdet_mcmcmc_config* config,
                                const cdet_histogram_config* histogram, uint64_t base_seed, double* tau_prob,
                                double* space_prob, double* replica_prob, double* total_pair_weight) {
    if (!ctx || !config || !histogram || !tau_prob || !space_prob || !replica_prob)
        return fail(CDET_ERR_INVALID, "null argument");
    const cdet_mcmcmc_config& c = *config;
    const cdet_histogram_config& h = *histogram;
    const int env = c.envelope_order;
    if (c.order_min < 1 || c.order_max < c.order_min || env <= c.order_max || env > cdet::kMcmcmcMaxEnvelope)
        return fail(CDET_ERR_INVALID, "invalid MCMCMC order range or envelope");
    if (h.learning_steps <= 0)
        return fail(CDET_ERR_INVALID, "MCMCMC_SEED_HISTOGRAM_LEARNING_STEPS must be positive for histogram seed");
    const int n1 = ctx->scalars.n1, n2 = ctx->scalars.n2;
    if (h.tau_bins <= 0 || n1 <= 0 || n2 <= 0) return fail(CDET_ERR_INVALID, "Histogram seed dimensions must be positive");
    if (!(h.uniform_mix >= 0.0 && h.uniform_mix <= 1.0))
        return fail(CDET_ERR_INVALID, "MCMCMC_SEED_HISTOGRAM_UNIFORM_MIX must lie in [0, 1]");
    if (h.pseudo_count < 0.0 || !std::isfinite(h.pseudo_count))
        return fail(CDET_ERR_INVALID, "MCMCMC_SEED_HISTOGRAM_PSEUDO_COUNT must be nonnegative and finite");
    for (int k = 0; k < 4; ++k)
        if (!resolve(ctx, k)) return fail(CDET_ERR_STATE, "Green-function tables have not been uploaded");
    DeviceGuard guard(ctx->device);
    // learn_factorized_histogram_seed (mcmcmc_sampler.h:607-664): uniform
    // envelopes from the std::mt19937_64 stream derive_mcmcmc_seed(base,
    // "HISTOSEE"), their all-subset integrands, pair weights accumulated in
    // long double (FactorizedHistogramSeedAccumulator, mcmcmc_seed.h:232-330).
    // The envelopes only consume the generator, so they are drawn first and
    // the integrands evaluated on the GPU in batches.
    auto splitmix = [](uint64_t x) {
        x += 0x9e3779b97f4a7c15ULL;
        x = (x ^ (x >> 30U)) * 0xbf58476d1ce4e5b9ULL;
        x = (x ^ (x >> 27U)) * 0x94d049bb133111ebULL;
        return x ^ (x >> 31U);
    };
    uint64_t mixed = splitmix(base_seed ^ 0x484953544F534545ULL);
    mixed ^= 0x9e3779b97f4a7c15ULL * 1ULL;
    std::mt19937_64 rng(splitmix(mixed));
    std::uniform_real_distribution<double> uniform01(0.0, 1.0);
    const int64_t steps = h.learning_steps;
    std::vector<double> vertices(static_cast<size_t>(steps) * env * 4);
    for (double& x : vertices) x = uniform01(rng);

    const int sites = n1 * n2;
    const int bins = h.tau_bins;
    std::vector<long double> tau_c(static_cast<size_t>(bins) * bins, 0.0L);
    std::vector<long double> space_c(static_cast<size_t>(sites) * sites, 0.0L);
    std::vector<long double> rep_c(4, 0.0L);
    long double total = 0.0L;
    auto index = [](double value, int extent) {
        const int i = static_cast<int>(std::floor(value * static_cast<double>(extent)));
        return i < 0 ? 0 : (i >= extent ? extent - 1 : i);
    };
    double binom[cdet::kMcmcmcMaxEnvelope + 1];
    for (int o = 0; o <= env; ++o) {
        uint64_t b = 1;
        const int k = o < env - o ? o : env - o;
        for (int i = 1; i <= k; ++i) b = b * static_cast<uint64_t>(env - k + i) / static_cast<uint64_t>(i);
        binom[o] = static_cast<double>(b);
    }
    const uint64_t subsets = uint64_t{1} << env;
    // batches of envelopes whose integrands fit 256 MiB
    const int64_t batch = std::max<int64_t>(1, std::min<int64_t>(steps, (int64_t{256} << 20) / (subsets * 8)));
    double* dverts = nullptr;
    double* dvals = nullptr;
    int32_t* dstatus = nullptr;
    cudaError_t err = cudaMalloc(&dverts, static_cast<size_t>(batch) * env * 4 * 8);
    if (err == cudaSuccess) err = cudaMalloc(&dvals, static_cast<size_t>(batch) * subsets * 8);
    if (err == cudaSuccess) err = cudaMalloc(&dstatus, static_cast<size_t>(batch) * 4);
    int rc = err == cudaSuccess ? CDET_OK : cuda_fail(err, "cudaMalloc(histogram learning)");
    std::vector<double> values;
    std::vector<int32_t> status;
    for (int64_t first = 0; rc == CDET_OK && first < steps; first += batch) {
        const int64_t n = std::min<int64_t>(batch, steps - first);
        const double* hv = vertices.data() + static_cast<size_t>(first) * env * 4;
        err = cudaMemcpy(dverts, hv, static_cast<size_t>(n) * env * 4 * 8, cudaMemcpyHostToDevice);
        if (err != cudaSuccess) {
            rc = cuda_fail(err, "histogram learning upload");
            break;
        }
        rc = run(ctx, dverts, nullptr, n, env, 1, dvals, dstatus, nullptr);
        if (rc != CDET_OK) break;
        values.resize(static_cast<size_t>(n) * subsets);
        status.resize(static_cast<size_t>(n));
        err = cudaMemcpy(values.data(), dvals, values.size() * 8, cudaMemcpyDeviceToHost);
        if (err == cudaSuccess) err = cudaMemcpy(status.data(), dstatus, status.size() * 4, cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) {
            rc = cuda_fail(err, "histogram learning values");
            break;
        }
        for (int64_t e = 0; e < n && rc == CDET_OK; ++e) {
            if (status[e] & cdet::kStatusNonFinite) {
                rc = fail(CDET_ERR_VALUE, "Error (all-subset integrand): Value is not finite");
                break;
            }
            const double* v = hv + static_cast<size_t>(e) * env * 4;
            const double* val = values.data() + static_cast<size_t>(e) * subsets;
            for (uint64_t mask = 1; mask < subsets; ++mask) {
                const int order = __builtin_popcountll(mask);
                if (order < c.order_min || order > c.order_max || order < 2) continue;
                const double value = val[mask];
                if (!std::isfinite(value)) continue;
                const long double subset_weight =
                    static_cast<long double>(std::abs(value)) / static_cast<long double>(binom[order]);
                const long double pair_weight = subset_weight / static_cast<long double>(order * (order - 1));
                if (!(pair_weight > 0.0L) || !std::isfinite(static_cast<double>(pair_weight))) continue;
                for (int parent = 0; parent < env; ++parent) {
                    if (!(mask & (uint64_t{1} << parent))) continue;
                    const double* pv = v + 4 * parent;
                    for (int child = 0; child < env; ++child) {
                        if (child == parent || !(mask & (uint64_t{1} << child))) continue;
                        const double* cv = v + 4 * child;
                        tau_c[static_cast<size_t>(index(pv[0], bins)) * bins + index(cv[0], bins)] += pair_weight;
                        const int ps = index(pv[1], n1) * n2 + index(pv[2], n2);
                        const int cs = index(cv[1], n1) * n2 + index(cv[2], n2);
                        space_c[static_cast<size_t>(ps) * sites + cs] += pair_weight;
                        rep_c[index(pv[3], 2) * 2 + index(cv[3], 2)] += pair_weight;
                        total += pair_weight;
                    }
                }
            }
        }
    }
    if (dverts) cudaFree(dverts);
    if (dvals) cudaFree(dvals);
    if (dstatus) cudaFree(dstatus);
    if (rc != CDET_OK) return rc;
    // normalize_rows (mcmcmc_seed.h:288-327)
    auto normalize = [&](const std::vector<long double>& counts, int columns, double* out) {
        const int rows = static_cast<int>(counts.size()) / columns;
        const long double uniform = 1.0L / static_cast<long double>(columns);
        const long double mix = static_cast<long double>(h.uniform_mix);
        const long double pseudo = static_cast<long double>(h.pseudo_count);
        for (int r = 0; r < rows; ++r) {
            long double row_sum = 0.0L;
            for (int k = 0; k < columns; ++k) row_sum += counts[static_cast<size_t>(r) * columns + k];
            const long double denominator = row_sum + pseudo * static_cast<long double>(columns);
            for (int k = 0; k < columns; ++k) {
                long double learned = uniform;
                if (denominator > 0.0L) learned = (counts[static_cast<size_t>(r) * columns + k] + pseudo) / denominator;
                out[static_cast<size_t>(r) * columns + k] = static_cast<double>((1.0L - mix) * learned + mix * uniform);
            }
            double row_total = 0.0;
            for (int k = 0; k < columns; ++k) row_total += out[static_cast<size_t>(r) * columns + k];
            if (row_total > 0.0 && std::isfinite(row_total))
                for (int k = 0; k < columns; ++k) out[static_cast<size_t>(r) * columns + k] /= row_total;
        }
    };
    normalize(tau_c, bins, tau_prob);
    normalize(space_c, sites, space_prob);
    normalize(rep_c, 2, replica_prob);
    if (total_pair_weight) *total_pair_weight = static_cast<double>(total);
    return CDET_OK;
}

int cdet_mcmcmc_result(const cdet_mcmcmc* m, int64_t chain, cdet_mcmcmc_chain_result* out) {
    if (!m || !out || chain < 0 || chain >= m->chains) return fail(CDET_ERR_INVALID, "bad argument");
    *out = m->results[static_cast<size_t>(chain)];
    return CDET_OK;
}

int cdet_mcmcmc_summary(const cdet_mcmcmc* m, int32_t normalization_order, cdet_running_stats* cross_chain,
                        long double* ratios) {
    if (!m || !cross_chain || !ratios) return fail(CDET_ERR_INVALID, "null argument");
    const int omin = m->cfg.order_min, omax = m->cfg.order_max, env = m->cfg.envelope_order;
    if (normalization_order < omin || normalization_order > omax)
        return fail(CDET_ERR_INVALID, "MCMCMC_NORMALIZATION_ORDER must lie inside the measured order range");
    for (int o = 0; o <= env; ++o) {
        cross_chain[o] = cdet_running_stats{};
        ratios[o] = std::numeric_limits<long double>::quiet_NaN();
    }
    // each chain mean is one sample (:1123-1131)
    for (const cdet_mcmcmc_chain_result& r : m->results)
        for (int o = omin; o <= omax; ++o)
            if (r.order_signal_stats[o].count > 0) stats_add(cross_chain[o], r.order_signal_stats[o].mean);
    const long double ref_mean = cross_chain[normalization_order].mean;
    for (int o = omin; o <= omax; ++o)
        ratios[o] = ref_mean == 0.0L ? std::numeric_limits<long double>::quiet_NaN() : cross_chain[o].mean / ref_mean;
    return CDET_OK;
}

int cdet_mcmcmc_estimates(const cdet_mcmcmc* m, double order1_hi, double order1_lo, long double* normalization,
                          long double* normalization_stderr, long double* estimate, long double* estimate_stderr) {
    if (!m || !normalization || !normalization_stderr || !estimate || !estimate_stderr)
        return fail(CDET_ERR_INVALID, "null argument");
    const int omin = m->cfg.order_min, omax = m->cfg.order_max, env = m->cfg.envelope_order;
    if (omin > 1 || omax < 1) return fail(CDET_ERR_INVALID, "the estimates need order 1 inside the measured range");
    std::vector<cdet_running_stats> cross(static_cast<size_t>(env + 1));
    std::vector<long double> ratios(static_cast<size_t>(env + 1));
    int rc = cdet_mcmcmc_summary(m, 1, cross.data(), ratios.data());
    if (rc != CDET_OK) return rc;
    const long double ref_mean = cross[1].mean;
    if (ref_mean == 0.0L || !std::isfinite(static_cast<double>(ref_mean)))
        return fail(CDET_ERR_VALUE, "MCMCMC order-1 de-lambda mean is zero or non-finite");
    const long double ref_stderr = stats_stderr(cross[1]);
    const long double known = static_cast<long double>(order1_hi) + static_cast<long double>(order1_lo);
    const long double constant = known / ref_mean;
    const long double constant_stderr = std::abs(known * ref_stderr / (ref_mean * ref_mean));
    *normalization = constant;
    *normalization_stderr = constant_stderr;
    for (int o = 0; o <= env; ++o) {
        estimate[o] = std::numeric_limits<long double>::quiet_NaN();
        estimate_stderr[o] = std::numeric_limits<long double>::quiet_NaN();
    }
    for (int o = omin; o <= omax; ++o) {
        if (o == 1) {
            estimate[o] = known;  // deterministic
            estimate_stderr[o] = 0.0L;
            continue;
        }
        const long double mean = cross[o].mean;
        const long double se = stats_stderr(cross[o]);
        const long double variance =
            constant * constant * se * se + (mean * constant_stderr) * (mean * constant_stderr);
        estimate[o] = constant * mean;
        estimate_stderr[o] = variance >= 0.0L ? std::sqrt(variance) : std::numeric_limits<long double>::quiet_NaN();
    }
    return CDET_OK;
}

}  // extern "C"

// ------------------------------------------------- checkpoint files ----
namespace {

void write_stats(std::ostream& out, const cdet_running_stats& s) {
    out << s.count << ' ' << std::hexfloat << s.mean << ' ' << s.m2 << std::defaultfloat << '\n';
}

void write_u64s(std::ostream& out, const char* label, const uint64_t* v, int n) {
    out << label << ' ' << n;
    for (int i = 0; i < n; ++i) out << ' ' << v[i];
    out << '\n';
}

void write_doubles(std::ostream& out, const char* label, const double* v, int n) {
    out << label << ' ' << n << std::hexfloat;
    for (int i = 0; i < n; ++i) out << ' ' << v[i];
    out << std::defaultfloat << '\n';
}

// Token reader with the reference's checks and messages
// (load_mcmcmc_chain_checkpoint and its helpers, mcmcmc_sampler.h:717-806, 872-985).
struct CheckpointReader {
    std::ifstream in;
    std::string error;

    bool label(const char* expected) {
        std::string got;
        in >> got;
        if (got != expected) {
            if (error.empty())
                error = "MCMCMC checkpoint expected label " + std::string(expected) + " but found " + got;
            return false;
        }
        return true;
    }
    bool float_token(const char* context, long double* value) {
        std::string token;
        in >> token;
        if (!in) {
            if (error.empty()) error = "Missing MCMCMC checkpoint floating value for " + std::string(context);
            return false;
        }
        errno = 0;
        char* end = nullptr;
        *value = std::strtold(token.c_str(), &end);
        if (end == token.c_str() || *end != '\0' || errno == ERANGE) {
            if (error.empty())
                error = "Could not parse MCMCMC checkpoint floating value for " + std::string(context) + ": " + token;
            return false;
        }
        return true;
    }
    template <typename T>
    bool scalar(const char* name, T* value) {
        if (!label(name)) return false;
        in >> *value;
        return static_cast<bool>(in) || fail_read(name);
    }
    bool fail_read(const char* what) {
        if (error.empty()) error = "Malformed MCMCMC checkpoint field " + std::string(what);
        return false;
    }
    bool stats(cdet_running_stats* s) {
        in >> s->count;
        if (!in) {
            if (error.empty()) error = "Malformed MCMCMC checkpoint running-stat count";
            return false;
        }
        return float_token("running-stat mean", &s->mean) && float_token("running-stat m2", &s->m2);
    }
    bool size_is(size_t got, int want, const char* what) {
        if (got != static_cast<size_t>(want)) {
            if (error.empty())
                error = std::string("MCMCMC checkpoint ") + what + " has " + std::to_string(got) + " entries, expected " +
                        std::to_string(want);
            return false;
        }
        return true;
    }
    bool u64s(const char* name, uint64_t* v, int n) {
        size_t size = 0;
        if (!label(name)) return false;
        in >> size;
        if (!size_is(size, n, name)) return false;
        for (int i = 0; i < n; ++i) in >> v[i];
        return static_cast<bool>(in) || fail_read(name);
    }
    bool doubles(const char* name, double* v, int n) {
        size_t size = 0;
        if (!label(name)) return false;
        in >> size;
        if (!size_is(size, n, name)) return false;
        for (int i = 0; i < n; ++i) {
            long double x = 0.0L;
            if (!float_token(name, &x)) return false;
            v[i] = static_cast<double>(x);
        }
        return true;
    }
};

}  // namespace

extern "C" {

int cdet_write_mcmcmc_checkpoint(const char* path, const cdet_mcmcmc_checkpoint* k) {
    if (!path || !k) return fail(CDET_ERR_INVALID, "null argument");
    const int env = k->envelope_order, e1 = env + 1;
    if (env < 1 || env > CDET_MCMCMC_MAX_ENVELOPE) return fail(CDET_ERR_INVALID, "envelope_order out of range");
    const std::string tmp = std::string(path) + ".tmp";
    {
        std::ofstream out(tmp, std::ios::out | std::ios::trunc);
        if (!out.is_open()) return fail(CDET_ERR_INVALID, "Could not open MCMCMC checkpoint for writing: " + tmp);
        out << std::setprecision(std::numeric_limits<long double>::max_digits10);
        out << "CDET_MCMCMC_CHAIN_CHECKPOINT_V1\n";
        out << "chain_index " << k->chain_index << '\n';
        out << "seed " << k->seed << '\n';
        out << "order_min " << k->order_min << '\n';
        out << "order_max " << k->order_max << '\n';
        out << "envelope_order " << k->envelope_order << '\n';
        out << "normalization_order " << k->normalization_order << '\n';
        out << "lambda_warmup_steps " << k->lambda_warmup_steps << '\n';
        out << "production_steps " << k->production_steps << '\n';
        out << "seed_mode " << k->seed_mode << '\n';
        // std::mt19937_64's operator<<: every word followed by a space, then the position
        out << "rng_state\n";
        for (int i = 0; i < 312; ++i) out << k->rng_state[i] << ' ';
        out << k->rng_state[312] << '\n';
        write_doubles(out, "lambdas", k->lambdas, e1);
        write_u64s(out, "warmup_block_counts", k->warmup_block_counts, e1);
        out << "vertices " << env << '\n' << std::hexfloat;
        for (int i = 0; i < env; ++i)
            out << k->vertices[i][0] << ' ' << k->vertices[i][1] << ' ' << k->vertices[i][2] << ' ' << k->vertices[i][3]
                << '\n';
        out << std::defaultfloat;
        const cdet_mcmcmc_chain_result& r = k->result;
        out << "warmup_proposed_steps " << r.warmup_proposed_steps << '\n';
        out << "warmup_accepted_steps " << r.warmup_accepted_steps << '\n';
        out << "production_proposed_steps " << r.production_proposed_steps << '\n';
        out << "production_accepted_steps " << r.production_accepted_steps << '\n';
        write_u64s(out, "warmup_chosen_counts", r.warmup_chosen_counts, e1);
        write_u64s(out, "production_chosen_counts", r.production_chosen_counts, e1);
        out << "warmup_retained_fraction_stats ";
        write_stats(out, r.warmup_retained_fraction_stats);
        out << "production_retained_fraction_stats ";
        write_stats(out, r.production_retained_fraction_stats);
        out << "order_signal_stats " << e1 << '\n';
        for (int o = 0; o < e1; ++o) write_stats(out, r.order_signal_stats[o]);
        out << "END\n";
        out.close();
        if (!out) return fail(CDET_ERR_INVALID, "Failed while writing MCMCMC checkpoint: " + tmp);
    }
    std::error_code ec;
    std::filesystem::rename(tmp, path, ec);
    if (ec) return fail(CDET_ERR_INVALID, "Could not move MCMCMC checkpoint into place: " + std::string(path));
    return CDET_OK;
}

int cdet_read_mcmcmc_checkpoint(const char* path, cdet_mcmcmc_checkpoint* k) {
    if (!path || !k) return fail(CDET_ERR_INVALID, "null argument");
    *k = cdet_mcmcmc_checkpoint{};
    CheckpointReader rd;
    rd.in.open(path);
    if (!rd.in.is_open()) return fail(CDET_ERR_INVALID, "Could not open MCMCMC checkpoint: " + std::string(path));
    std::string magic;
    rd.in >> magic;
    if (magic != "CDET_MCMCMC_CHAIN_CHECKPOINT_V1")
        return fail(CDET_ERR_INVALID, "Unsupported MCMCMC checkpoint format: " + std::string(path));
    std::string seed_mode;
    bool ok = rd.scalar("chain_index", &k->chain_index) && rd.scalar("seed", &k->seed) &&
              rd.scalar("order_min", &k->order_min) && rd.scalar("order_max", &k->order_max) &&
              rd.scalar("envelope_order", &k->envelope_order) &&
              rd.scalar("normalization_order", &k->normalization_order) &&
              rd.scalar("lambda_warmup_steps", &k->lambda_warmup_steps) &&
              rd.scalar("production_steps", &k->production_steps) && rd.scalar("seed_mode", &seed_mode);
    const int env = k->envelope_order, e1 = env + 1;
    if (ok && (env < 1 || env > CDET_MCMCMC_MAX_ENVELOPE || seed_mode.size() >= sizeof(k->seed_mode)))
        return fail(CDET_ERR_INVALID, "MCMCMC checkpoint envelope_order or seed_mode out of range: " + std::string(path));
    if (ok) {
        std::memcpy(k->seed_mode, seed_mode.c_str(), seed_mode.size() + 1);
        ok = rd.label("rng_state");
        for (int i = 0; ok && i < 313; ++i) ok = static_cast<bool>(rd.in >> k->rng_state[i]) || rd.fail_read("rng_state");
    }
    ok = ok && rd.doubles("lambdas", k->lambdas, e1) && rd.u64s("warmup_block_counts", k->warmup_block_counts, e1);
    if (ok && rd.label("vertices")) {
        size_t count = 0;
        rd.in >> count;
        ok = rd.size_is(count, env, "vertices");
        static const char* const names[4] = {"vertex tau", "vertex x", "vertex y", "vertex replica"};
        for (int i = 0; ok && i < env; ++i)
            for (int j = 0; ok && j < 4; ++j) {
                long double x = 0.0L;
                ok = rd.float_token(names[j], &x);
                k->vertices[i][j] = static_cast<double>(x);
            }
    } else {
        ok = false;
    }
    cdet_mcmcmc_chain_result& r = k->result;
    r.seed = k->seed;
    ok = ok && rd.scalar("warmup_proposed_steps", &r.warmup_proposed_steps) &&
         rd.scalar("warmup_accepted_steps", &r.warmup_accepted_steps) &&
         rd.scalar("production_proposed_steps", &r.production_proposed_steps) &&
         rd.scalar("production_accepted_steps", &r.production_accepted_steps) &&
         rd.u64s("warmup_chosen_counts", r.warmup_chosen_counts, e1) &&
         rd.u64s("production_chosen_counts", r.production_chosen_counts, e1) &&
         rd.label("warmup_retained_fraction_stats") && rd.stats(&r.warmup_retained_fraction_stats) &&
         rd.label("production_retained_fraction_stats") && rd.stats(&r.production_retained_fraction_stats);
    if (ok && rd.label("order_signal_stats")) {
        size_t count = 0;
        rd.in >> count;
        ok = rd.size_is(count, e1, "order_signal_stats");
        for (int o = 0; ok && o < e1; ++o) ok = rd.stats(&r.order_signal_stats[o]);
    } else {
        ok = false;
    }
    if (ok) {
        std::string end;
        rd.in >> end;
        if (end != "END") return fail(CDET_ERR_INVALID, "Malformed MCMCMC checkpoint footer: " + std::string(path));
    }
    if (!ok) return fail(CDET_ERR_INVALID, rd.error.empty() ? "Malformed MCMCMC checkpoint: " + std::string(path) : rd.error);
    return CDET_OK;
}

int cdet_mcmcmc_save_checkpoints(const cdet_mcmcmc* m, const char* dir, const cdet_mcmcmc_run_info* info) {
    if (!m || !dir || !info) return fail(CDET_ERR_INVALID, "null argument");
    const int env = m->cfg.envelope_order, e1 = env + 1;
    const int64_t chains = m->chains;
    std::vector<double> vertices(static_cast<size_t>(chains) * env * 4), lambdas(static_cast<size_t>(chains) * e1);
    std::vector<uint64_t> rng(static_cast<size_t>(chains) * 313), counts(static_cast<size_t>(chains) * e1);
    int rc = cdet_mcmcmc_state(m, vertices.data(), lambdas.data(), rng.data());
    if (rc != CDET_OK) return rc;
    {
        DeviceGuard guard(m->ctx->device);
        const cudaError_t err = cudaMemcpy(counts.data(), m->counts, counts.size() * 8, cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) return cuda_fail(err, "MCMCMC checkpoint state");
    }
    std::error_code ec;
    std::filesystem::create_directories(dir, ec);
    if (ec) return fail(CDET_ERR_INVALID, "Could not create MCMCMC checkpoint directory: " + std::string(dir));
    auto* k = new cdet_mcmcmc_checkpoint;
    for (int64_t c = 0; c < chains; ++c) {
        *k = cdet_mcmcmc_checkpoint{};
        k->chain_index = static_cast<uint64_t>(c);
        k->seed = m->seeds[static_cast<size_t>(c)];
        k->order_min = m->cfg.order_min;
        k->order_max = m->cfg.order_max;
        k->envelope_order = env;
        k->normalization_order = info->normalization_order;
        k->lambda_warmup_steps = info->lambda_warmup_steps;
        k->production_steps = info->production_steps;
        std::snprintf(k->seed_mode, sizeof(k->seed_mode), "%s", m->tau_bins > 0 ? "histogram" : "uniform");
        std::memcpy(k->rng_state, rng.data() + c * 313, 313 * 8);
        std::memcpy(k->lambdas, lambdas.data() + c * e1, e1 * 8);
        std::memcpy(k->warmup_block_counts, counts.data() + c * e1, e1 * 8);
        std::memcpy(k->vertices, vertices.data() + c * env * 4, static_cast<size_t>(env) * 4 * 8);
        k->result = m->results[static_cast<size_t>(c)];
        char name[32];
        std::snprintf(name, sizeof(name), "chain_%06lld.chk", static_cast<long long>(c));
        rc = cdet_write_mcmcmc_checkpoint((std::filesystem::path(dir) / name).string().c_str(), k);
        if (rc != CDET_OK) break;
    }
    delete k;
    return rc;
}

int cdet_mcmcmc_load_checkpoints(cdet_mcmcmc* m, const char* dir, const cdet_mcmcmc_run_info* info, int require,
                                 int64_t* restored) {
    if (!m || !dir || !info) return fail(CDET_ERR_INVALID, "null argument");
    const int env = m->cfg.envelope_order, e1 = env + 1;
    const int64_t chains = m->chains;
    const char* mode = m->tau_bins > 0 ? "histogram" : "uniform";
    std::vector<cdet_mcmcmc_checkpoint> loaded;
    std::vector<int64_t> which;
    for (int64_t c = 0; c < chains; ++c) {
        char name[32];
        std::snprintf(name, sizeof(name), "chain_%06lld.chk", static_cast<long long>(c));
        const std::filesystem::path path = std::filesystem::path(dir) / name;
        if (!std::filesystem::exists(path)) {
            if (require)
                return fail(CDET_ERR_INVALID,
                            "MCMCMC_RESUME=require but checkpoint is missing for chain " + std::to_string(c));
            continue;
        }
        cdet_mcmcmc_checkpoint k;
        const int rc = cdet_read_mcmcmc_checkpoint(path.string().c_str(), &k);
        if (rc != CDET_OK) return rc;
        // load_mcmcmc_chain_checkpoint's settings check (:914-924)
        if (k.chain_index != static_cast<uint64_t>(c) || k.seed != m->seeds[static_cast<size_t>(c)] ||
            k.order_min != m->cfg.order_min || k.order_max != m->cfg.order_max || k.envelope_order != env ||
            k.normalization_order != info->normalization_order ||
            k.lambda_warmup_steps != info->lambda_warmup_steps || k.production_steps > info->production_steps ||
            std::strcmp(k.seed_mode, mode) != 0)
            return fail(CDET_ERR_INVALID, "MCMCMC checkpoint does not match current run settings: " + path.string());
        loaded.push_back(k);
        which.push_back(c);
    }
    if (restored) *restored = static_cast<int64_t>(loaded.size());
    if (loaded.empty()) return CDET_OK;
    const uint64_t wp = loaded[0].result.warmup_proposed_steps, pp = loaded[0].result.production_proposed_steps;
    for (const cdet_mcmcmc_checkpoint& k : loaded)
        if (k.result.warmup_proposed_steps != wp || k.result.production_proposed_steps != pp)
            return fail(CDET_ERR_INVALID, "MCMCMC checkpoints of the batch are at different steps");
    if (static_cast<int64_t>(loaded.size()) != chains && (wp != 0 || pp != 0))
        return fail(CDET_ERR_INVALID, "MCMCMC checkpoints are missing for some chains of a batch that has advanced");
    DeviceGuard guard(m->ctx->device);
    std::vector<double> vertices(static_cast<size_t>(chains) * env * 4);
    std::vector<uint64_t> counts(static_cast<size_t>(chains) * e1), words(static_cast<size_t>(chains) * 312);
    std::vector<int32_t> index(static_cast<size_t>(chains));
    cudaError_t err = cudaDeviceSynchronize();
    if (err == cudaSuccess)
        err = cudaMemcpy(vertices.data(), m->vert[m->cur], vertices.size() * 8, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(counts.data(), m->counts, counts.size() * 8, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(words.data(), m->mt, words.size() * 8, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(index.data(), m->mt_index, index.size() * 4, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC checkpoint restore");
    for (size_t i = 0; i < loaded.size(); ++i) {
        const cdet_mcmcmc_checkpoint& k = loaded[i];
        const int64_t c = which[i];
        if (k.rng_state[312] > 312)
            return fail(CDET_ERR_INVALID, "MCMCMC checkpoint generator position out of range (chain " +
                                              std::to_string(c) + ")");
        std::memcpy(vertices.data() + c * env * 4, k.vertices, static_cast<size_t>(env) * 4 * 8);
        std::memcpy(m->host_lambdas.data() + c * e1, k.lambdas, e1 * 8);
        std::memcpy(counts.data() + c * e1, k.warmup_block_counts, e1 * 8);
        for (int w = 0; w < 312; ++w) words[static_cast<size_t>(w) * chains + c] = k.rng_state[w];
        index[static_cast<size_t>(c)] = static_cast<int32_t>(k.rng_state[312]);
        m->results[static_cast<size_t>(c)] = k.result;
    }
    err = cudaMemcpy(m->vert[m->cur], vertices.data(), vertices.size() * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess)
        err = cudaMemcpy(m->lambdas, m->host_lambdas.data(), m->host_lambdas.size() * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(m->counts, counts.data(), counts.size() * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(m->mt, words.data(), words.size() * 8, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(m->mt_index, index.data(), index.size() * 4, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemset(m->error, 0, chains * 4);
    if (err == cudaSuccess) err = cudaMemset(m->retained, 0, chains * 8);  // restored vertices: no reuse
    if (err != cudaSuccess) return cuda_fail(err, "MCMCMC checkpoint restore");
    m->warmup_done = static_cast<int64_t>(wp);
    return CDET_OK;
}

}  // extern "C"
