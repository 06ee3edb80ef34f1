// cdet_gb300.hpp - C++20 drop-in adapter over the C ABI in cdet_gb300.h.
//
// Gives the reference's MCMCMC driver the two integrand entry points it calls,
// with the reference's signatures, argument meaning and exceptions:
//
//   double evaluate_cdet_density_integrand_double(const std::vector<UnitVertex>&)
//       (include/cdet/cdet_integrand_evaluator.h:542-560)
//   void evaluate_cdet_density_all_subset_integrands_double_into(
//       const std::vector<UnitVertex>&, std::vector<double>&)        (:562-583)
//   std::vector<double> evaluate_cdet_density_all_subset_integrands_double(...)  (:585-590)
//
// The reference reads its parameters and tables from process globals
// (parameters.h:11-91); here one Integrand object holds them on the GPU and
// install() makes it the one the free functions use. A driver that evaluates
// many proposals per step calls Integrand::evaluate_batch instead.
//
// McmcmcChains keeps a batch of the reference's MCMCMC chains on the GPU
// (run_single_mcmcmc_chain, mcmcmc_sampler.h:994-1088, for every chain at
// once): seeds, lambdas, warmup with lambda adaptation, production, the
// factorized histogram seed, the per-chain MCMCMCChainResult, the cross-chain
// summary and estimates, and the reference's V1 checkpoint files.
#pragma once

#include "cdet_gb300.h"

#include <algorithm>
#include <cstdint>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace cdet_gb300 {

// UnitVertex (cdet_integrand_evaluator.h:16-21): coordinates in [0, 1).
struct UnitVertex {
    double tau = 0.0;
    double x = 0.0;
    double y = 0.0;
    double replica = 0.0;
};

// One PiecewiseChebyshevTable<double> (replica_chebyshev_tables.h:25-33).
struct TableView {
    const std::vector<double>* upper_coeffs = nullptr;
    const std::vector<double>* lower_coeffs = nullptr;
    const std::vector<double>* upper_corners = nullptr;
    const std::vector<double>* lower_corners = nullptr;
};

inline void check(int rc) {
    if (rc != CDET_OK) throw std::runtime_error(cdet_last_error());
}

class Integrand {
public:
    Integrand(const cdet_runtime_scalars& scalars, int device = 0) {
        cdet_context* ctx = nullptr;
        check(cdet_create(&scalars, device, &ctx));
        ctx_.reset(ctx);
    }

    // Copies one of the four tables (kind = cdet_table_kind) to the GPU.
    void upload(int kind, const TableView& t) {
        const cdet_table_view view{t.upper_coeffs->data(), t.lower_coeffs->data(),
                                   t.upper_corners->data(), t.lower_corners->data()};
        check(cdet_upload_table(ctx_.get(), kind, &view, t.upper_coeffs->size(),
                                t.upper_corners->size()));
    }

    // The reference's ALPHA_UP == ALPHA_DOWN sharing (load_data.h:70-91).
    void alias(int kind, int source_kind) { check(cdet_alias_table(ctx_.get(), kind, source_kind)); }

    void set_assembly(int mode) { check(cdet_set_assembly(ctx_.get(), mode)); }

    double integrand(const std::vector<UnitVertex>& vertices) {
        const int order = static_cast<int>(vertices.size());
        if (order <= 0) throw std::runtime_error("The replica integrand is defined only for order >= 1");
        double value = 0.0;
        int32_t status = 0;
        const int32_t orders = order;
        const int rc = cdet_integrand_host(ctx_.get(), &vertices[0].tau, &orders, 1, order, &value, &status);
        if (status & CDET_CONFIG_NONFINITE) throw std::runtime_error("Error (integrand): Value is not finite");
        if (status & CDET_CONFIG_BAD_INPUT) throw std::runtime_error("Error (integrand): vertex coordinates rejected");
        check(rc);
        return value;
    }

    void all_subsets_into(const std::vector<UnitVertex>& vertices, std::vector<double>& values) {
        const int envelope = static_cast<int>(vertices.size());
        if (envelope <= 1)
            throw std::runtime_error("The all-subset replica integrand is defined only for envelope order >= 2");
        values.resize(std::size_t{1} << envelope);
        int32_t status = 0;
        const int rc = cdet_all_subsets_host(ctx_.get(), &vertices[0].tau, envelope, 1, values.data(), &status);
        if (status & CDET_CONFIG_NONFINITE)
            throw std::runtime_error("Error (all-subset integrand): Value is not finite");
        if (status & CDET_CONFIG_BAD_INPUT)
            throw std::runtime_error("Error (all-subset integrand): vertex coordinates rejected");
        check(rc);
    }

    // Many configurations at once: vertices [batch][max_order], orders [batch].
    void evaluate_batch(const std::vector<UnitVertex>& vertices, const std::vector<int32_t>& orders,
                        int max_order, std::vector<double>& values, std::vector<int32_t>& status) {
        const int64_t batch = static_cast<int64_t>(orders.size());
        values.resize(orders.size());
        status.resize(orders.size());
        const int rc = cdet_integrand_host(ctx_.get(), &vertices[0].tau, orders.data(), batch, max_order,
                                           values.data(), status.data());
        if (rc != CDET_OK && rc != CDET_ERR_VALUE) check(rc);
    }

    // Deterministic order-1 diagonal observable of the uploaded tables
    // (diagonal_observable_density_dd, diagonal_green_observable.h:357-366):
    // the normalised coefficient twisted - 2 ordinary. The reference reads
    // ALPHA_UP and ALPHA_DOWN from its globals; pass their double values.
    double diagonal_observable_density(double alpha_up, double alpha_down) {
        double out[3] = {0.0, 0.0, 0.0};
        check(cdet_diagonal_order1_density(ctx_.get(), alpha_up, alpha_down, out));
        return out[0];
    }

    // Loads the four tables of a directory written by the reference's chunked
    // load-data workflow (in place of load_chunked_data_into_resident_tables,
    // chunked_load_data.h:1372-1511); returns its precomputed order-1 value
    // (double-double hi, lo) when the directory has one.
    std::optional<std::pair<double, double>> load_chunks(const std::string& dir) {
        double order1[2] = {0.0, 0.0};
        check(cdet_load_chunks(ctx_.get(), dir.c_str(), order1));
        if (order1[0] != order1[0]) return std::nullopt;  // NaN: not in the directory
        return std::make_pair(order1[0], order1[1]);
    }

    cdet_context* context() const { return ctx_.get(); }

    // Makes this object the one the free functions below use.
    void install() { current() = this; }

    static Integrand*& current() {
        static Integrand* instance = nullptr;
        return instance;
    }

private:
    struct Deleter {
        void operator()(cdet_context* c) const { cdet_destroy(c); }
    };
    std::unique_ptr<cdet_context, Deleter> ctx_;
};

static_assert(sizeof(UnitVertex) == 4 * sizeof(double), "UnitVertex is passed as [order][4] doubles");

// Cross-chain statistics and ratios (run_mcmcmc_chains_parallel's summary).
struct McmcmcSummary {
    std::vector<cdet_running_stats> cross_chain;  // index = order
    std::vector<long double> ratios;              // to the normalisation order
};

// Absolute estimates normalised by the deterministic order-1 value
// (print_mcmcmc_summary, main.cpp:831-870).
struct McmcmcEstimates {
    long double normalization = 0.0L, normalization_stderr = 0.0L;
    std::vector<long double> estimate, stderr_;  // index = order
};

// A batch of MCMCMC chains resident on the GPU; see the cdet_mcmcmc_* entry
// points of cdet_gb300.h for the meaning of each call.
class McmcmcChains {
public:
    // seeds: one per chain (derive_mcmcmc_seed(base_seed, stream tag, chain) for
    // the reference's chains); lambdas: MCMCMC_LAMBDAS, envelope_order + 1 entries.
    McmcmcChains(const Integrand& integrand, const cdet_mcmcmc_config& config, const std::vector<uint64_t>& seeds,
                 const std::vector<double>& lambdas)
        : config_(config) {
        if (lambdas.size() != static_cast<std::size_t>(config.envelope_order) + 1)
            throw std::runtime_error("MCMCMC_LAMBDAS needs envelope_order + 1 entries");
        cdet_mcmcmc* m = nullptr;
        check(cdet_mcmcmc_create(integrand.context(), &config, static_cast<int64_t>(seeds.size()), seeds.data(),
                                 lambdas.data(), &m));
        m_.reset(m);
        chains_ = static_cast<int64_t>(seeds.size());
    }

    // MCMCMC_SEED_MODE=histogram with the given row probabilities.
    void set_histogram(int tau_bins, const std::vector<double>& tau, const std::vector<double>& space,
                       const std::vector<double>& replica) {
        check(cdet_mcmcmc_set_histogram(m_.get(), tau_bins, tau.data(), space.data(), replica.data()));
    }

    // learn_factorized_histogram_seed (mcmcmc_sampler.h:607-664) on the integrand's tables.
    static void learn_histogram(const Integrand& integrand, const cdet_mcmcmc_config& config,
                                const cdet_histogram_config& histogram, uint64_t base_seed, int sites,
                                std::vector<double>& tau, std::vector<double>& space, std::vector<double>& replica,
                                double* total_pair_weight = nullptr) {
        tau.assign(static_cast<std::size_t>(histogram.tau_bins) * histogram.tau_bins, 0.0);
        space.assign(static_cast<std::size_t>(sites) * sites, 0.0);
        replica.assign(4, 0.0);
        check(cdet_mcmcmc_learn_histogram(integrand.context(), &config, &histogram, base_seed, tau.data(),
                                          space.data(), replica.data(), total_pair_weight));
    }

    void run(bool warmup, int64_t steps) { check(cdet_mcmcmc_run(m_.get(), warmup ? 1 : 0, steps, nullptr, nullptr, nullptr)); }
    void end_warmup() { check(cdet_mcmcmc_end_warmup(m_.get())); }

    cdet_mcmcmc_chain_result result(int64_t chain) const {
        cdet_mcmcmc_chain_result r{};
        check(cdet_mcmcmc_result(m_.get(), chain, &r));
        return r;
    }

    McmcmcSummary summary(int normalization_order) const {
        McmcmcSummary s;
        s.cross_chain.resize(static_cast<std::size_t>(config_.envelope_order) + 1);
        s.ratios.resize(s.cross_chain.size());
        check(cdet_mcmcmc_summary(m_.get(), normalization_order, s.cross_chain.data(), s.ratios.data()));
        return s;
    }

    McmcmcEstimates estimates(double order1_hi, double order1_lo = 0.0) const {
        McmcmcEstimates e;
        e.estimate.resize(static_cast<std::size_t>(config_.envelope_order) + 1);
        e.stderr_.resize(e.estimate.size());
        check(cdet_mcmcmc_estimates(m_.get(), order1_hi, order1_lo, &e.normalization, &e.normalization_stderr,
                                    e.estimate.data(), e.stderr_.data()));
        return e;
    }

    // Vertices [chain][envelope][4], lambdas [chain][envelope + 1] and the
    // generator states [chain][313] (words, then the position).
    void state(std::vector<double>& vertices, std::vector<double>& lambdas, std::vector<uint64_t>& rng) const {
        const std::size_t c = static_cast<std::size_t>(chains_), env = static_cast<std::size_t>(config_.envelope_order);
        vertices.resize(c * env * 4);
        lambdas.resize(c * (env + 1));
        rng.resize(c * 313);
        check(cdet_mcmcmc_state(m_.get(), vertices.data(), lambdas.data(), rng.data()));
    }

    void save_checkpoints(const std::string& dir, const cdet_mcmcmc_run_info& info) const {
        check(cdet_mcmcmc_save_checkpoints(m_.get(), dir.c_str(), &info));
    }

    // MCMCMC_RESUME=auto (require = false) or require; returns the chains restored.
    int64_t load_checkpoints(const std::string& dir, const cdet_mcmcmc_run_info& info, bool require) {
        int64_t restored = 0;
        check(cdet_mcmcmc_load_checkpoints(m_.get(), dir.c_str(), &info, require ? 1 : 0, &restored));
        return restored;
    }

    // run_single_mcmcmc_chain's loop for the whole batch: the remaining warmup
    // steps, the adaptation of a partial last block, the remaining production
    // steps; with a directory, checkpoints whenever the completed steps reach
    // a multiple of interval (if > 0) and at the end.
    void run_to(const cdet_mcmcmc_run_info& info, const std::string& checkpoint_dir = "", uint64_t interval = 0) {
        const cdet_mcmcmc_chain_result r0 = result(0);
        uint64_t done = r0.warmup_proposed_steps + r0.production_proposed_steps;
        auto advance = [&](uint64_t steps, bool warmup) {
            while (steps > 0) {
                uint64_t chunk = steps;
                if (!checkpoint_dir.empty() && interval > 0) chunk = std::min<uint64_t>(chunk, interval - done % interval);
                run(warmup, static_cast<int64_t>(chunk));
                done += chunk;
                steps -= chunk;
                if (!checkpoint_dir.empty() && interval > 0 && done % interval == 0) save_checkpoints(checkpoint_dir, info);
            }
        };
        const uint64_t warm = static_cast<uint64_t>(info.lambda_warmup_steps);
        const uint64_t prod = static_cast<uint64_t>(info.production_steps);
        advance(warm > r0.warmup_proposed_steps ? warm - r0.warmup_proposed_steps : 0, true);
        end_warmup();
        advance(prod > r0.production_proposed_steps ? prod - r0.production_proposed_steps : 0, false);
        if (!checkpoint_dir.empty()) save_checkpoints(checkpoint_dir, info);
    }

    int64_t chains() const { return chains_; }

private:
    struct Deleter {
        void operator()(cdet_mcmcmc* m) const { cdet_mcmcmc_destroy(m); }
    };
    std::unique_ptr<cdet_mcmcmc, Deleter> m_;
    cdet_mcmcmc_config config_{};
    int64_t chains_ = 0;
};

// One CDET_MCMCMC_CHAIN_CHECKPOINT_V1 file (no GPU needed).
inline cdet_mcmcmc_checkpoint read_mcmcmc_checkpoint(const std::string& path) {
    cdet_mcmcmc_checkpoint k{};
    check(cdet_read_mcmcmc_checkpoint(path.c_str(), &k));
    return k;
}

inline void write_mcmcmc_checkpoint(const std::string& path, const cdet_mcmcmc_checkpoint& k) {
    check(cdet_write_mcmcmc_checkpoint(path.c_str(), &k));
}

inline Integrand& installed() {
    Integrand* p = Integrand::current();
    if (!p) throw std::runtime_error("Green-function tables have not been uploaded (no Integrand installed)");
    return *p;
}

inline double evaluate_cdet_density_integrand_double(const std::vector<UnitVertex>& vertices) {
    return installed().integrand(vertices);
}

inline void evaluate_cdet_density_all_subset_integrands_double_into(const std::vector<UnitVertex>& vertices,
                                                                    std::vector<double>& values) {
    installed().all_subsets_into(vertices, values);
}

inline std::vector<double> evaluate_cdet_density_all_subset_integrands_double(
    const std::vector<UnitVertex>& vertices) {
    std::vector<double> values;
    evaluate_cdet_density_all_subset_integrands_double_into(vertices, values);
    return values;
}

}  // namespace cdet_gb300
