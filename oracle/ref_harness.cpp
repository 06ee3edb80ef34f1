// C-ABI harness around the reference's own integrand headers.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled by oracle/Makefile against
// the unmodified reference headers (include/cdet/*.h of
// Boyuan-Shi-0607/cdet-renyi-entanglement-hpc) and the quad-precision Boost
// stand-in in oracle/boost_shim/. The result, oracle/_ref/libcdet_ref.so, is
// used by tests/golden/make_golden.py to produce golden vectors and to pin the
// C restatement in oracle/cdet_oracle.c. Nothing in the product links it.
//
// Every entry point mirrors one reference function:
//   ref_configure          -> the process globals of parameters.h:11-33 and
//                             ztransform_roundoff_config() (precision_config.h:284)
//   ref_build_tables       -> load_data_into_resident_tables<double,double>()
//                             (load_data.h:49-99)
//   ref_get/set_table      -> g_table_{up,down,ordinary_up,ordinary_down}
//                             (parameters.h:81-84)
//   ref_eval_integrand     -> evaluate_cdet_density_integrand_double
//                             (cdet_integrand_evaluator.h:542-560)
//   ref_eval_all_subsets   -> evaluate_cdet_density_all_subset_integrands_double_into
//                             (cdet_integrand_evaluator.h:562-583)
//   ref_mat2pm             -> mat2pm_from_buffer (fast_principle_minors.h:120-246)
//   ref_minors_by_lu       -> determinant_principal_minors_from_buffer (:107-115)
//   ref_ztransform[_all]   -> compute_dp_ztransform[_all_subsets]
//                             (integrand_replica_randomly_sampled.h:226-347)
//   ref_lookup_descriptor  -> prepare_green_lookup_descriptor (g_funcs.h:609-653)
//   ref_green_replica      -> ReplicaGreenCalculator::green_replica_matrix
//                             (replica_free_greens.h:314-331), the direct kernel
//                             solve the Chebyshev accuracy audit compares with.
//   ref_diagonal_order1    -> normalized_log_partition_first_order_density_dd and its
//                             twisted / ordinary parts (diagonal_green_observable.h:237-327)
//   ref_chunk_workflow     -> the chunked load-data stages main.cpp runs one job at a
//                             time (chunked_load_data.h:1530-1570): plan, node
//                             samples, corners, sitepair transforms, diagonal
//                             reduce, validate
//   ref_load_chunks        -> load_chunked_data_into_resident_tables (:1467-1479)
//   ref_mcmcmc_chain       -> the step loop of run_single_mcmcmc_chain
//                             (mcmcmc_sampler.h:994-1088) with the uniform seed or a
//                             FactorizedHistogramSeed of given probabilities
//                             (mcmcmc_seed.h:71-229), no checkpoints, recording every step
//   ref_learn_histogram    -> learn_factorized_histogram_seed (mcmcmc_sampler.h:602-664)
//   ref_mcmcmc_run         -> run_mcmcmc_chains_parallel (mcmcmc_sampler.h:1090-1150):
//                             per-chain MCMCMCChainResult, the cross-chain summary,
//                             optional checkpoint files and resume

#include "cdet/cdet_integrand_evaluator.h"
#include "cdet/chunked_load_data.h"
#include "cdet/diagonal_green_observable.h"
#include "cdet/load_data.h"
#include "cdet/mcmcmc_sampler.h"

#include <cstdint>
#include <cstring>
#include <cmath>
#include <limits>
#include <exception>
#include <string>
#include <thread>
#include <vector>

namespace {

std::string g_last_error;

ResidentGreenFunctionTable& table_slot(int kind) {
    switch (kind) {
        case 0: return g_table_up;
        case 1: return g_table_down;
        case 2: return g_table_ordinary_up;
        case 3: return g_table_ordinary_down;
    }
    throw std::runtime_error("table kind must be 0..3");
}

template <typename F>
int guarded(F&& body) {
    try {
        body();
        return 0;
    } catch (const std::exception& error) {
        g_last_error = error.what();
        return 1;
    }
}

std::vector<UnitVertex> unpack_vertices(const double* unit_vertices, int order) {
    std::vector<UnitVertex> vertices(static_cast<std::size_t>(order));
    for (int i = 0; i < order; ++i) {
        vertices[static_cast<std::size_t>(i)] = UnitVertex{
            unit_vertices[4 * i + 0], unit_vertices[4 * i + 1],
            unit_vertices[4 * i + 2], unit_vertices[4 * i + 3]};
    }
    return vertices;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_last_error.c_str(); }

int ref_configure(int n1, int n2, const char* beta_s, const char* mu_s, const char* u_s,
                  const char* alpha_up_s, const char* alpha_down_s, int pbc_flag,
                  const char* mask_name, int square_radius, int nu, int nv,
                  const char* branch_eps_s, const char* tol_fpm_s, const char* fpm_shift_s,
                  const char* z_eps0_s, const char* z_safety_s) {
    return guarded([&] {
        N1 = n1;
        N2 = n2;
        beta = MP_Real(beta_s);
        mu = MP_Real(mu_s);
        U = MP_Real(u_s);
        alpha_shift_up = MP_Real(alpha_up_s);
        alpha_shift_down = MP_Real(alpha_down_s);
        pbc = pbc_flag != 0;
        subregion_mask_name = mask_name;
        subregion_square_radius = square_radius;
        cheb_nu = nu;
        cheb_nv = nv;
        branch_epsilon = MP_Real(branch_eps_s);
        tol_fpm = MP_Real(tol_fpm_s);
        fpm_global_shift = std::string(fpm_shift_s) == "auto" ? MP_Real(-1) : MP_Real(fpm_shift_s);
        green_table_drop_bits = 0;
        load_data_real_name = "double";
        vector_real_name = "double";
        integrand_real_name = "double";
        load_data_workflow = "resident";
        load_data_calculator_cache = "off";
        mcmcmc_table_backend = "resident";
        table_build_threads = 1;
        internal_integrand_threads = 1;
        load_data_condition_check_mode = LinearSolveConditionCheckMode::Off;
        if (std::string(z_eps0_s) == "auto") {
            ztransform_roundoff_config().set_epsilon0_auto();
        } else {
            ztransform_roundoff_config().set_epsilon0_literal(z_eps0_s);
        }
        ztransform_roundoff_config().set_safety_factor_literal(z_safety_s);
    });
}

int ref_set_precision(const char* vector_real, const char* integrand_real) {
    return guarded([&] {
        vector_real_name = vector_real;
        integrand_real_name = integrand_real;
    });
}

int ref_build_tables(int threads) {
    return guarded([&] {
        table_build_threads = threads;
        load_data_into_resident_tables<double, double>();
    });
}

std::size_t ref_coeff_count() {
    return replica_sitepair_count(N1, N2) * static_cast<std::size_t>(cheb_nu) *
           static_cast<std::size_t>(cheb_nv);
}

std::size_t ref_corner_count() { return replica_sitepair_count(N1, N2); }

int ref_get_table(int kind, double* upper, double* lower, double* upper_corners,
                  double* lower_corners) {
    return guarded([&] {
        const auto& table = std::get<GreenFunctionTableDouble>(table_slot(kind));
        std::memcpy(upper, table.upper_coeffs.data(), table.upper_coeffs.size() * sizeof(double));
        std::memcpy(lower, table.lower_coeffs.data(), table.lower_coeffs.size() * sizeof(double));
        std::memcpy(upper_corners, table.upper_corners.data(),
                    table.upper_corners.size() * sizeof(double));
        std::memcpy(lower_corners, table.lower_corners.data(),
                    table.lower_corners.size() * sizeof(double));
    });
}

int ref_set_table(int kind, const double* upper, const double* lower, const double* upper_corners,
                  const double* lower_corners) {
    return guarded([&] {
        GreenFunctionTableDouble table;
        const std::size_t coeffs = ref_coeff_count();
        const std::size_t corners = ref_corner_count();
        table.upper_coeffs.assign(upper, upper + coeffs);
        table.lower_coeffs.assign(lower, lower + coeffs);
        table.upper_corners.assign(upper_corners, upper_corners + corners);
        table.lower_corners.assign(lower_corners, lower_corners + corners);
        table_slot(kind) = std::move(table);
    });
}

// The same table widened to long double (exactly), for the reference's
// VECTOR_REAL=long_double mode, which requires resident tables of that type.
int ref_set_table_long_double(int kind, const double* upper, const double* lower,
                              const double* upper_corners, const double* lower_corners) {
    return guarded([&] {
        GreenFunctionTableLongDouble table;
        const std::size_t coeffs = ref_coeff_count();
        const std::size_t corners = ref_corner_count();
        table.upper_coeffs.assign(upper, upper + coeffs);
        table.lower_coeffs.assign(lower, lower + coeffs);
        table.upper_corners.assign(upper_corners, upper_corners + corners);
        table.lower_corners.assign(lower_corners, lower_corners + corners);
        table_slot(kind) = std::move(table);
    });
}

int ref_eval_integrand(const double* unit_vertices, int order, double* out) {
    return guarded([&] {
        *out = evaluate_cdet_density_integrand_double(unpack_vertices(unit_vertices, order));
    });
}

// Single-order integrand over a batch of configurations, one std::thread per
// worker with its own contiguous slice (the reference integrand is re-entrant;
// mcmcmc_sampler.h:1101-1110 calls it from one thread per chain). Returns the
// number of configurations that raised.
int ref_eval_integrand_batch(const double* unit_vertices, const int* orders, int batch,
                             int max_order, double* out, int threads) {
    if (threads < 1) threads = 1;
    std::vector<int> failures(static_cast<std::size_t>(threads), 0);
    std::vector<std::thread> workers;
    for (int worker = 0; worker < threads; ++worker) {
        workers.emplace_back([&, worker] {
            const long begin = static_cast<long>(batch) * worker / threads;
            const long end = static_cast<long>(batch) * (worker + 1) / threads;
            for (long c = begin; c < end; ++c) {
                try {
                    out[c] = evaluate_cdet_density_integrand_double(
                        unpack_vertices(unit_vertices + c * max_order * 4, orders[c]));
                } catch (const std::exception&) {
                    out[c] = std::numeric_limits<double>::quiet_NaN();
                    ++failures[static_cast<std::size_t>(worker)];
                }
            }
        });
    }
    for (auto& worker : workers) worker.join();
    int total = 0;
    for (int f : failures) total += f;
    return total;
}

int ref_eval_all_subsets(const double* unit_vertices, int envelope_order, double* out) {
    return guarded([&] {
        std::vector<double> values;
        evaluate_cdet_density_all_subset_integrands_double_into(
            unpack_vertices(unit_vertices, envelope_order), values);
        std::memcpy(out, values.data(), values.size() * sizeof(double));
    });
}

int ref_mat2pm(const double* matrix, int n, double tol, double shift, double* out) {
    return guarded([&] {
        const std::vector<double> pm = mat2pm_from_buffer<double>(matrix, n, tol, shift);
        std::memcpy(out, pm.data(), pm.size() * sizeof(double));
    });
}

int ref_minors_by_lu(const double* matrix, int n, double* out) {
    return guarded([&] {
        const std::vector<double> pm = determinant_principal_minors_from_buffer<double>(matrix, n);
        std::memcpy(out, pm.data(), pm.size() * sizeof(double));
    });
}

double ref_ztransform(const double* up, const double* down, int n, double eps0, double safety) {
    const std::size_t count = (std::size_t{1} << n) - 1;
    const std::vector<double> u(up, up + count), d(down, down + count);
    return compute_dp_ztransform<double>(u, d, n, eps0, safety);
}

int ref_ztransform_all(const double* up, const double* down, int n, double eps0, double safety,
                       double* out) {
    return guarded([&] {
        const std::size_t count = (std::size_t{1} << n) - 1;
        const std::vector<double> u(up, up + count), d(down, down + count);
        const std::vector<double> dp = compute_dp_ztransform_all_subsets<double>(u, d, n, eps0, safety);
        std::memcpy(out, dp.data(), dp.size() * sizeof(double));
    });
}

int ref_lookup_descriptor(int ra, int rb, double tau1, double tau2, int x1, int y1, int x2, int y2,
                          double beta_value, double branch_eps, int nu, int nv, int n1, int n2,
                          int upper, int* use_corner, unsigned long long* index, double* u,
                          double* v) {
    return guarded([&] {
        const auto d = prepare_green_lookup_descriptor<double>(
            ra, rb, tau1, tau2, x1, y1, x2, y2, beta_value, branch_eps, nu, nv, n1, n2, upper != 0);
        *use_corner = d.use_corner ? 1 : 0;
        *index = d.use_corner ? d.corner_index : d.coeff_base_index;
        *u = d.u;
        *v = d.v;
    });
}

int ref_green_replica(int n1, int n2, double beta_value, double mu_value, int pbc_flag,
                      const char* mask_name, int square_radius, int ra, int rb, double tau,
                      double tau_prime, int upper, double* out) {
    return guarded([&] {
        load_data_condition_check_mode = LinearSolveConditionCheckMode::Off;
        const ReplicaSubregionMask mask = parse_subregion_mask(mask_name);
        ReplicaGreenCalculator<double> calculator(n1, n2, beta_value, mu_value, pbc_flag != 0, mask,
                                                  square_radius);
        const auto matrix = calculator.green_replica_matrix(
            ra, rb, tau, tau_prime, upper ? TriangleBranch::Upper : TriangleBranch::Lower);
        const int sites = n1 * n2;
        for (int i = 0; i < sites; ++i) {
            for (int j = 0; j < sites; ++j) {
                out[i * sites + j] = matrix(i, j);
            }
        }
    });
}

// sample_uniform_unit_vertex (mcmcmc_sampler.h:187-190) drawn `count` times
// from std::mt19937_64(seed); out is [count][4] = tau, x, y, replica.
void ref_sample_vertices(unsigned long long seed, int count, double* out) {
    std::mt19937_64 rng(seed);
    for (int i = 0; i < count; ++i) {
        const UnitVertex v = sample_uniform_unit_vertex(rng);
        out[4 * i + 0] = v.tau;
        out[4 * i + 1] = v.x;
        out[4 * i + 2] = v.y;
        out[4 * i + 3] = v.replica;
    }
}

unsigned long long ref_fpm_fallbacks() { return snapshot_cdet_runtime_counters().fpm_fallbacks; }

void ref_reset_counters() { reset_cdet_runtime_counters(); }

// One chain: make_initial_mcmcmc_chain_state, then warmup steps with lambda
// adaptation every adapt_interval steps (and once more for a partial last
// block), then production steps, exactly as run_single_mcmcmc_chain does.
// chosen[k], norms[k]: chosen mask and local normalisation of step k (warmup
// first); signal[p * (envelope + 1) + order]: the raw order signal of
// production step p; vertices_out [envelope][4], lambdas_out [envelope + 1];
// rng_out: the next 8 raw outputs of the chain's generator after the run.
// hist_tau_bins > 0 selects a FactorizedHistogramSeed with the given row
// probabilities (tau [bins][bins], space [S][S], replica [2][2]) instead of the
// uniform seed.
int ref_mcmcmc_chain(int order_min, int order_max, int envelope_order, const double* lambdas_in,
                     int warmup_steps, int adapt_interval, double adapt_rate, int production_steps,
                     unsigned long long seed, int hist_tau_bins, const double* hist_tau, const double* hist_space,
                     const double* hist_replica, unsigned long long* chosen, double* norms, double* signal,
                     double* vertices_out, double* lambdas_out, unsigned long long* rng_out) {
    return guarded([&] {
        MCMCMCConfig config;
        config.order_min = order_min;
        config.order_max = order_max;
        config.envelope_order = envelope_order;
        config.normalization_order = order_min;
        config.lambdas.assign(lambdas_in, lambdas_in + envelope_order + 1);
        config.lambda_warmup_steps = warmup_steps;
        config.lambda_adapt_interval = adapt_interval;
        config.lambda_adapt_rate = adapt_rate;
        config.production_steps = production_steps;
        config.chain_count = 1;
        config.seed_mode = "uniform";
        validate_mcmcmc_config(config);
        MCMCMCChainState state = make_initial_mcmcmc_chain_state(config, 0, seed);
        const MCMCMCMaskPlan plan = make_mcmcmc_mask_plan(config);
        std::shared_ptr<const MCMCMCSeedKernel> kernel;
        if (hist_tau_bins > 0) {
            FactorizedHistogramSeedSettings settings;
            settings.tau_bins = hist_tau_bins;
            settings.N1 = N1;
            settings.N2 = N2;
            const int sites = N1 * N2;
            kernel = std::make_shared<FactorizedHistogramSeed>(
                settings, std::vector<double>(hist_tau, hist_tau + hist_tau_bins * hist_tau_bins),
                std::vector<double>(hist_space, hist_space + sites * sites),
                std::vector<double>(hist_replica, hist_replica + 4));
            config.seed_mode = "histogram";
            config.histogram_learning_steps = 1;
        } else {
            kernel = make_uniform_mcmcmc_seed();
        }
        const MCMCMCSeedKernel& seed_kernel = *kernel;
        MCMCMCStepWorkspace workspace;
        int k = 0;
        for (int step = 0; step < warmup_steps; ++step, ++k) {
            const MCMCMCStepResult r =
                run_mcmcmc_step(state.vertices, config, plan, state.lambdas, seed_kernel, state.rng, workspace);
            state.vertices.swap(workspace.next_vertices);
            chosen[k] = r.chosen_mask;
            norms[k] = r.local_normalization;
            ++state.warmup_block_counts[static_cast<std::size_t>(r.chosen_order)];
            if ((step + 1) % adapt_interval == 0) {
                adapt_mcmcmc_lambdas(state.lambdas, config, state.warmup_block_counts);
                std::fill(state.warmup_block_counts.begin(), state.warmup_block_counts.end(), 0);
            }
        }
        if (warmup_steps % adapt_interval != 0 && mcmcmc_has_pending_warmup_block(state.warmup_block_counts)) {
            adapt_mcmcmc_lambdas(state.lambdas, config, state.warmup_block_counts);
            std::fill(state.warmup_block_counts.begin(), state.warmup_block_counts.end(), 0);
        }
        for (int step = 0; step < production_steps; ++step, ++k) {
            const MCMCMCStepResult r =
                run_mcmcmc_step(state.vertices, config, plan, state.lambdas, seed_kernel, state.rng, workspace);
            state.vertices.swap(workspace.next_vertices);
            chosen[k] = r.chosen_mask;
            norms[k] = r.local_normalization;
            for (int order = 0; order <= envelope_order; ++order)
                signal[static_cast<std::size_t>(step) * (envelope_order + 1) + order] =
                    workspace.order_signal[static_cast<std::size_t>(order)];
        }
        for (int i = 0; i < envelope_order; ++i) {
            vertices_out[4 * i + 0] = state.vertices[static_cast<std::size_t>(i)].tau;
            vertices_out[4 * i + 1] = state.vertices[static_cast<std::size_t>(i)].x;
            vertices_out[4 * i + 2] = state.vertices[static_cast<std::size_t>(i)].y;
            vertices_out[4 * i + 3] = state.vertices[static_cast<std::size_t>(i)].replica;
        }
        for (int order = 0; order <= envelope_order; ++order) lambdas_out[order] = state.lambdas[static_cast<std::size_t>(order)];
        for (int i = 0; i < 8; ++i) rng_out[i] = state.rng();
    });
}

// long double as an exact (hi, lo) pair of doubles (exact for the x87 80-bit format)
static void split_ld(long double x, double* out) {
    const double hi = static_cast<double>(x);
    out[0] = hi;
    out[1] = std::isfinite(hi) ? static_cast<double>(x - static_cast<long double>(hi)) : 0.0;
}

static void put_stats(const RunningStatsLongDouble& st, double* out) {
    out[0] = static_cast<double>(st.count);
    split_ld(st.mean, out + 1);
    split_ld(st.m2, out + 3);
}

// u64_out [chains][5 + 2 (env + 1)]: seed, warmup proposed / accepted,
// production proposed / accepted, warmup then production chosen counts;
// stats_out [chains][3 + env][5]: warmup retained fraction, production
// retained fraction, order signal 0..env as (count, mean hi, lo, m2 hi, lo);
// lambdas_out [chains][env + 1]; cross_out [env + 1][5]; ratios_out [env + 1][2]
// (NaN outside order_min..order_max).
int ref_mcmcmc_run(int order_min, int order_max, int envelope_order, int normalization_order,
                   const double* lambdas_in, int warmup_steps, int adapt_interval, double adapt_rate,
                   int production_steps, int chain_count, unsigned long long base_seed, int hist_tau_bins,
                   const double* hist_tau, const double* hist_space, const double* hist_replica,
                   const char* checkpoint_dir, unsigned long long checkpoint_interval, const char* resume_mode,
                   unsigned long long* u64_out, double* stats_out, double* lambdas_out, double* cross_out,
                   double* ratios_out) {
    return guarded([&] {
        MCMCMCConfig config;
        config.order_min = order_min;
        config.order_max = order_max;
        config.envelope_order = envelope_order;
        config.normalization_order = normalization_order;
        config.lambdas.assign(lambdas_in, lambdas_in + envelope_order + 1);
        config.lambda_warmup_steps = warmup_steps;
        config.lambda_adapt_interval = adapt_interval;
        config.lambda_adapt_rate = adapt_rate;
        config.production_steps = production_steps;
        config.chain_count = chain_count;
        config.base_seed = base_seed;
        config.seed_mode = "uniform";
        std::shared_ptr<const MCMCMCSeedKernel> kernel;
        if (hist_tau_bins > 0) {
            FactorizedHistogramSeedSettings settings;
            settings.tau_bins = hist_tau_bins;
            settings.N1 = N1;
            settings.N2 = N2;
            const int sites = N1 * N2;
            kernel = std::make_shared<FactorizedHistogramSeed>(
                settings, std::vector<double>(hist_tau, hist_tau + hist_tau_bins * hist_tau_bins),
                std::vector<double>(hist_space, hist_space + sites * sites),
                std::vector<double>(hist_replica, hist_replica + 4));
            config.seed_mode = "histogram";
            config.histogram_learning_steps = 1;
            config.histogram_tau_bins = hist_tau_bins;
        } else {
            kernel = make_uniform_mcmcmc_seed();
        }
        if (checkpoint_dir && checkpoint_dir[0]) {
            config.checkpoint_enabled = true;
            config.checkpoint_dir = checkpoint_dir;
            config.checkpoint_interval_steps = checkpoint_interval;
            config.resume_mode = resume_mode;
        }
        const MCMCMCSummary summary = run_mcmcmc_chains_parallel(config, kernel);
        const int e1 = envelope_order + 1;
        for (int c = 0; c < chain_count; ++c) {
            const MCMCMCChainResult& r = summary.chains[static_cast<std::size_t>(c)];
            unsigned long long* u = u64_out + static_cast<std::size_t>(c) * (5 + 2 * e1);
            u[0] = r.seed;
            u[1] = r.warmup_proposed_steps;
            u[2] = r.warmup_accepted_steps;
            u[3] = r.production_proposed_steps;
            u[4] = r.production_accepted_steps;
            for (int o = 0; o < e1; ++o) {
                u[5 + o] = r.warmup_chosen_counts[static_cast<std::size_t>(o)];
                u[5 + e1 + o] = r.production_chosen_counts[static_cast<std::size_t>(o)];
            }
            double* st = stats_out + static_cast<std::size_t>(c) * (2 + e1) * 5;
            put_stats(r.warmup_retained_fraction_stats, st);
            put_stats(r.production_retained_fraction_stats, st + 5);
            for (int o = 0; o < e1; ++o) put_stats(r.order_signal_stats[static_cast<std::size_t>(o)], st + 10 + 5 * o);
            for (int o = 0; o < e1; ++o)
                lambdas_out[static_cast<std::size_t>(c) * e1 + o] = r.final_lambdas[static_cast<std::size_t>(o)];
        }
        for (int o = 0; o < e1; ++o) {
            put_stats(summary.cross_chain_order_signal_stats[static_cast<std::size_t>(o)], cross_out + 5 * o);
            const auto it = summary.ratios_to_normalization.find(o);
            if (it == summary.ratios_to_normalization.end()) {
                ratios_out[2 * o] = ratios_out[2 * o + 1] = std::numeric_limits<double>::quiet_NaN();
            } else {
                split_ld(it->second, ratios_out + 2 * o);
            }
        }
    });
}

int ref_chunk_workflow(const char* dir, int node_chunk_size, int sitepair_chunk_size) {
    return guarded([&] {
        load_data_chunk_dir = dir;
        load_data_node_chunk_size = node_chunk_size;
        load_data_sitepair_chunk_size = sitepair_chunk_size;
        run_chunked_load_data_planner();
        for (const ChunkedNodeJob& job : read_chunked_node_jobs()) {
            setenv("CDET_LOAD_DATA_JOB_INDEX", std::to_string(job.index).c_str(), 1);
            run_chunked_load_data_sample_node_job();
        }
        for (const ChunkedCornerJob& job : read_chunked_corner_jobs()) {
            setenv("CDET_LOAD_DATA_JOB_INDEX", std::to_string(job.index).c_str(), 1);
            run_chunked_load_data_corner_job();
        }
        for (const ChunkedSitepairJob& job : read_chunked_transform_jobs()) {
            setenv("CDET_LOAD_DATA_JOB_INDEX", std::to_string(job.index).c_str(), 1);
            run_chunked_load_data_transform_sitepair_job();
        }
        run_chunked_load_data_diagonal_reduce();
        validate_chunked_load_data_outputs();
    });
}

int ref_load_chunks(const char* dir) {
    return guarded([&] {
        load_data_chunk_dir = dir;
        load_chunked_data_into_resident_tables();
    });
}

// learn_factorized_histogram_seed with these settings; writes the row
// probabilities of the learned seed (tau [bins][bins], space [S][S],
// replica [2][2]) and the total pair weight.
int ref_learn_histogram(int order_min, int order_max, int envelope_order, int learning_steps, int tau_bins,
                        double uniform_mix, double pseudo_count, unsigned long long base_seed, double* tau_out,
                        double* space_out, double* replica_out, double* total_weight_out) {
    return guarded([&] {
        MCMCMCConfig config;
        config.order_min = order_min;
        config.order_max = order_max;
        config.envelope_order = envelope_order;
        config.histogram_learning_steps = learning_steps;
        config.histogram_tau_bins = tau_bins;
        config.histogram_uniform_mix = uniform_mix;
        config.histogram_pseudo_count = pseudo_count;
        config.base_seed = base_seed;
        long double total = 0.0L;
        const auto kernel = learn_factorized_histogram_seed(config, &total);
        const auto& h = dynamic_cast<const FactorizedHistogramSeed&>(*kernel);
        std::copy(h.tau_probabilities().begin(), h.tau_probabilities().end(), tau_out);
        std::copy(h.space_probabilities().begin(), h.space_probabilities().end(), space_out);
        std::copy(h.replica_probabilities().begin(), h.replica_probabilities().end(), replica_out);
        *total_weight_out = static_cast<double>(total);
    });
}

int ref_diagonal_order1(double* out) {
    return guarded([&] {
        const auto& tu = std::get<PiecewiseChebyshevTable<double>>(g_table_up);
        const auto& td = std::get<PiecewiseChebyshevTable<double>>(g_table_down);
        const auto& ou = std::get<PiecewiseChebyshevTable<double>>(g_table_ordinary_up);
        const auto& od = std::get<PiecewiseChebyshevTable<double>>(g_table_ordinary_down);
        out[1] = replica_log_partition_first_order_density_typed<double>(tu, td);
        out[2] = ordinary_log_partition_first_order_density_typed<double>(ou, od);
        const DoubleDouble normalized = normalized_log_partition_first_order_density_dd();
        out[0] = normalized.hi;
        out[3] = normalized.lo;
    });
}

}  // extern "C"
