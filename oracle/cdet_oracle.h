/*
 * CPU restatement of the reference CDet Renyi-2 integrand (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg call this library as the checker. The product path never
 * links or loads it.
 *
 * Built with -ffp-contract=off so that every floating-point operation is the
 * separately rounded IEEE operation the reference performs when compiled for
 * x86-64 (no FMA contraction there; explicit std::fma calls stay fused). The
 * result is the same bits on x86-64 and aarch64 hosts.
 *
 * Pinned against the reference build in oracle/_ref/ through the golden
 * vectors in tests/golden/ (see tests/golden/make_golden.py).
 */
#ifndef CDET_ORACLE_H
#define CDET_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Runtime scalars of one parameter set (IntegrandRuntimeScalars<double>,
 * integrand_replica_randomly_sampled.h:41-51, built by
 * make_integrand_runtime_scalars, :98-119). */
typedef struct oracle_scalars {
    int32_t n1, n2;           /* lattice extents N1, N2 */
    int32_t cheb_nu, cheb_nv; /* Chebyshev coefficients per axis */
    double beta;              /* inverse temperature */
    double u;                 /* Hubbard U */
    double branch_eps;        /* BRANCH_EPSILON */
    double scale;             /* sqrt(U*N1*N2*beta) */
    double diag_up_shift;     /* alpha_down / U (added to the up diagonal) */
    double diag_down_shift;   /* alpha_up / U (added to the down diagonal) */
    double tol_fpm;           /* TOL_FPM */
    double fpm_shift;         /* FPM_GLOBAL_SHIFT, < 0 means auto */
    double z_eps0;            /* ZTRANSFORM_EPSILON0 (2e-16 for double) */
    double z_safety;          /* ZTRANSFORM_SAFETY_FACTOR */
} oracle_scalars;

/* One PiecewiseChebyshevTable<double> (replica_chebyshev_tables.h:25-33). */
typedef struct oracle_table {
    const double* upper_coeffs;
    const double* lower_coeffs;
    const double* upper_corners;
    const double* lower_corners;
} oracle_table;

/* The four resident tables: twisted up, twisted down, ordinary up, ordinary
 * down (parameters.h:81-84). */
typedef struct oracle_tables {
    oracle_table twisted_up, twisted_down, ordinary_up, ordinary_down;
} oracle_tables;

/* Status bits returned per configuration. */
enum {
    ORACLE_OK = 0,
    ORACLE_NONFINITE = 1,   /* the reference throws "Value is not finite" */
    ORACLE_FPM_FALLBACK = 2 /* at least one whole-matrix pivoted-LU fallback */
};

int oracle_lookup_descriptor(int ra, int rb, double tau1, double tau2, int x1, int y1, int x2,
                             int y2, double beta, double branch_eps, int nu, int nv, int n1,
                             int n2, int upper, int* use_corner, uint64_t* index, double* u,
                             double* v);

void oracle_green_pair(const oracle_table* up, const oracle_table* down, int upper,
                       int use_corner, uint64_t index, double u, double v, int nu, int nv,
                       double* up_value, double* down_value);

int oracle_fill_green(const oracle_scalars* s, const oracle_table* up, const oracle_table* down,
                      const double* unit_vertices, int order, int replica_count, double* mat_up,
                      double* mat_down, double* diag_up, double* diag_down);

int oracle_mat2pm(const double* a, int n, double tol, double shift, double* pm_out);
void oracle_minors_by_lu(const double* a, int n, double* pm_out);

double oracle_ztransform(const double* up, const double* down, int n, double eps0,
                         double safety);
void oracle_ztransform_all(const double* up, const double* down, int n, double eps0,
                           double safety, double* dp_out);

void oracle_prefactor_dd(int order, int n1, int n2, int replica_count, double* hi, double* lo);
double oracle_prefactor_ld(int order, int n1, int n2, int replica_count);

int oracle_integrand(const oracle_scalars* s, const oracle_tables* t,
                     const double* unit_vertices, int order, double* value);
int oracle_all_subsets(const oracle_scalars* s, const oracle_tables* t,
                       const double* unit_vertices, int envelope_order, double* values);

/* Batched single-order integrand with `threads` POSIX threads; each thread
 * takes a contiguous slice. unit_vertices is [batch][max_order][4]. */
int oracle_integrand_batch(const oracle_scalars* s, const oracle_tables* t,
                           const double* unit_vertices, const int32_t* orders, int64_t batch,
                           int max_order, double* values, int32_t* status, int threads);
int oracle_all_subsets_batch(const oracle_scalars* s, const oracle_tables* t,
                             const double* unit_vertices, int envelope_order, int64_t batch,
                             double* values, int32_t* status, int threads);

/* Long double evaluation of the same integrand (the same decoded vertices
 * and double (u, v); Chebyshev sums, minors by LU, the connected recursion
 * without the round-off filter and the prefactor in long double): a truth
 * for measuring the FP64 and split forms' errors, compared bit for bit with
 * nothing. Same batch layout as oracle_integrand_batch. */
int oracle_integrand_ld(const oracle_scalars* s, const oracle_tables* t,
                        const double* unit_vertices, int order, double* value);
int oracle_integrand_ld_batch(const oracle_scalars* s, const oracle_tables* t,
                              const double* unit_vertices, const int32_t* orders, int64_t batch,
                              int max_order, double* values, int32_t* status, int threads);
/* The same truth with its parts: parts[0] = the twisted (r = 2) set's
 * value, parts[1] = the ordinary (r = 1) set's, value = parts[0] - 2 parts[1]
 * (each rounded to double from long double); parts[2], parts[3] = each
 * set's magnitude: its prefactor's absolute value times the connected
 * recursion run on absolute values (|dp|[m] = |a[m]| + sum |dp|[s]
 * |a[m \ s]|), the scale of every term that enters the set's value (order
 * 1: the two terms of the singleton). parts may be NULL; the batch form
 * writes parts[c][4]. |twisted| + 2 |ordinary| measures the combine's
 * cancellation, parts[2] + 2 parts[3] the whole recursion's. */
int oracle_integrand_ld_parts(const oracle_scalars* s, const oracle_tables* t,
                              const double* unit_vertices, int order, double* value, double* parts);
int oracle_integrand_ld_parts_batch(const oracle_scalars* s, const oracle_tables* t,
                                    const double* unit_vertices, const int32_t* orders, int64_t batch,
                                    int max_order, double* values, double* parts, int32_t* status,
                                    int threads);

/* Deterministic order-1 diagonal observable (diagonal_green_observable.h:237-327):
 * out[0] = twisted - 2 * ordinary (the normalised first-order coefficient of
 * ln Z_2[A]), out[1] = the twisted (two-replica) part, out[2] = the ordinary
 * part. alpha_up and alpha_down are the double values of ALPHA_UP and
 * ALPHA_DOWN; the shifts are formed from them in double as the reference does.
 * Returns 1 (and writes nothing) when U == 0, which the reference rejects. */
int oracle_diagonal_order1(const oracle_scalars* s, const oracle_tables* t, double alpha_up,
                           double alpha_down, double* out);

/* std::mt19937_64 (the published MT19937-64 generator, libstdc++'s
 * mersenne_twister_engine parameters and seeding). */
typedef struct oracle_mt64 {
    uint64_t mt[312];
    int index;
} oracle_mt64;
void oracle_mt64_seed(oracle_mt64* g, uint64_t seed);
uint64_t oracle_mt64_next(oracle_mt64* g);
/* std::generate_canonical<double, 53>(mt19937_64) as libstdc++ computes it. */
double oracle_canonical(oracle_mt64* g);
/* std::uniform_int_distribution<int>(0, n - 1)(mt19937_64) (libstdc++'s
 * 128-bit nearly-divisionless downscaling). */
int oracle_uniform_int(oracle_mt64* g, int n);

/* One MCMCMC chain with the uniform seed kernel: make_initial_mcmcmc_chain_state,
 * warmup steps with lambda adaptation every adapt_interval steps (and once more
 * for a partial last block), production steps (run_single_mcmcmc_chain,
 * mcmcmc_sampler.h:994-1088, without checkpoints). Outputs as
 * ref_mcmcmc_chain in oracle/ref_harness.cpp: chosen[k], norms[k] per step
 * (warmup first), signal[p * (envelope + 1) + order] per production step,
 * vertices_out [envelope][4], lambdas_out [envelope + 1], rng_out the next 8
 * raw generator outputs. Returns 0, or 1 when the integrand is not finite, 2
 * when a local normalisation is zero or not finite (the reference throws). */
int oracle_mcmcmc_chain(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max,
                        int envelope, const double* lambdas, int warmup, int adapt_interval, double adapt_rate,
                        int production, uint64_t seed, uint64_t* chosen, double* norms, double* signal,
                        double* vertices_out, double* lambdas_out, uint64_t* rng_out);

/* The same with the FactorizedHistogramSeed (mcmcmc_seed.h:71-229) of the
 * given row probabilities: tau [tau_bins][tau_bins], space [S][S] (S = N1 N2),
 * replica [2][2]; the conditional generation probabilities
 * (mcmcmc_sampler.h:252-335) weight the fluxes. Returns 4 when a seed density
 * is negative or not finite. */
int oracle_mcmcmc_chain_hist(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max,
                             int envelope, const double* lambdas, int warmup, int adapt_interval, double adapt_rate,
                             int production, uint64_t seed, int tau_bins, const double* tau_prob,
                             const double* space_prob, const double* replica_prob, uint64_t* chosen, double* norms,
                             double* signal, double* vertices_out, double* lambdas_out, uint64_t* rng_out);

/* learn_factorized_histogram_seed (mcmcmc_sampler.h:602-664): the learned row
 * probabilities (long double accumulation, as the reference) and the total
 * pair weight. */
int oracle_learn_histogram(const oracle_scalars* s, const oracle_tables* t, int order_min, int order_max,
                           int envelope, int learning_steps, int tau_bins, double uniform_mix, double pseudo_count,
                           uint64_t base_seed, double* tau_out, double* space_out, double* replica_out,
                           double* total_weight_out);

#ifdef __cplusplus
}
#endif

#endif
