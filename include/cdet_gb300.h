/*
 * cdet_gb300.h - C ABI of the GB300 (sm_103a) CDet Renyi-2 integrand.
 *
 * Drop-in boundary for the integrand of Boyuan-Shi-0607/cdet-renyi-entanglement-hpc.
 * Each declaration names the reference interface it replaces (paths are
 * relative to that project). All arguments are plain pointers and sizes; the
 * library owns no host state beyond the opaque context. Errors are status
 * codes (the reference throws std::runtime_error) with the message available
 * from cdet_last_error(); include/cdet_gb300.hpp re-throws them with the
 * reference's messages.
 *
 * Numerics: every kernel evaluates the reference's FP64 operations in the
 * reference's order without contraction, so on equal inputs the values equal
 * the reference compiled for x86-64 bit for bit.
 */
#ifndef CDET_GB300_H
#define CDET_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CDET_GB300_ABI_VERSION 1

/* Return codes of every entry point. */
enum cdet_result {
    CDET_OK = 0,
    CDET_ERR_INVALID = 1, /* bad argument: null pointer, size or order out of range */
    CDET_ERR_STATE = 2,   /* a table the call needs is not uploaded */
    CDET_ERR_CUDA = 3,    /* a CUDA runtime call failed; see cdet_last_error() */
    CDET_ERR_VALUE = 4    /* at least one configuration is flagged in `status` */
};

/* Per-configuration status bits written to the `status` arrays. */
enum cdet_config_status {
    CDET_CONFIG_NONFINITE = 1,    /* integrand_replica_randomly_sampled.h:543-545, 842-844, 873-875 */
    CDET_CONFIG_FPM_FALLBACK = 2, /* fast_principle_minors.h:180-186 (counted, not an error) */
    CDET_CONFIG_BAD_INPUT = 4     /* order outside [1, 24], or a coordinate the decode rejects */
};

/* Table kinds: the four resident tables g_table_up, g_table_down,
 * g_table_ordinary_up, g_table_ordinary_down (include/cdet/parameters.h:81-84). */
enum cdet_table_kind {
    CDET_TWISTED_UP = 0,
    CDET_TWISTED_DOWN = 1,
    CDET_ORDINARY_UP = 2,
    CDET_ORDINARY_DOWN = 3
};

/* IntegrandRuntimeScalars<double> (integrand_replica_randomly_sampled.h:41-51)
 * as built by make_integrand_runtime_scalars (:98-119) and the z-transform
 * roundoff filter of ztransform_roundoff_config() (precision_config.h:208-287). */
typedef struct cdet_runtime_scalars {
    int32_t n1, n2;            /* N1, N2 */
    int32_t cheb_nu, cheb_nv;  /* CHEB_NU, CHEB_NV (coefficients per axis) */
    double beta;               /* beta */
    double u;                  /* U */
    double branch_eps;         /* BRANCH_EPSILON */
    double scale;              /* sqrt(U * N1 * N2 * beta) */
    double diag_up_shift;      /* ALPHA_DOWN / U, added to the spin-up diagonal */
    double diag_down_shift;    /* ALPHA_UP / U, added to the spin-down diagonal */
    double tol_fpm;            /* TOL_FPM */
    double fpm_shift;          /* FPM_GLOBAL_SHIFT; negative means auto (max|A| / n^2) */
    double z_eps0;             /* ZTRANSFORM_EPSILON0 (2e-16 when auto) */
    double z_safety;           /* ZTRANSFORM_SAFETY_FACTOR (0 disables the filter) */
} cdet_runtime_scalars;

/* One PiecewiseChebyshevTable<double> (replica_chebyshev_tables.h:25-33):
 * coefficients [4*S*S][nu][nv] per branch and corners [4*S*S], S = N1*N2,
 * indexed by replica_sitepair_index (replica_chebyshev_tables.h:365-400). */
typedef struct cdet_table_view {
    const double* upper_coeffs;
    const double* lower_coeffs;
    const double* upper_corners;
    const double* lower_corners;
} cdet_table_view;

typedef struct cdet_context cdet_context;

/* Creates a context on CUDA device `device` for one parameter set. Replaces
 * the process globals the integrand reads (include/cdet/parameters.h:11-33)
 * and the cached scalars of cached_integrand_runtime_scalars_for_real
 * (cdet_integrand_evaluator.h:73-96). */
int cdet_create(const cdet_runtime_scalars* scalars, int device, cdet_context** out);

/* Releases the context and every device buffer it owns. */
void cdet_destroy(cdet_context* ctx);

/* Copies one table from host memory into HBM. Replaces the assignment of
 * g_table_* by load_data_into_resident_tables (load_data.h:49-99).
 * coeff_count = 4*S*S*nu*nv, corner_count = 4*S*S. */
int cdet_upload_table(cdet_context* ctx, int kind, const cdet_table_view* host_table,
                      size_t coeff_count, size_t corner_count);

/* Uses a table that already lives in device memory (no copy); the caller
 * keeps it alive. Same layout and sizes as cdet_upload_table. */
int cdet_bind_device_table(cdet_context* ctx, int kind, const cdet_table_view* device_table,
                           size_t coeff_count, size_t corner_count);

/* Makes `kind` share the table of `source_kind`, as load_data does when
 * ALPHA_UP == ALPHA_DOWN (load_data.h:70-91). When a set's up and down
 * tables are shared and the two diagonal shifts are equal the spin-down
 * Green matrix equals the spin-up one and is not evaluated twice. */
int cdet_alias_table(cdet_context* ctx, int kind, int source_kind);

/* Sizes the device scratch for batches up to `batch` configurations of
 * order (or envelope) up to `max_order`, so that later calls of that size
 * allocate nothing. */
int cdet_reserve(cdet_context* ctx, int64_t batch, int max_order);

/* Batched single-order integrand on device buffers, asynchronous on `stream`
 * (a cudaStream_t; NULL = legacy default stream). For configuration c with
 * order orders[c] (1..max_order), vertices[c][i][0..3] hold the unit-cube
 * coordinates tau, x, y, replica of vertex i. values[c] receives
 * evaluate_cdet_density_integrand_double (cdet_integrand_evaluator.h:542-560);
 * status[c] receives cdet_config_status bits (zeroed by the call). */
int cdet_integrand_device(cdet_context* ctx, const double* vertices, const int32_t* orders,
                          int64_t batch, int max_order, double* values, int32_t* status,
                          void* stream);

/* Batched all-subset integrand on device buffers, asynchronous on `stream`.
 * values[c][mask] (2^envelope_order per configuration, values[c][0] = 0)
 * receives evaluate_cdet_density_all_subset_integrands_double_into
 * (cdet_integrand_evaluator.h:562-583). envelope_order is 2..24. */
int cdet_all_subsets_device(cdet_context* ctx, const double* vertices, int envelope_order,
                            int64_t batch, double* values, int32_t* status, void* stream);

/* No counterpart in the reference. The single-order FP64 integrand of
 * cdet_integrand_device (same values bit for bit), for callers that cannot
 * let the library allocate device memory: a process that has given HBM to
 * its tables or to a pool allocator of its own, where a library's
 * cudaMalloc would take memory the owner has not accounted for. Its scratch
 * is a fixed 64 MiB array of device memory held by every GPU that loads the
 * library. A batch whose regions leave room for fewer than eight warps of
 * minors workspace is rejected with CDET_ERR_INVALID and a message; the
 * largest batches accepted, by maximum order:
 *
 *   order      1..4         5      6      7      8      9     10
 *   batch   >= 57,823  33,662 19,712 11,360  6,368  3,456  1,824
 *   order     11     12     13     14     15    >= 16
 *   batch  1,774    928    448    224     32   refused
 *
 * (near these limits the minors run on few warps). Tables must already be
 * on the device (cdet_bind_device_table allocates nothing). The first call
 * on a device looks up the array's device address, so it should come before
 * any stream capture; the address is cached for the life of the process
 * (the device's primary context must not be reset in between). All calls
 * share the array: calls that overlap on the GPU race, so keep them on one
 * stream or order them. Always the FP64 assembly, whatever the context's
 * assembly setting (the split assembly needs allocations). */
int cdet_integrand_device_noalloc(cdet_context* ctx, const double* vertices, const int32_t* orders,
                                  int64_t batch, int max_order, double* values, int32_t* status,
                                  void* stream);

/* Host-buffer forms of the two calls above: copy the inputs in, evaluate,
 * copy the results out, and return when they are in host memory. Pinned
 * host buffers make the copies asynchronous DMA. Returns CDET_ERR_VALUE when
 * any configuration is flagged NONFINITE or BAD_INPUT. */
int cdet_integrand_host(cdet_context* ctx, const double* vertices, const int32_t* orders,
                        int64_t batch, int max_order, double* values, int32_t* status);
int cdet_all_subsets_host(cdet_context* ctx, const double* vertices, int envelope_order,
                          int64_t batch, double* values, int32_t* status);

/* Deterministic order-1 diagonal observable from the bound tables: out[0] =
 * the normalised first-order coefficient of ln Z_2[A] (twisted - 2 ordinary;
 * normalized_log_partition_first_order_density_dd and
 * diagonal_observable_density_dd, diagonal_green_observable.h:305-366),
 * out[1] = the twisted part (replica_log_partition_first_order_density_typed,
 * :237-273), out[2] = the ordinary part (:275-303). alpha_up and alpha_down
 * are ALPHA_UP and ALPHA_DOWN as doubles (the shifts are formed from them in
 * double, as the reference does). Bit-identical to the reference's double
 * build. Blocking; fails with CDET_ERR_INVALID when U == 0 (the reference
 * throws "The diagonal observable is undefined for U = 0"). */
int cdet_diagonal_order1_density(cdet_context* ctx, double alpha_up, double alpha_down, double* out);

/* Loads the four tables from a chunked load-data directory written by the
 * reference's chunk workflow (chunked_load_data.h: manifest.txt, READY,
 * transform_jobs.tsv, coeffs/<kind>/<branch>/sitepairs_<begin>_<end>.bin,
 * corners/<kind>/<branch>.bin), replacing load_chunked_data_into_resident_tables
 * (:1467-1479) and the disk-LRU backend (:1481-1515): every coefficient chunk is
 * streamed from disk through pinned buffers straight into HBM, once. The
 * manifest must match the context (layout_version, N1, N2, CHEB_NU, CHEB_NV,
 * node and sitepair counts, BETA, double tables). order1 (optional, [2]): the
 * precomputed diagonal order-1 value (diagonal_observable.txt, hi and lo), NaN
 * when the directory has none. */
int cdet_load_chunks(cdet_context* ctx, const char* dir, double* order1);

/* ------------------------------------------------- MCMCMC chains on the GPU
 * A batch of MCMCMC chains (run_single_mcmcmc_chain, mcmcmc_sampler.h:994-1088)
 * resident on the GPU, with the uniform seed kernel (MCMCMC_SEED_MODE=uniform,
 * mcmcmc_seed.h:41-61). Every step evaluates the all-subset integrand of each
 * chain's envelope with the context's assembly and runs run_mcmcmc_step
 * (:524-577) in one thread per chain. Each chain keeps the reference's
 * std::mt19937_64 stream and draws from it as libstdc++'s distributions do,
 * so with the FP64 assembly the chains follow the reference's chains step for
 * step. The lambda adaptation (adapt_mcmcmc_lambdas, :579-600) runs on the
 * host after every adapt interval of warmup steps. cdet_mcmcmc_set_histogram
 * switches the chains to the factorized histogram seed kernel
 * (MCMCMC_SEED_MODE=histogram, mcmcmc_seed.h:71-229); the chains are then the
 * reference's histogram-seeded chains step for step. Checkpoint files are not
 * part of this interface. */
typedef struct cdet_mcmcmc cdet_mcmcmc;

typedef struct cdet_mcmcmc_config {
    int32_t order_min;             /* MCMCMC_ORDER_MIN (>= 1) */
    int32_t order_max;             /* MCMCMC_ORDER_MAX (>= order_min) */
    int32_t envelope_order;        /* MCMCMC_ENVELOPE_ORDER (> order_max, <= 24 here) */
    int32_t lambda_adapt_interval; /* MCMCMC_LAMBDA_ADAPT_INTERVAL (> 0) */
    double lambda_adapt_rate;      /* MCMCMC_LAMBDA_ADAPT_RATE */
} cdet_mcmcmc_config;

/* Creates `chains` chains: chain k is make_initial_mcmcmc_chain_state with
 * seed seeds[k] (std::mt19937_64(seed), then envelope_order uniform vertices)
 * and lambdas[0..envelope_order] (MCMCMC_LAMBDAS). validate_mcmcmc_config's
 * checks apply, with its messages. The context's tables must be uploaded. */
int cdet_mcmcmc_create(cdet_context* ctx, const cdet_mcmcmc_config* config, int64_t chains, const uint64_t* seeds,
                       const double* lambdas, cdet_mcmcmc** out);

/* Advances every chain `steps` steps. warmup = 1: warmup steps (the chosen
 * orders are counted and lambdas adapted every lambda_adapt_interval warmup
 * steps); warmup = 0: production steps. Each step also updates the chain's
 * MCMCMCChainResult (below) as run_single_mcmcmc_chain does (:1036-1084).
 * Optional host outputs (null to skip): chosen[step][chain] masks,
 * norms[step][chain] local normalisations, signal[step][chain][envelope + 1]
 * the raw order signals (the reference's workspace.order_signal). A chain
 * whose integrand is not finite or whose local normalisation is not positive
 * stops (the reference throws); the call then returns CDET_ERR_VALUE naming
 * the chain, and the results of that call are not defined. Steps after the
 * first are replayed from a CUDA graph of one step. Blocking. */
int cdet_mcmcmc_run(cdet_mcmcmc* m, int warmup, int64_t steps, uint64_t* chosen, double* norms, double* signal);

#define CDET_MCMCMC_MAX_ENVELOPE 24

/* RunningStatsLongDouble (mcmcmc_sampler.h:31-77): Welford's running mean
 * and sum of squared deviations, in the host's long double. */
typedef struct cdet_running_stats {
    uint64_t count;
    long double mean;
    long double m2;
} cdet_running_stats;

/* MCMCMCChainResult (mcmcmc_sampler.h:126-139) of one chain; arrays are
 * indexed by order (0..envelope_order used). The order signal statistics
 * collect order_signal[order] / lambdas[order] of every production step. */
typedef struct cdet_mcmcmc_chain_result {
    uint64_t seed;
    uint64_t warmup_proposed_steps;
    uint64_t warmup_accepted_steps;
    uint64_t production_proposed_steps;
    uint64_t production_accepted_steps;
    uint64_t warmup_chosen_counts[CDET_MCMCMC_MAX_ENVELOPE + 1];
    uint64_t production_chosen_counts[CDET_MCMCMC_MAX_ENVELOPE + 1];
    cdet_running_stats warmup_retained_fraction_stats;
    cdet_running_stats production_retained_fraction_stats;
    cdet_running_stats order_signal_stats[CDET_MCMCMC_MAX_ENVELOPE + 1];
} cdet_mcmcmc_chain_result;

int cdet_mcmcmc_result(const cdet_mcmcmc* m, int64_t chain, cdet_mcmcmc_chain_result* out);

/* The aggregation of run_mcmcmc_chains_parallel (mcmcmc_sampler.h:1118-1146):
 * cross_chain[order] = running statistics of the chain means (each chain with
 * samples is one sample, in chain order) and ratios[order] = its mean over the
 * mean at normalization_order (NaN when that is 0), for order_min..order_max;
 * other orders are zero statistics and NaN ratios. Arrays of envelope + 1. */
int cdet_mcmcmc_summary(const cdet_mcmcmc* m, int32_t normalization_order, cdet_running_stats* cross_chain,
                        long double* ratios);

/* The absolute estimates of print_mcmcmc_summary (main.cpp:831-870): with
 * the deterministic order-1 value (a double-double, hi + lo) and the order-1
 * cross-chain statistics, the normalisation constant and its error, and per
 * order (envelope + 1 entries; order_min..order_max filled, order 1 = the
 * deterministic value) the estimate and its propagated error. Needs
 * order_min <= 1 <= order_max; CDET_ERR_VALUE when the order-1 mean is zero
 * or not finite (the reference skips the estimates). */
int cdet_mcmcmc_estimates(const cdet_mcmcmc* m, double order1_hi, double order1_lo, long double* normalization,
                          long double* normalization_stderr, long double* estimate, long double* estimate_stderr);

/* One CDET_MCMCMC_CHAIN_CHECKPOINT_V1 file (save_mcmcmc_chain_checkpoint /
 * load_mcmcmc_chain_checkpoint, mcmcmc_sampler.h:807-992): the chain's
 * state, the run settings it was written under, and its result. Arrays are
 * indexed by order (envelope_order + 1 used) or vertex. */
typedef struct cdet_mcmcmc_checkpoint {
    uint64_t chain_index;
    uint64_t seed;
    int32_t order_min, order_max, envelope_order, normalization_order;
    int32_t lambda_warmup_steps, production_steps;
    char seed_mode[16]; /* "uniform" or "histogram" */
    uint64_t rng_state[313]; /* the 312 mt19937_64 words, then the position */
    double lambdas[CDET_MCMCMC_MAX_ENVELOPE + 1];
    uint64_t warmup_block_counts[CDET_MCMCMC_MAX_ENVELOPE + 1];
    double vertices[CDET_MCMCMC_MAX_ENVELOPE][4];
    cdet_mcmcmc_chain_result result;
} cdet_mcmcmc_checkpoint;

/* Writes / reads one checkpoint file, in the reference's text format (host
 * only; no GPU needed). The writer goes through "<path>.tmp" and a rename,
 * as the reference does. The reader applies the reference's label and size
 * checks, with its messages. */
int cdet_write_mcmcmc_checkpoint(const char* path, const cdet_mcmcmc_checkpoint* checkpoint);
int cdet_read_mcmcmc_checkpoint(const char* path, cdet_mcmcmc_checkpoint* checkpoint);

/* Run settings recorded in checkpoints (MCMCMCConfig fields). */
typedef struct cdet_mcmcmc_run_info {
    int32_t normalization_order; /* MCMCMC_NORMALIZATION_ORDER */
    int32_t lambda_warmup_steps; /* MCMCMC_LAMBDA_WARMUP_STEPS */
    int32_t production_steps;    /* MCMCMC_PRODUCTION_STEPS */
} cdet_mcmcmc_run_info;

/* Writes dir/chain_NNNNNN.chk for every chain (chain index = position in the
 * batch), creating dir: the checkpoint the reference writes for the same
 * chain state. seed_mode is "histogram" after cdet_mcmcmc_set_histogram. */
int cdet_mcmcmc_save_checkpoints(const cdet_mcmcmc* m, const char* dir, const cdet_mcmcmc_run_info* info);

/* Restores chains from dir/chain_NNNNNN.chk (MCMCMC_RESUME): each file must
 * match the batch's settings and seed (the reference's "does not match"
 * check) and all restored chains must have completed the same numbers of
 * warmup and production steps, since the batch advances in lockstep. A chain
 * without a file keeps its fresh state, unless require = 1 (the reference's
 * MCMCMC_RESUME=require message). Returns the number of chains restored in
 * *restored (may be null). */
int cdet_mcmcmc_load_checkpoints(cdet_mcmcmc* m, const char* dir, const cdet_mcmcmc_run_info* info, int require,
                                 int64_t* restored);

/* The adaptation for a partial last warmup block (run_single_mcmcmc_chain,
 * :1050-1054): chains with pending counts adapt once more. */
int cdet_mcmcmc_end_warmup(cdet_mcmcmc* m);

/* Current state (null to skip): vertices[chain][envelope][4],
 * lambdas[chain][envelope + 1], rng_state[chain][313] = the 312 words of the
 * mt19937_64 state and its position, in the order std::mt19937_64 writes them. */
int cdet_mcmcmc_state(const cdet_mcmcmc* m, double* vertices, double* lambdas, uint64_t* rng_state);

int cdet_mcmcmc_destroy(cdet_mcmcmc* m);

/* Kernels of this library the batch's runs have launched so far (graph
 * replays count every kernel node), and how many steps were graph replays
 * (either may be null). */
int cdet_mcmcmc_launch_count(const cdet_mcmcmc* m, int64_t* launches, int64_t* graph_steps);

/* Green-pair reuse across steps (on by default): a step's envelope keeps the
 * chosen subset's vertices first, and the Green entries of pairs of them are
 * copied from the previous step's matrices instead of evaluated again, as the
 * reference's integrand reuses the entries of retained vertices from its
 * previous call (integrand_replica_randomly_sampled.h:57-86, 664-696,
 * 778-791). An entry depends only on its two vertices, so the chains are the
 * same bit for bit either way; enable = 0 evaluates every pair each step. */
int cdet_mcmcmc_set_green_reuse(cdet_mcmcmc* m, int enable);

/* Settings of the factorized histogram seed (MCMCMCConfig's histogram_*
 * fields, mcmcmc_sampler.h:92-95). */
typedef struct cdet_histogram_config {
    int32_t learning_steps; /* MCMCMC_SEED_HISTOGRAM_LEARNING_STEPS (> 0) */
    int32_t tau_bins;       /* MCMCMC_SEED_HISTOGRAM_TAU_BINS (> 0) */
    double uniform_mix;     /* MCMCMC_SEED_HISTOGRAM_UNIFORM_MIX, in [0, 1] */
    double pseudo_count;    /* MCMCMC_SEED_HISTOGRAM_PSEUDO_COUNT (>= 0, finite) */
} cdet_histogram_config;

/* learn_factorized_histogram_seed (mcmcmc_sampler.h:607-664) on the context's
 * tables: learning_steps uniform envelopes from std::mt19937_64 seeded with
 * derive_mcmcmc_seed(base_seed, 0x484953544F534545), their all-subset
 * integrands on the GPU (the context's assembly), the pair weights
 * accumulated on the host in long double as the reference does. Outputs the
 * row probabilities tau_prob[tau_bins][tau_bins], space_prob[N1 N2][N1 N2]
 * (site x * N2 + y), replica_prob[2][2] and (if not null) the total pair
 * weight. */
int cdet_mcmcmc_learn_histogram(cdet_context* ctx, const cdet_mcmcmc_config* config,
                                const cdet_histogram_config* histogram, uint64_t base_seed, double* tau_prob,
                                double* space_prob, double* replica_prob, double* total_pair_weight);

/* Seeds every later step of the chains with the FactorizedHistogramSeed of
 * these row probabilities (layouts as above; its CDFs are built here as
 * build_cdfs does). Allocates 2^envelope_order doubles per chain for the
 * conditional generation probabilities. A step whose seed density is negative
 * or not finite fails with "MCMCMC seed density is negative or non-finite". */
int cdet_mcmcmc_set_histogram(cdet_mcmcmc* m, int32_t tau_bins, const double* tau_prob, const double* space_prob,
                              const double* replica_prob);

/* Counters of the host entry points: integrand calls and whole-matrix
 * principal-minor fallbacks (runtime_counters.h:14-51). */
int cdet_counters(const cdet_context* ctx, uint64_t* integrand_calls, uint64_t* fpm_fallbacks);

/* Message of the last failed call on this thread ("" when none). */
const char* cdet_last_error(void);

/* Kernel launches the last evaluation issued (for launch accounting). */
int cdet_last_launch_count(const cdet_context* ctx);

/* Green-matrix assembly modes (cdet_set_assembly). */
enum cdet_assembly_mode {
    /* The reference's Clenshaw recurrences in FP64 on the CUDA cores: every
     * value bit-identical to the reference integrand (the drop-in default). */
    CDET_ASSEMBLY_FP64 = 0,
    /* Batched split-precision assembly on the tcgen05 tensor cores: lookups
     * grouped by coefficient block, each block's Chebyshev contraction as
     * eight-slice bf16 products with exact FP32 accumulation and an integer
     * epilogue (FP64-level accuracy, not bit-identical). Minors and the CDet
     * recursion stay FP64. Needs CHEB_NU and CHEB_NV <= 256 (degrees above
     * 128 run as sub-blocks of at most 128 x 128 coefficients). */
    CDET_ASSEMBLY_SPLIT_BF16 = 1
};

/* Selects the assembly of later evaluations. Replaces the VECTOR_REAL /
 * INTEGRAND_REAL precision switch (cdet_integrand_evaluator.h:431-465) with
 * the two GB300 assembly forms above. */
int cdet_set_assembly(cdet_context* ctx, int mode);

/* Work layout of the all-subsets CDet recursion (cdet_set_all_subsets_form).
 * Both forms compute every mask with the same operations in the same order,
 * so they give the same values bit for bit; they differ only in speed. */
enum cdet_all_subsets_form {
    CDET_FORM_AUTO = 0, /* the warp form below 8 warps' worth of configurations per SM, else the lane form */
    CDET_FORM_LANE = 1, /* one lane per configuration (full FP64 warps; for large batches) */
    CDET_FORM_WARP = 2  /* one warp per configuration (small batches; orders <= 11, else the lane form) */
};

int cdet_set_all_subsets_form(cdet_context* ctx, int form);

/* Under CDET_FORM_AUTO the first all-subsets evaluation of each (order,
 * assembly, batch size class = floor(log2 batch)) outside a CUDA-graph
 * capture times both forms and keeps the faster for later evaluations; this
 * reports the kept form (CDET_FORM_AUTO before any measurement). fused = 1
 * for the split assembly. */
int cdet_all_subsets_form_tuned(const cdet_context* ctx, int max_order, int fused, int64_t batch, int* form);

/* How a single-top batch (cdet_integrand_device / _host) of max_order <= 10
 * runs after its Green matrices are assembled. Every form performs the same
 * operations per configuration, so all give the same values bit for bit.
 * Replaces nothing in the reference: its integrand evaluates one
 * configuration per call (integrand_replica_randomly_sampled.h:498-560);
 * these are the batched layouts of that call. */
enum cdet_integrand_form {
    CDET_INTEGRAND_AUTO = 0,   /* measured per (order, assembly, batch size class); see below */
    CDET_INTEGRAND_STAGED = 1, /* minors kernel (a warp per configuration and set), a[] in HBM, CDet kernel */
    CDET_INTEGRAND_QUEUE = 2   /* one persistent kernel: minors and CDet of a configuration in shared
                                  memory, configurations taken from order-sorted slots (decreasing
                                  order) through an atomic queue head */
};

/* Selects the form; for CDET_INTEGRAND_QUEUE also its launch shape:
 * warps_per_sm = resident warps per SM (0: as many as shared memory holds),
 * pair = 1 for two warps per configuration (one per table set), grab = slots
 * a warp takes per queue pop (>= 1). CDET_INTEGRAND_AUTO (the default) makes
 * the first evaluation of each (max_order, assembly, floor(log2 batch))
 * outside a CUDA-graph capture time the staged form and four queue shapes on
 * its own Green matrices and keep the fastest. */
int cdet_set_integrand_form(cdet_context* ctx, int form, int warps_per_sm, int pair, int grab);

/* The form the tuner kept for (max_order, fused = 1 for the split assembly,
 * batch): *form is CDET_INTEGRAND_AUTO before any measurement of that key. */
int cdet_integrand_form_tuned(const cdet_context* ctx, int max_order, int fused, int64_t batch, int* form,
                              int* warps_per_sm, int* pair, int* grab);

/* The DoubleDouble value of one of the reference's MP_Real parameters,
 * DoubleDouble(MP_Real(literal)) = {the nearest double, the nearest double to
 * the rest} (utility/types.h:41-45). */
typedef struct cdet_dd {
    double hi, lo;
} cdet_dd;

/* What the DoubleDouble integrand reads besides the FP64 scalars:
 * IntegrandRuntimeScalars<DoubleDouble> as make_integrand_runtime_scalars
 * builds it from the MP_Real parameters (integrand_replica_randomly_sampled.h:
 * 98-119: the diagonal shifts are alpha / U in DoubleDouble) and the round-off
 * filter constants in DoubleDouble (precision_config.h:158-186). */
typedef struct cdet_dd_scalars {
    cdet_dd beta, u;                /* beta, U */
    cdet_dd alpha_up, alpha_down;   /* ALPHA_UP, ALPHA_DOWN */
    cdet_dd tol_fpm, fpm_shift;     /* TOL_FPM, FPM_GLOBAL_SHIFT (-1 when auto) */
    cdet_dd z_eps0, z_safety;       /* ZTRANSFORM_EPSILON0 (1e-31 when auto), ZTRANSFORM_SAFETY_FACTOR */
} cdet_dd_scalars;

enum cdet_integrand_real {
    CDET_INTEGRAND_REAL_DOUBLE = 0,        /* INTEGRAND_REAL=double (default): the FP64 drop-in */
    CDET_INTEGRAND_REAL_DOUBLE_DOUBLE = 1  /* INTEGRAND_REAL=double_double with VECTOR_REAL=double */
};

/* The reference's INTEGRAND_REAL switch (precision_config.h:15-26,
 * cdet_integrand_evaluator.h:431-465). In the double-double mode the minors,
 * the CDet recursion and the order-1 branch run in the reference's
 * DoubleDouble arithmetic on the Green matrices of the context's assembly:
 * with CDET_ASSEMBLY_FP64 (VECTOR_REAL=double) cdet_integrand_device / _host
 * return the reference's double-double values bit for bit; with
 * CDET_ASSEMBLY_SPLIT_BF16 the same arithmetic runs on the tensor-core
 * Green matrices (no counterpart in the reference: its values differ from
 * the reference mode's by what the Green entries' last bits move, not by the
 * FP64 recursion's round-off). dd may be null for CDET_INTEGRAND_REAL_DOUBLE.
 * Single-configuration integrands of order <= 10 only: an all-subsets call or
 * a higher order fails with CDET_ERR_INVALID. Its work layout follows
 * cdet_set_integrand_form: CDET_INTEGRAND_STAGED = minors by warps, then the
 * recursion one lane per configuration; CDET_INTEGRAND_QUEUE = one warp per
 * configuration; AUTO = the lane layout from one warp of configurations per
 * SM. On the FP64 assembly both layouts give the reference's values; on the
 * split assembly the lane layout's minors and recursion take lighter
 * double-double steps (FMA products, one renormalisation per sum, the
 * filter's magnitude sum in FP64), so there they differ in the last bits. */
int cdet_set_integrand_real(cdet_context* ctx, int real_type, const cdet_dd_scalars* dd);

/* Builds the bf16 slices of every uploaded table for the split assembly
 * (otherwise done by the first split evaluation). Allocates about twice the
 * FP64 table size of device memory. */
int cdet_prepare_split(cdet_context* ctx);

/* Runs only the Green-matrix assembly of the current mode, for testing:
 * green[c][set][spin][i*n+j] and diag[c][set][spin][i] (set 0 twisted,
 * 1 ordinary; spin 0 up, 1 down; n = orders[c]) receive the matrices the
 * integrand's fill step builds (integrand_replica_randomly_sampled.h:434-484),
 * including the diagonal shifts and the scale. Device buffers, asynchronous. */
int cdet_assemble_device(cdet_context* ctx, const double* vertices, const int32_t* orders,
                         int64_t batch, int max_order, double* green, double* diag,
                         int32_t* status, void* stream);

/* Measurement hooks; no counterpart in the reference. While enabled, every
 * evaluation records CUDA events between its stages on the stream it runs
 * on. cdet_profile_read waits for the recorded events, adds the elapsed
 * milliseconds per stage to kernel_ms[0..3] (0: descriptors and sort of the
 * split assembly, 1: Green-matrix assembly, 2: principal minors, 3: CDet and
 * prefactors), adds the number of kernel launches to *launches, and clears
 * the record. */
int cdet_profile_enable(cdet_context* ctx, int enable);
int cdet_profile_read(cdet_context* ctx, double* kernel_ms, int64_t* launches);

/* Measurement hook; no counterpart in the reference. Counters of the last
 * split-assembly evaluation on this context (waits for it): out[0] = the
 * accumulator columns its tcgen05.mma instructions wrote (M = 128, K = 16:
 * 2 x 128 x 16 flops of issued tensor work each), out[1] = the
 * coefficient-slice bytes it streamed from global memory. Both are zero
 * before the first split evaluation. */
int cdet_split_counters(cdet_context* ctx, uint64_t* out);

#ifdef __cplusplus
}
#endif

#endif /* CDET_GB300_H */
