// Device-resident MCMCMC chains: one thread per chain runs run_mcmcmc_step
// (mcmcmc_sampler.h:524-577) on the all-subset integrand values of its
// envelope, so a batch of chains advances one step per launch pair
// (integrand, step) with no host round trip. The seed kernel is the uniform
// one (mcmcmc_seed.h:41-61) or the factorized histogram (:71-229), whose
// conditional generation probabilities (mcmcmc_sampler.h:252-335) weight the
// fluxes.
//
// Each chain keeps the reference's std::mt19937_64 stream (the published
// MT19937-64 generator with libstdc++'s seeding) and draws from it exactly as
// libstdc++'s distributions do: std::generate_canonical<double, 53> takes one
// 64-bit output, converts it to double (round to nearest) and divides by 2^64;
// std::uniform_int_distribution<int> downscales with a 128-bit product
// (nearly-divisionless rejection). With the FP64 integrand the device chains
// therefore follow the reference's chains step for step. The generator state
// is stored interleaved ([word][chain]) so that the threads of a warp touch
// consecutive addresses.
#include "cdet_device.cuh"
#include "cdet_kernels.cuh"

namespace cdet {

namespace {

constexpr int kMtN = 312;
constexpr int kMtM = 156;

struct Mt64 {
    uint64_t* words;  // word i of this chain at words[i * stride]
    int64_t stride;
    int32_t* index;

    __device__ __forceinline__ uint64_t& at(int i) const { return words[static_cast<int64_t>(i) * stride]; }

    __device__ uint64_t next() const {
        if (*index >= kMtN) {
            const uint64_t upper = 0xFFFFFFFF80000000ull, lower = 0x7FFFFFFFull, matrix = 0xB5026F5AA96619E9ull;
            for (int i = 0; i < kMtN; ++i) {
                const uint64_t x = (at(i) & upper) | (at(i + 1 < kMtN ? i + 1 : 0) & lower);
                at(i) = at(i + kMtM < kMtN ? i + kMtM : i + kMtM - kMtN) ^ (x >> 1) ^ ((x & 1ull) ? matrix : 0ull);
            }
            *index = 0;
        }
        uint64_t y = at((*index)++);
        y ^= (y >> 29) & 0x5555555555555555ull;
        y ^= (y << 17) & 0x71D67FFFEDA60000ull;
        y ^= (y << 37) & 0xFFF7EEE000000000ull;
        y ^= y >> 43;
        return y;
    }

    // std::generate_canonical<double, 53> as libstdc++ computes it
    __device__ double canonical() const {
        const double r = ddiv(__ull2double_rn(next()), 18446744073709551616.0);
        return r >= 1.0 ? __longlong_as_double(0x3FEFFFFFFFFFFFFFll) : r;
    }

    // std::uniform_int_distribution<int>(0, n - 1)
    __device__ int uniform_int(int n) const {
        const uint64_t range = static_cast<uint64_t>(n);
        uint64_t x = next();
        uint64_t low = x * range;
        uint64_t high = __umul64hi(x, range);
        if (low < range) {
            const uint64_t threshold = (0ull - range) % range;
            while (low < threshold) {
                x = next();
                low = x * range;
                high = __umul64hi(x, range);
            }
        }
        return static_cast<int>(high);
    }
};

// unit_coordinate_to_index (mcmcmc_seed.h:30-39)
__device__ __forceinline__ int unit_index(double value, int extent) {
    const int index = static_cast<int>(floor(dmul(value, static_cast<double>(extent))));
    if (index < 0) return 0;
    if (index >= extent) return extent - 1;
    return index;
}

// sample_from_row (mcmcmc_seed.h:205-218): std::lower_bound (the binary search
// for the first entry not below the draw) in one CDF row; past the end, the
// last column
__device__ int sample_row(const double* __restrict__ cdf, int columns, int row, const Mt64& g) {
    const double threshold = g.canonical();
    const double* b = cdf + static_cast<int64_t>(row) * columns;
    int first = 0, len = columns;
    while (len > 0) {
        const int half = len >> 1;
        if (b[first + half] < threshold) {
            first += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    return first == columns ? columns - 1 : first;
}

// density_child_given_parent (mcmcmc_seed.h:130-150)
__device__ double hist_density(const McmcmcStepArgs& a, const double* child, const double* parent) {
    const int sites = a.n1 * a.n2;
    const double tau_d = dmul(a.tau_prob[unit_index(parent[0], a.tau_bins) * a.tau_bins +
                                         unit_index(child[0], a.tau_bins)],
                              static_cast<double>(a.tau_bins));
    const int ps = unit_index(parent[1], a.n1) * a.n2 + unit_index(parent[2], a.n2);
    const int cs = unit_index(child[1], a.n1) * a.n2 + unit_index(child[2], a.n2);
    const double space_d = dmul(a.space_prob[static_cast<int64_t>(ps) * sites + cs], static_cast<double>(sites));
    const double rep_d = dmul(a.replica_prob[unit_index(parent[3], 2) * 2 + unit_index(child[3], 2)], 2.0);
    return dmul(dmul(tau_d, space_d), rep_d);
}

// sample_child_from_parent (mcmcmc_seed.h:106-128): three row draws, then the
// four in-cell offsets in vertex order
__device__ void hist_child(const McmcmcStepArgs& a, const Mt64& g, const double* parent, double* child) {
    const int child_tau = sample_row(a.tau_cdf, a.tau_bins, unit_index(parent[0], a.tau_bins), g);
    const int parent_site = unit_index(parent[1], a.n1) * a.n2 + unit_index(parent[2], a.n2);
    const int child_site = sample_row(a.space_cdf, a.n1 * a.n2, parent_site, g);
    const int child_x = child_site / a.n2;
    const int child_y = child_site - child_x * a.n2;
    const int child_rep = sample_row(a.replica_cdf, 2, unit_index(parent[3], 2), g);
    child[0] = ddiv(dadd(static_cast<double>(child_tau), g.canonical()), static_cast<double>(a.tau_bins));
    child[1] = ddiv(dadd(static_cast<double>(child_x), g.canonical()), static_cast<double>(a.n1));
    child[2] = ddiv(dadd(static_cast<double>(child_y), g.canonical()), static_cast<double>(a.n2));
    child[3] = ddiv(dadd(static_cast<double>(child_rep), g.canonical()), 2.0);
}

// compute_conditional_generation_probabilities_typed_into<double>
// (mcmcmc_sampler.h:252-335), one warp per chain. The reference tabulates the
// remaining child densities cd[gm][c] by peeling the lowest bit of gm; here
// each one is formed on the spot from the row sum with the same subtractions
// in the same order (the highest bit of gm first), each result clamped as the
// table's is, so only the 2^n probabilities are stored. The subsets of one
// popcount level depend only on the level below, so the lanes share each
// level; every subset's sum runs on one lane in the reference's order, so the
// values are the reference's bit for bit. sd: this warp's n x n densities in
// shared memory. false (on every lane): a density is negative or not finite.
__device__ bool conditional_probabilities_warp(const McmcmcStepArgs& a, const double* v, int n, double* prob,
                                               double* sd, double* cd0, int lane) {
    bool bad = false;
    for (int idx = lane; idx < n * n; idx += 32) {
        const int c = idx / n, p = idx - (idx / n) * n;
        double d = 0.0;
        if (c != p) {
            d = hist_density(a, v + 4 * c, v + 4 * p);
            bad |= d < 0.0 || !isfinite(d);
        }
        sd[idx] = d;
    }
    if (__any_sync(0xffffffffu, bad)) return false;
    __syncwarp();
    if (lane < n) {
        double sum = 0.0;
        for (int p = 0; p < n; ++p) sum = dadd(sum, sd[lane * n + p]);
        cd0[lane] = sum;
    }
    const uint64_t full = (uint64_t{1} << n) - 1;
    if (lane == 0) {
        prob[0] = 1.0;
        prob[full] = 0.0;
    }
    __syncwarp();
    for (int level = 1; level < n; ++level) {
        const int pc = n - level;
        const double denom = dmul(static_cast<double>(level), static_cast<double>(pc));
        const uint32_t per = kBinomial.c[n][level];
        for (uint32_t r = lane; r < per; r += 32) {
            const uint64_t gm = colex_subset(r, level, n);  // the level's subsets dealt out evenly
            double sum = 0.0;
            for (int c = 0; c < n; ++c) {
                const uint64_t cb = uint64_t{1} << c;
                if (!(gm & cb)) continue;
                double d = cd0[c];
                for (uint64_t rest = gm; rest;) {
                    const int b = 63 - __clzll(static_cast<long long>(rest));
                    rest ^= uint64_t{1} << b;
                    d = dsub(d, sd[c * n + b]);
                    if (d < 0.0 && d > -1.0e-12) d = 0.0;
                }
                sum = dadd(sum, dmul(prob[gm ^ cb], d));
            }
            prob[gm] = ddiv(sum, denom);
        }
        __syncwarp();  // the next level reads this one
    }
    return true;
}

// std::mt19937_64(seed) and sample_uniform_vertex_set (mcmcmc_sampler.h:187-198)
__global__ void mcmcmc_init(int64_t chains, int envelope, const uint64_t* __restrict__ seeds, uint64_t* mt,
                            int32_t* mt_index, double* vertices) {
    const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= chains) return;
    const Mt64 g{mt + c, chains, mt_index + c};
    uint64_t x = seeds[c];
    g.at(0) = x;
    for (int i = 1; i < kMtN; ++i) {
        x = 6364136223846793005ull * (x ^ (x >> 62)) + static_cast<uint64_t>(i);
        g.at(i) = x;
    }
    *g.index = kMtN;
    double* v = vertices + c * envelope * 4;
    for (int k = 0; k < envelope * 4; ++k) v[k] = g.canonical();
}

// The serial part of run_mcmcmc_step (:540-577) for chain c, after the seed
// kernel's conditional probabilities (cprob; null for the uniform kernel).
template <bool Hist>
__device__ void finish_step(const McmcmcStepArgs& a, int64_t c, int64_t row, const double* cprob) {
    const int env = a.envelope;
    const uint64_t subsets = uint64_t{1} << env;
    const double* values = a.values + c * static_cast<int64_t>(subsets);
    const double* lam = a.lambdas + c * (env + 1);
    const Mt64 g{a.mt + c, a.chains, a.mt_index + c};
    const double* v = a.vertices + c * env * 4;
    const uint64_t full = subsets - 1;
    // flux = lambda * value * conditional probability of the complement
    // (1 for the uniform kernel)
    auto flux_of = [&](uint64_t mask, int o) {
        return dmul(dmul(lam[o], values[mask]), Hist ? cprob[full ^ mask] : 1.0);
    };
    // fluxes and selection weights in the mask plan's order (:411-430, :540-560)
    double norm = 0.0;
    for (uint64_t mask = 1; mask < subsets; ++mask) {
        const int o = __popcll(mask);
        if (o < a.order_min || o > a.order_max) continue;
        norm = dadd(norm, dmul(fabs(flux_of(mask, o)), a.inv_binom[o]));
    }
    // sample_weighted_candidate_mask (:225-250)
    if (!(norm > 0.0) || !isfinite(norm)) {
        a.error[c] = 2;  // "MCMCMC local normalization is zero or non-finite"
        return;
    }
    const double threshold = dadd(dmul(g.canonical(), dsub(norm, 0.0)), 0.0);
    double cumulative = 0.0;
    uint64_t chosen = 0, last_positive = 0;
    bool found = false;
    for (uint64_t mask = 1; mask < subsets && !found; ++mask) {
        const int o = __popcll(mask);
        if (o < a.order_min || o > a.order_max) continue;
        const double w = dmul(fabs(flux_of(mask, o)), a.inv_binom[o]);
        if (!(w > 0.0)) continue;
        if (isfinite(w)) last_positive = mask;
        cumulative = dadd(cumulative, w);
        if (cumulative > threshold) {
            chosen = mask;
            found = true;
        }
    }
    if (!found) chosen = last_positive;
    // order signal: time = flux / local_normalization, weighted by 1/binomial (:566-571)
    if (a.signal_out) {
        double* sig = a.signal_out + (row * a.chains + c) * (env + 1);
        for (int o = 0; o <= env; ++o) sig[o] = 0.0;
        for (uint64_t mask = 1; mask < subsets; ++mask) {
            const int o = __popcll(mask);
            if (o < a.order_min || o > a.order_max) continue;
            const double time = ddiv(flux_of(mask, o), norm);
            sig[o] = dadd(sig[o], dmul(time, a.inv_binom[o]));
        }
    }
    // create_next_vertices_from_seed_into (:380-400): the retained vertices in
    // order, then children of uniformly chosen parents among the vertices so
    // far (the uniform kernel, mcmcmc_seed.h:51-55, ignores the parent)
    double* nv = a.next_vertices + c * env * 4;
    int size = 0;
    for (int i = 0; i < env; ++i)
        if (chosen & (uint64_t{1} << i)) {
            for (int k = 0; k < 4; ++k) nv[4 * size + k] = v[4 * i + k];
            ++size;
        }
    while (size < env) {
        const int parent = g.uniform_int(size);
        if constexpr (Hist) {
            hist_child(a, g, nv + 4 * parent, nv + 4 * size);
        } else {
            (void)parent;
            for (int k = 0; k < 4; ++k) nv[4 * size + k] = g.canonical();
        }
        ++size;
    }
    const int order = __popcll(chosen);
    if (a.chosen_out) a.chosen_out[row * a.chains + c] = chosen;
    if (a.retained_out) a.retained_out[c] = chosen;
    if (a.norm_out) a.norm_out[row * a.chains + c] = norm;
    if (a.warmup) ++a.counts[c * (env + 1) + order];
}

// The step, one thread per chain (after mcmcmc_hist_probs for the histogram
// seed kernel).
template <bool Hist>
__global__ void __launch_bounds__(128) mcmcmc_step(const __grid_constant__ McmcmcStepArgs a) {
    const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= a.chains) return;
    const int64_t row = a.ring_row ? *a.ring_row : 0;
    if (a.chosen_out) a.chosen_out[row * a.chains + c] = 0;  // 0: no step (a failed chain)
    if (a.retained_out) a.retained_out[c] = 0;
    if (a.error[c]) return;  // a chain that failed stays where it stopped
    if (a.integrand_status[c] & kStatusNonFinite) {
        a.error[c] = 1;  // "Error (all-subset integrand): Value is not finite"
        return;
    }
    finish_step<Hist>(a, c, row, Hist ? a.cprob + c * (int64_t{1} << a.envelope) : nullptr);
}

// The serial part of the step with one warp per chain (small batches): the
// fluxes elementwise on all lanes, the local normalisation and the weighted
// draw on lane 0 (both are running sums in mask order), each order's signal
// sum on its own lane (its masks in increasing order, as the reference adds
// them), then the next vertices on lane 0. Same values as finish_step.
template <bool Hist>
__device__ void finish_step_warp(const McmcmcStepArgs& a, int64_t c, int64_t row, const double* cprob, double* flux,
                                 int lane) {
    const int env = a.envelope;
    const uint32_t subsets = 1u << env, full = subsets - 1;
    const double* values = a.values + c * static_cast<int64_t>(subsets);
    const double* lam = a.lambdas + c * (env + 1);
    for (uint32_t mask = lane; mask < subsets; mask += 32) {
        const int o = __popc(mask);
        flux[mask] = (mask == 0 || o < a.order_min || o > a.order_max)
                         ? 0.0
                         : dmul(dmul(lam[o], values[mask]), Hist ? cprob[full ^ mask] : 1.0);
    }
    __syncwarp();
    double norm = 0.0;
    if (lane == 0)
        for (uint32_t mask = 1; mask < subsets; ++mask) {
            const int o = __popc(mask);
            if (o < a.order_min || o > a.order_max) continue;
            norm = dadd(norm, dmul(fabs(flux[mask]), a.inv_binom[o]));
        }
    norm = __shfl_sync(0xffffffffu, norm, 0);
    if (!(norm > 0.0) || !isfinite(norm)) {
        if (lane == 0) a.error[c] = 2;  // "MCMCMC local normalization is zero or non-finite"
        return;
    }
    if (a.signal_out && lane <= env) {
        double sig = 0.0;
        if (lane >= 1 && lane >= a.order_min && lane <= a.order_max) {
            const uint32_t masks = kBinomial.c[env][lane];
            uint32_t m = (1u << lane) - 1u;
            for (uint32_t r = 0; r < masks; ++r, m = next_same_popcount(m))
                sig = dadd(sig, dmul(ddiv(flux[m], norm), a.inv_binom[lane]));
        }
        a.signal_out[(row * a.chains + c) * (env + 1) + lane] = sig;
    }
    if (lane != 0) return;
    const Mt64 g{a.mt + c, a.chains, a.mt_index + c};
    const double threshold = dadd(dmul(g.canonical(), dsub(norm, 0.0)), 0.0);
    double cumulative = 0.0;
    uint64_t chosen = 0, last_positive = 0;
    bool found = false;
    for (uint32_t mask = 1; mask < subsets && !found; ++mask) {
        const int o = __popc(mask);
        if (o < a.order_min || o > a.order_max) continue;
        const double w = dmul(fabs(flux[mask]), a.inv_binom[o]);
        if (!(w > 0.0)) continue;
        if (isfinite(w)) last_positive = mask;
        cumulative = dadd(cumulative, w);
        if (cumulative > threshold) {
            chosen = mask;
            found = true;
        }
    }
    if (!found) chosen = last_positive;
    const double* v = a.vertices + c * env * 4;
    double* nv = a.next_vertices + c * env * 4;
    int size = 0;
    for (int i = 0; i < env; ++i)
        if (chosen & (uint64_t{1} << i)) {
            for (int k = 0; k < 4; ++k) nv[4 * size + k] = v[4 * i + k];
            ++size;
        }
    while (size < env) {
        const int parent = g.uniform_int(size);
        if constexpr (Hist) {
            hist_child(a, g, nv + 4 * parent, nv + 4 * size);
        } else {
            (void)parent;
            for (int k = 0; k < 4; ++k) nv[4 * size + k] = g.canonical();
        }
        ++size;
    }
    if (a.chosen_out) a.chosen_out[row * a.chains + c] = chosen;
    if (a.retained_out) a.retained_out[c] = chosen;
    if (a.norm_out) a.norm_out[row * a.chains + c] = norm;
    if (a.warmup) ++a.counts[c * (env + 1) + __popcll(chosen)];
}

// The whole step for a small batch: one warp (and block) per chain, its
// fluxes, and for the histogram seed kernel its densities and conditional
// probabilities, in shared memory.
constexpr int kStepWarpMaxEnvelope = 12;
constexpr int64_t kStepWarpMaxChains = 2048;
template <bool Hist>
__global__ void __launch_bounds__(32) mcmcmc_step_warp(const __grid_constant__ McmcmcStepArgs a) {
    extern __shared__ double step_smem[];
    const int lane = threadIdx.x;
    const int64_t c = blockIdx.x;
    const int env = a.envelope;
    const uint32_t subsets = 1u << env;
    double* flux = step_smem;
    double* prob = flux + subsets;
    double* sd = prob + subsets;
    double* cd0 = sd + env * env;
    const int64_t row = a.ring_row ? *a.ring_row : 0;
    if (lane == 0 && a.chosen_out) a.chosen_out[row * a.chains + c] = 0;  // 0: no step (a failed chain)
    if (lane == 0 && a.retained_out) a.retained_out[c] = 0;
    if (a.error[c]) return;  // the same value on every lane
    if (a.integrand_status[c] & kStatusNonFinite) {
        if (lane == 0) a.error[c] = 1;  // "Error (all-subset integrand): Value is not finite"
        return;
    }
    if constexpr (Hist) {
        if (!conditional_probabilities_warp(a, a.vertices + c * env * 4, env, prob, sd, cd0, lane)) {
            if (lane == 0) a.error[c] = 3;  // "MCMCMC seed density is negative or non-finite"
            return;
        }
        __syncwarp();
    }
    finish_step_warp<Hist>(a, c, row, prob, flux, lane);
}

// The histogram seed kernel's conditional generation probabilities, one warp
// per chain, into a.cprob; a negative or non-finite seed density stops the
// chain (error 3), which the step kernel then skips.
constexpr int kHistWarps = 4;
__global__ void __launch_bounds__(kHistWarps * 32) mcmcmc_hist_probs(const __grid_constant__ McmcmcStepArgs a) {
    __shared__ double sd_all[kHistWarps][kMcmcmcMaxEnvelope * kMcmcmcMaxEnvelope];
    __shared__ double cd0_all[kHistWarps][kMcmcmcMaxEnvelope];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c = static_cast<int64_t>(blockIdx.x) * kHistWarps + warp;
    if (c >= a.chains) return;  // whole warps
    // both read the same value on every lane; the step kernel reports a non-finite integrand
    if (a.error[c] || (a.integrand_status[c] & kStatusNonFinite)) return;
    const int env = a.envelope;
    double* cprob = a.cprob + c * (int64_t{1} << env);
    const double* v = a.vertices + c * env * 4;
    if (!conditional_probabilities_warp(a, v, env, cprob, sd_all[warp], cd0_all[warp], lane) && lane == 0)
        a.error[c] = 3;  // "MCMCMC seed density is negative or non-finite"
}

__global__ void mcmcmc_advance_row(int64_t* row, int64_t rows) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *row = (*row + 1) % rows;
}

}  // namespace

cudaError_t launch_mcmcmc_advance_row(int64_t* row, int64_t rows, cudaStream_t stream) {
    mcmcmc_advance_row<<<1, 32, 0, stream>>>(row, rows);
    return cudaGetLastError();
}

cudaError_t launch_mcmcmc_init(int64_t chains, int envelope, const uint64_t* seeds, uint64_t* mt, int32_t* mt_index,
                               double* vertices, cudaStream_t stream) {
    if (chains <= 0) return cudaSuccess;
    mcmcmc_init<<<static_cast<unsigned>((chains + 127) / 128), 128, 0, stream>>>(chains, envelope, seeds, mt,
                                                                                mt_index, vertices);
    return cudaGetLastError();
}

cudaError_t launch_mcmcmc_step(const McmcmcStepArgs& args, cudaStream_t stream, int* kernels) {
    *kernels = 0;
    if (args.chains <= 0) return cudaSuccess;
    const bool hist = args.tau_bins > 0;
    if (args.chains < kStepWarpMaxChains && args.envelope <= kStepWarpMaxEnvelope) {
        const size_t subsets = size_t{1} << args.envelope;
        const size_t smem =
            (subsets + (hist ? subsets + static_cast<size_t>(args.envelope) * (args.envelope + 1) : 0)) *
            sizeof(double);
        const void* fn = hist ? reinterpret_cast<const void*>(mcmcmc_step_warp<true>)
                              : reinterpret_cast<const void*>(mcmcmc_step_warp<false>);
        cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (err != cudaSuccess) return err;
        if (hist)
            mcmcmc_step_warp<true><<<static_cast<unsigned>(args.chains), 32, smem, stream>>>(args);
        else
            mcmcmc_step_warp<false><<<static_cast<unsigned>(args.chains), 32, smem, stream>>>(args);
        *kernels = 1;
        return cudaGetLastError();
    }
    const unsigned grid = static_cast<unsigned>((args.chains + 127) / 128);
    *kernels = hist ? 2 : 1;
    if (hist) {
        mcmcmc_hist_probs<<<static_cast<unsigned>((args.chains + kHistWarps - 1) / kHistWarps), kHistWarps * 32, 0,
                            stream>>>(args);
        const cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        mcmcmc_step<true><<<grid, 128, 0, stream>>>(args);
    } else {
        mcmcmc_step<false><<<grid, 128, 0, stream>>>(args);
    }
    return cudaGetLastError();
}

}  // namespace cdet
