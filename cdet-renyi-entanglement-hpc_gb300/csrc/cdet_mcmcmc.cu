// Device-resident MCMCMC chains with the uniform seed kernel: one thread per
// chain runs run_mcmcmc_step (mcmcmc_sampler.h:524-577) on the all-subset
// integrand values of its envelope, so a batch of chains advances one step
// per launch pair (integrand, step) with no host round trip.
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

__global__ void __launch_bounds__(128) mcmcmc_step_uniform(const __grid_constant__ McmcmcStepArgs a) {
    const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= a.chains) return;
    if (a.error[c]) return;  // a chain that failed stays where it stopped
    if (a.integrand_status[c] & kStatusNonFinite) {
        a.error[c] = 1;  // "Error (all-subset integrand): Value is not finite"
        return;
    }
    const int env = a.envelope;
    const uint64_t subsets = uint64_t{1} << env;
    const double* values = a.values + c * static_cast<int64_t>(subsets);
    const double* lam = a.lambdas + c * (env + 1);
    const Mt64 g{a.mt + c, a.chains, a.mt_index + c};
    // fluxes and selection weights in the mask plan's order (:411-430, :540-560)
    double norm = 0.0;
    for (uint64_t mask = 1; mask < subsets; ++mask) {
        const int o = __popcll(mask);
        if (o < a.order_min || o > a.order_max) continue;
        const double flux = dmul(dmul(lam[o], values[mask]), 1.0);
        norm = dadd(norm, dmul(fabs(flux), a.inv_binom[o]));
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
        const double w = dmul(fabs(dmul(dmul(lam[o], values[mask]), 1.0)), a.inv_binom[o]);
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
        double* sig = a.signal_out + c * (env + 1);
        for (int o = 0; o <= env; ++o) sig[o] = 0.0;
        for (uint64_t mask = 1; mask < subsets; ++mask) {
            const int o = __popcll(mask);
            if (o < a.order_min || o > a.order_max) continue;
            const double time = ddiv(dmul(dmul(lam[o], values[mask]), 1.0), norm);
            sig[o] = dadd(sig[o], dmul(time, a.inv_binom[o]));
        }
    }
    // create_next_vertices_from_seed_into (:380-400) with the uniform seed
    // kernel (mcmcmc_seed.h:51-55): the retained vertices in order, then
    // children from uniformly chosen parents (the uniform kernel ignores them)
    const double* v = a.vertices + c * env * 4;
    double* nv = a.next_vertices + c * env * 4;
    int size = 0;
    for (int i = 0; i < env; ++i)
        if (chosen & (uint64_t{1} << i)) {
            for (int k = 0; k < 4; ++k) nv[4 * size + k] = v[4 * i + k];
            ++size;
        }
    while (size < env) {
        (void)g.uniform_int(size);
        for (int k = 0; k < 4; ++k) nv[4 * size + k] = g.canonical();
        ++size;
    }
    const int order = __popcll(chosen);
    if (a.chosen_out) a.chosen_out[c] = chosen;
    if (a.norm_out) a.norm_out[c] = norm;
    if (a.warmup) ++a.counts[c * (env + 1) + order];
}

}  // namespace

cudaError_t launch_mcmcmc_init(int64_t chains, int envelope, const uint64_t* seeds, uint64_t* mt, int32_t* mt_index,
                               double* vertices, cudaStream_t stream) {
    if (chains <= 0) return cudaSuccess;
    mcmcmc_init<<<static_cast<unsigned>((chains + 127) / 128), 128, 0, stream>>>(chains, envelope, seeds, mt,
                                                                                mt_index, vertices);
    return cudaGetLastError();
}

cudaError_t launch_mcmcmc_step(const McmcmcStepArgs& args, cudaStream_t stream) {
    if (args.chains <= 0) return cudaSuccess;
    mcmcmc_step_uniform<<<static_cast<unsigned>((args.chains + 127) / 128), 128, 0, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace cdet
