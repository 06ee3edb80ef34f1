// Drop-in check of include/cdet_gb300.hpp, in the style of the reference's
// audit tests/test_integrand_all_subsets.cpp: load a parameter set and its
// four tables, install the GPU integrand, evaluate single-order and
// all-subset integrands through the reference-named free functions, write the
// values for the Python side to compare with the golden vectors, and check
// every subset of each all-subset envelope against an independent
// single-order call within 2e-9 (the audit's tolerance). Then runs the
// reference's histogram-seeded MCMCMC chains of the set through
// McmcmcChains, with a checkpoint half-way, and writes their final state and
// results.
//
// usage: adapter_check <dir>  (files written by tests/test_gpu_cpp_adapter.py)
#include "cdet_gb300.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

using cdet_gb300::UnitVertex;

template <typename T>
static std::vector<T> read_all(const std::string& path) {
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    if (!in) throw std::runtime_error("cannot open " + path);
    const std::streamsize bytes = in.tellg();
    in.seekg(0);
    std::vector<T> data(static_cast<std::size_t>(bytes) / sizeof(T));
    in.read(reinterpret_cast<char*>(data.data()), bytes);
    return data;
}

template <typename T>
static void write_all(const std::string& path, const std::vector<T>& data) {
    std::ofstream out(path, std::ios::binary);
    out.write(reinterpret_cast<const char*>(data.data()), static_cast<std::streamsize>(data.size() * sizeof(T)));
}

int main(int argc, char** argv) try {
    if (argc != 2) throw std::runtime_error("usage: adapter_check <dir>");
    const std::string dir = argv[1];
    const auto raw = read_all<char>(dir + "/scalars.bin");
    cdet_runtime_scalars scalars{};
    if (raw.size() != sizeof(scalars)) throw std::runtime_error("scalars.bin has the wrong size");
    std::copy(raw.begin(), raw.end(), reinterpret_cast<char*>(&scalars));

    cdet_gb300::Integrand gpu(scalars, 0);
    const char* kinds[4] = {"twisted_up", "twisted_down", "ordinary_up", "ordinary_down"};
    const auto alias = read_all<int32_t>(dir + "/alias.bin");  // [4]: source kind or -1
    std::vector<std::vector<double>> keep;
    keep.reserve(16);
    for (int k = 0; k < 4; ++k) {
        if (alias[k] >= 0) {
            gpu.alias(k, alias[k]);
            continue;
        }
        const std::string base = dir + "/" + kinds[k];
        for (const char* part : {"upper", "lower", "upper_corners", "lower_corners"})
            keep.push_back(read_all<double>(base + "." + part + ".bin"));
        const std::size_t n = keep.size();
        gpu.upload(k, cdet_gb300::TableView{&keep[n - 4], &keep[n - 3], &keep[n - 2], &keep[n - 1]});
    }
    gpu.install();

    const auto vflat = read_all<double>(dir + "/vertices.bin");  // [N][8][4]
    const auto orders = read_all<int32_t>(dir + "/orders.bin");
    std::vector<double> single(orders.size());
    for (std::size_t c = 0; c < orders.size(); ++c) {
        std::vector<UnitVertex> v(static_cast<std::size_t>(orders[c]));
        for (int i = 0; i < orders[c]; ++i)
            v[i] = UnitVertex{vflat[(c * 8 + i) * 4], vflat[(c * 8 + i) * 4 + 1], vflat[(c * 8 + i) * 4 + 2],
                              vflat[(c * 8 + i) * 4 + 3]};
        single[c] = cdet_gb300::evaluate_cdet_density_integrand_double(v);
    }
    write_all(dir + "/single_out.bin", single);

    const auto env = read_all<double>(dir + "/envelopes.bin");  // [E][6][4]
    const std::size_t envelopes = env.size() / 24;
    std::vector<double> all_out;
    int checked = 0;
    for (std::size_t e = 0; e < envelopes; ++e) {
        std::vector<UnitVertex> v(6);
        for (int i = 0; i < 6; ++i)
            v[i] = UnitVertex{env[(e * 6 + i) * 4], env[(e * 6 + i) * 4 + 1], env[(e * 6 + i) * 4 + 2],
                              env[(e * 6 + i) * 4 + 3]};
        std::vector<double> values;
        cdet_gb300::evaluate_cdet_density_all_subset_integrands_double_into(v, values);
        if (values.size() != 64) throw std::runtime_error("all-subset integrand returned the wrong size");
        for (std::uint64_t mask = 1; mask < 64; ++mask) {
            std::vector<UnitVertex> subset;
            for (int i = 0; i < 6; ++i)
                if (mask & (std::uint64_t{1} << i)) subset.push_back(v[i]);
            const double direct = cdet_gb300::evaluate_cdet_density_integrand_double(subset);
            const double scale = std::max({1.0, std::abs(direct), std::abs(values[mask])});
            if (!(std::abs(values[mask] - direct) <= 2e-9 + 2e-9 * scale))
                throw std::runtime_error("all-subset hot path differs from independent variable-order evaluation");
            ++checked;
        }
        all_out.insert(all_out.end(), values.begin(), values.end());
    }
    write_all(dir + "/all_out.bin", all_out);
    bool threw = false;
    try {
        cdet_gb300::evaluate_cdet_density_integrand_double({});
    } catch (const std::runtime_error&) {
        threw = true;
    }
    if (!threw) throw std::runtime_error("order 0 did not raise");
    // MCMCMC chains through the C++ class: the reference's histogram-seeded
    // chains of this parameter set (tests/golden/mcmcmc_chains.*), a
    // checkpoint at half the production steps, then the rest
    const auto ints = read_all<int32_t>(dir + "/mc_ints.bin");  // omin omax env interval warmup production half bins
    const auto rate = read_all<double>(dir + "/mc_rate.bin");
    cdet_mcmcmc_config config{ints[0], ints[1], ints[2], ints[3], rate[0]};
    const auto seeds = read_all<uint64_t>(dir + "/mc_seeds.bin");
    cdet_gb300::McmcmcChains chains(gpu, config, seeds, read_all<double>(dir + "/mc_lambdas.bin"));
    chains.set_histogram(ints[7], read_all<double>(dir + "/mc_tau.bin"), read_all<double>(dir + "/mc_space.bin"),
                         read_all<double>(dir + "/mc_replica.bin"));
    cdet_mcmcmc_run_info half{ints[0], ints[4], ints[6]};
    chains.run_to(half, dir + "/ck_half");
    cdet_mcmcmc_run_info full{ints[0], ints[4], ints[5]};
    chains.run_to(full);
    std::vector<double> verts, lambdas;
    std::vector<uint64_t> rng;
    chains.state(verts, lambdas, rng);
    write_all(dir + "/mc_vertices_out.bin", verts);
    write_all(dir + "/mc_lambdas_out.bin", lambdas);
    write_all(dir + "/mc_rng_out.bin", rng);
    std::vector<uint64_t> counts;
    std::vector<double> means;
    const int e1 = config.envelope_order + 1;
    for (int64_t c = 0; c < chains.chains(); ++c) {
        const cdet_mcmcmc_chain_result r = chains.result(c);
        counts.insert(counts.end(), {r.seed, r.warmup_proposed_steps, r.warmup_accepted_steps,
                                     r.production_proposed_steps, r.production_accepted_steps});
        counts.insert(counts.end(), r.warmup_chosen_counts, r.warmup_chosen_counts + e1);
        counts.insert(counts.end(), r.production_chosen_counts, r.production_chosen_counts + e1);
        for (int o = 0; o < e1; ++o) means.push_back(static_cast<double>(r.order_signal_stats[o].mean));
    }
    write_all(dir + "/mc_counts_out.bin", counts);
    write_all(dir + "/mc_means_out.bin", means);
    const cdet_gb300::McmcmcSummary sum = chains.summary(config.order_min);
    std::vector<double> ratios;
    for (long double r : sum.ratios) ratios.push_back(static_cast<double>(r));
    write_all(dir + "/mc_ratios_out.bin", ratios);
    const cdet_mcmcmc_checkpoint ck = cdet_gb300::read_mcmcmc_checkpoint(dir + "/ck_half/chain_000000.chk");
    if (ck.result.production_proposed_steps != static_cast<uint64_t>(ints[6]))
        throw std::runtime_error("the half-way checkpoint has the wrong step count");

    std::printf("PASS adapter_check: %zu single-order, %d subset checks, %lld chains\n", single.size(), checked,
                static_cast<long long>(chains.chains()));
    return 0;
} catch (const std::exception& error) {
    std::fprintf(stderr, "FAIL adapter_check: %s\n", error.what());
    return 1;
}
