"""Reference MCMCMC chain trajectories (uniform seed kernel) for the device
chain step, from the reference itself.

Run from the repository root with the environment variable REFERENCE set
to the reference checkout, after make_golden.py:

    REFERENCE=<reference checkout> python tests/golden/make_mcmcmc_golden.py

For each golden parameter set it loads the reference-built tables stored in
<name>.npz into the reference build and runs, per chain, the step loop of
run_single_mcmcmc_chain (mcmcmc_sampler.h:994-1088): make_initial_mcmcmc_chain_state
from the chain's seed (derive_mcmcmc_seed, :159-172, with the parallel driver's
stream tag), warmup steps with lambda adaptation, production steps. It records
every step's chosen mask and local normalisation, the production order
signals, the final vertices and lambdas and the next 8 raw generator outputs,
in mcmcmc_chains.npz. A second set of chains per parameter set runs with the
FactorizedHistogramSeed (mcmcmc_seed.h:71-229) that
learn_factorized_histogram_seed (mcmcmc_sampler.h:602-664) learns for the
recorded settings; its row probabilities and total pair weight are stored too
(<name>.hist.*).

Finally, run_mcmcmc_chains_parallel (mcmcmc_sampler.h:1090-1150) itself runs
the same histogram-seeded chains (normalization order = order_min) and its
per-chain MCMCMCChainResult, cross-chain statistics and ratios are stored
(<name>.run.*; long doubles as exact hi/lo pairs of the x86-64 80-bit values).
A run of half the production length writes the reference's V1 checkpoint files
into mcmcmc_checkpoints/<name>/, and a resumed run (MCMCMC_RESUME=require) to
the full length is checked to reproduce the uninterrupted run.
"""
from __future__ import annotations

import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import bindings  # noqa: E402
from make_golden import CASES, REFERENCE  # noqa: E402

KINDS = ("twisted_up", "twisted_down", "ordinary_up", "ordinary_down")
KEYS = ("upper", "lower", "upper_corners", "lower_corners")
STREAM_TAG = 0x4D434D434D435348  # run_mcmcmc_chains_parallel (mcmcmc_sampler.h:1102)
M64 = (1 << 64) - 1

# name -> chain settings
RUNS = {
    "physical_2x2": dict(order_min=1, order_max=3, envelope=5, lambdas=[0.0, 1.0, 0.6, 0.3, 0.0, 0.0],
                         warmup=24, adapt_interval=5, adapt_rate=0.25, production=20, base_seed=20261203),
    "column_3x3": dict(order_min=2, order_max=4, envelope=6, lambdas=[0.0, 0.0, 1.0, 0.5, 0.25, 0.0, 0.0],
                       warmup=16, adapt_interval=4, adapt_rate=0.25, production=24, base_seed=7),
}
CHAINS = 8
HIST = dict(learning_steps=30, tau_bins=4, uniform_mix=0.05, pseudo_count=0.5, learn_seed=99,
            base_seed=424242)


def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def derive_seed(base, tag, index):
    mixed = splitmix64(base ^ tag)
    mixed ^= (0x9E3779B97F4A7C15 * (index + 1)) & M64
    return splitmix64(mixed)


def main():
    bindings.build(REFERENCE)
    ref = bindings.Reference()
    out, meta = {}, {}
    for name, run in RUNS.items():
        data = np.load(os.path.join(HERE, f"{name}.npz"))
        ref.configure(**CASES[name])
        ref.set_tables({k: {key: data[f"table.{k}.{key}"] for key in KEYS} for k in KINDS})
        seeds = [derive_seed(run["base_seed"], STREAM_TAG, i) for i in range(CHAINS)]
        per = [ref.mcmcmc_chain(run["order_min"], run["order_max"], run["envelope"], run["lambdas"],
                                run["warmup"], run["adapt_interval"], run["adapt_rate"], run["production"],
                                s) for s in seeds]
        out[f"{name}.seeds"] = np.array(seeds, dtype=np.uint64)
        for key in ("chosen", "norms", "signal", "vertices", "lambdas", "rng"):
            out[f"{name}.{key}"] = np.stack([p[key] for p in per])
        sites = CASES[name]["n1"] * CASES[name]["n2"]
        tau, space, rep, total = ref.learn_histogram(run["order_min"], run["order_max"], run["envelope"],
                                                     HIST["learning_steps"], HIST["tau_bins"],
                                                     HIST["uniform_mix"], HIST["pseudo_count"],
                                                     HIST["learn_seed"], sites)
        out[f"{name}.hist.tau"], out[f"{name}.hist.space"], out[f"{name}.hist.replica"] = tau, space, rep
        out[f"{name}.hist.total"] = np.array([total])
        hseeds = [derive_seed(HIST["base_seed"], STREAM_TAG, i) for i in range(CHAINS)]
        hper = [ref.mcmcmc_chain(run["order_min"], run["order_max"], run["envelope"], run["lambdas"],
                                 run["warmup"], run["adapt_interval"], run["adapt_rate"], run["production"], s,
                                 histogram=(HIST["tau_bins"], tau, space, rep)) for s in hseeds]
        out[f"{name}.hist.seeds"] = np.array(hseeds, dtype=np.uint64)
        for key in ("chosen", "norms", "signal", "vertices", "lambdas", "rng"):
            out[f"{name}.hist.{key}"] = np.stack([p[key] for p in hper])
        hist = (HIST["tau_bins"], tau, space, rep)
        full = ref.mcmcmc_run(run["order_min"], run["order_max"], run["envelope"], run["order_min"],
                              run["lambdas"], run["warmup"], run["adapt_interval"], run["adapt_rate"],
                              run["production"], CHAINS, HIST["base_seed"], histogram=hist)
        for key, val in full.items():
            out[f"{name}.run.{key}"] = val
        ck_dir = os.path.join(HERE, "mcmcmc_checkpoints", name)
        shutil.rmtree(ck_dir, ignore_errors=True)
        half = run["production"] // 2
        ref.mcmcmc_run(run["order_min"], run["order_max"], run["envelope"], run["order_min"], run["lambdas"],
                       run["warmup"], run["adapt_interval"], run["adapt_rate"], half, CHAINS, HIST["base_seed"],
                       histogram=hist, checkpoint_dir=ck_dir)
        with tempfile.TemporaryDirectory() as tmp:
            resume_dir = os.path.join(tmp, name)
            shutil.copytree(ck_dir, resume_dir)
            resumed = ref.mcmcmc_run(run["order_min"], run["order_max"], run["envelope"], run["order_min"],
                                     run["lambdas"], run["warmup"], run["adapt_interval"], run["adapt_rate"],
                                     run["production"], CHAINS, HIST["base_seed"], histogram=hist,
                                     checkpoint_dir=resume_dir, resume_mode="require")
        for key in full:
            assert np.array_equal(np.asarray(full[key]).view(np.uint64), np.asarray(resumed[key]).view(np.uint64)), key
        meta[name] = dict(run, histogram=HIST, checkpoint_production=half, chains=CHAINS)
    np.savez_compressed(os.path.join(HERE, "mcmcmc_chains.npz"), **out)
    with open(os.path.join(HERE, "mcmcmc_chains.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
