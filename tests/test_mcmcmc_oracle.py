"""The MCMCMC chain step's C restatement against reference trajectories.

mcmcmc_chains.npz holds, per golden parameter set, 8 chains of the reference's
step loop (run_single_mcmcmc_chain, mcmcmc_sampler.h:994-1088, uniform seed
kernel, lambda adaptation during warmup) written by
tests/golden/make_mcmcmc_golden.py. The oracle must reproduce every chosen
mask, local normalisation and order signal, the final vertices and lambdas and
the generator state bit for bit: the integrand, the mt19937_64 stream, the
libstdc++ distributions and the glibc exp/log of the adaptation all match.
"""
import json
import os

import numpy as np
import pytest

from bindings import Oracle
from helpers import GOLDEN, load_case

with open(os.path.join(GOLDEN, "mcmcmc_chains.json")) as f:
    RUNS = json.load(f)
GOLD = np.load(os.path.join(GOLDEN, "mcmcmc_chains.npz"))


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", sorted(RUNS))
def test_chains_bit_identical(name):
    run = RUNS[name]
    params, tables, _ = load_case(name)
    orc = Oracle(params.runtime_scalars(), tables)
    for c, seed in enumerate(GOLD[f"{name}.seeds"]):
        got = orc.mcmcmc_chain(run["order_min"], run["order_max"], run["envelope"], run["lambdas"], run["warmup"],
                               run["adapt_interval"], run["adapt_rate"], run["production"], int(seed))
        assert np.array_equal(got["chosen"], GOLD[f"{name}.chosen"][c]), c
        for key in ("norms", "signal", "vertices", "lambdas"):
            assert np.array_equal(_bits(got[key]), _bits(GOLD[f"{name}.{key}"][c])), (c, key)
        assert np.array_equal(got["rng"], GOLD[f"{name}.rng"][c]), c


@pytest.mark.parametrize("name", sorted(RUNS))
def test_learned_histogram_bit_identical(name):
    run = RUNS[name]
    h = run["histogram"]
    params, tables, _ = load_case(name)
    orc = Oracle(params.runtime_scalars(), tables)
    tau, space, rep, total = orc.learn_histogram(run["order_min"], run["order_max"], run["envelope"],
                                                 h["learning_steps"], h["tau_bins"], h["uniform_mix"],
                                                 h["pseudo_count"], h["learn_seed"])
    for key, got in (("tau", tau), ("space", space), ("replica", rep)):
        assert np.array_equal(_bits(got), _bits(GOLD[f"{name}.hist.{key}"])), key
    assert _bits([total])[0] == _bits(GOLD[f"{name}.hist.total"])[0]


@pytest.mark.parametrize("name", sorted(RUNS))
def test_histogram_chains_bit_identical(name):
    run = RUNS[name]
    params, tables, _ = load_case(name)
    orc = Oracle(params.runtime_scalars(), tables)
    hist = (run["histogram"]["tau_bins"], GOLD[f"{name}.hist.tau"], GOLD[f"{name}.hist.space"],
            GOLD[f"{name}.hist.replica"])
    for c, seed in enumerate(GOLD[f"{name}.hist.seeds"]):
        got = orc.mcmcmc_chain(run["order_min"], run["order_max"], run["envelope"], run["lambdas"], run["warmup"],
                               run["adapt_interval"], run["adapt_rate"], run["production"], int(seed),
                               histogram=hist)
        assert np.array_equal(got["chosen"], GOLD[f"{name}.hist.chosen"][c]), c
        for key in ("norms", "signal", "vertices", "lambdas"):
            assert np.array_equal(_bits(got[key]), _bits(GOLD[f"{name}.hist.{key}"][c])), (c, key)
        assert np.array_equal(got["rng"], GOLD[f"{name}.hist.rng"][c]), c
