"""GPU MCMCMC chains (cdet_mcmcmc_*) against the reference's own chains.

mcmcmc_chains.npz holds 8 reference chains per golden parameter set (the step
loop of run_single_mcmcmc_chain with the uniform seed kernel, lambda
adaptation during warmup; tests/golden/make_mcmcmc_golden.py). The GPU chains,
created from the same seeds and evaluated with the FP64 assembly, must choose
the same mask at every step and end on the same vertices and generator state,
bit for bit. Local normalisations, order signals and adapted lambdas are held
to 2e-16 relative: the adaptation's exp and log run on this host's libm,
which need not round exactly as the reference's did. The same holds for the
histogram-seeded chains (MCMCMC_SEED_MODE=histogram on the reference-learned
probabilities), and the GPU-assisted histogram learning matches the oracle.
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.mcmcmc import McmcmcChains, learn_histogram, mt64_outputs  # noqa: E402
from helpers import GOLDEN, load_case  # noqa: E402

with open(os.path.join(GOLDEN, "mcmcmc_chains.json")) as f:
    RUNS = json.load(f)
GOLD = np.load(os.path.join(GOLDEN, "mcmcmc_chains.npz"))


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


def _close(a, b, rtol=2e-16):
    a, b = np.asarray(a), np.asarray(b)
    return np.all(np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)))


@pytest.mark.parametrize("name", sorted(RUNS))
def test_chains_follow_reference(name):
    run = RUNS[name]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    seeds = GOLD[f"{name}.seeds"]
    chains = McmcmcChains(gpu, run["order_min"], run["order_max"], run["envelope"], seeds, run["lambdas"],
                          run["adapt_interval"], run["adapt_rate"])
    w = chains.run(run["warmup"], warmup=True, record=True)
    chains.end_warmup()
    p = chains.run(run["production"], warmup=False, record=True)
    verts, lams, rng = chains.state()
    chosen = np.concatenate([w["chosen"], p["chosen"]]).T        # [chains][steps]
    norms = np.concatenate([w["norms"], p["norms"]]).T
    signal = p["signal"].transpose(1, 0, 2)                      # [chains][production][env + 1]
    assert np.array_equal(chosen, GOLD[f"{name}.chosen"])
    assert np.array_equal(verts.view(np.uint64), GOLD[f"{name}.vertices"].view(np.uint64))
    for c in range(len(seeds)):
        assert np.array_equal(mt64_outputs(rng[c], 8), GOLD[f"{name}.rng"][c]), c
    assert _close(norms, GOLD[f"{name}.norms"])
    assert _close(signal, GOLD[f"{name}.signal"])
    assert _close(lams, GOLD[f"{name}.lambdas"])
    chains.close()


def test_config_checks():
    params, tables, _ = load_case("column_3x3")
    gpu = CdetIntegrand(params, tables)
    with pytest.raises(RuntimeError, match="ENVELOPE_ORDER must be larger"):
        McmcmcChains(gpu, 1, 4, 4, [1, 2], [0, 1, 1, 1, 1])
    with pytest.raises(RuntimeError, match="LAMBDAS entries must be positive"):
        McmcmcChains(gpu, 1, 2, 4, [1, 2], [0, 1, 0, 1, 1])


@pytest.mark.parametrize("name", sorted(RUNS))
def test_histogram_chains_follow_reference(name):
    """Chains on the reference-learned FactorizedHistogramSeed (the stored
    probabilities), with the conditional generation probabilities in the
    fluxes: the same masks, vertices and generator state as the reference's."""
    run = RUNS[name]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    seeds = GOLD[f"{name}.hist.seeds"]
    chains = McmcmcChains(gpu, run["order_min"], run["order_max"], run["envelope"], seeds, run["lambdas"],
                          run["adapt_interval"], run["adapt_rate"])
    chains.set_histogram(run["histogram"]["tau_bins"], GOLD[f"{name}.hist.tau"], GOLD[f"{name}.hist.space"],
                         GOLD[f"{name}.hist.replica"])
    w = chains.run(run["warmup"], warmup=True, record=True)
    chains.end_warmup()
    p = chains.run(run["production"], warmup=False, record=True)
    verts, lams, rng = chains.state()
    chosen = np.concatenate([w["chosen"], p["chosen"]]).T
    norms = np.concatenate([w["norms"], p["norms"]]).T
    signal = p["signal"].transpose(1, 0, 2)
    assert np.array_equal(chosen, GOLD[f"{name}.hist.chosen"])
    assert np.array_equal(verts.view(np.uint64), GOLD[f"{name}.hist.vertices"].view(np.uint64))
    for c in range(len(seeds)):
        assert np.array_equal(mt64_outputs(rng[c], 8), GOLD[f"{name}.hist.rng"][c]), c
    assert _close(norms, GOLD[f"{name}.hist.norms"])
    assert _close(signal, GOLD[f"{name}.hist.signal"])
    assert _close(lams, GOLD[f"{name}.hist.lambdas"])
    chains.close()


@pytest.mark.parametrize("name", sorted(RUNS))
def test_learned_histogram(name):
    """Histogram learning with the integrands on the GPU: bit-identical to the
    oracle on this machine (both accumulate in this host's long double), and
    to 1e-14 of the reference's x86-64 learning (80-bit long double)."""
    from bindings import Oracle
    run = RUNS[name]
    h = run["histogram"]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    got = learn_histogram(gpu, run["order_min"], run["order_max"], run["envelope"], h["learning_steps"],
                          h["tau_bins"], h["uniform_mix"], h["pseudo_count"], h["learn_seed"])
    want = Oracle(params.runtime_scalars(), tables).learn_histogram(
        run["order_min"], run["order_max"], run["envelope"], h["learning_steps"], h["tau_bins"],
        h["uniform_mix"], h["pseudo_count"], h["learn_seed"])
    for g, w in zip(got[:3], want[:3]):
        assert np.array_equal(np.asarray(g).view(np.uint64), np.asarray(w).view(np.uint64))
    assert np.float64(got[3]).view(np.uint64) == np.float64(want[3]).view(np.uint64)
    for g, key in zip(got[:3], ("tau", "space", "replica")):
        assert _close(g, GOLD[f"{name}.hist.{key}"], 1e-14), key
    assert _close([got[3]], [GOLD[f"{name}.hist.total"]], 1e-14)


def test_histogram_seed_density_error():
    """A negative seed density stops the chains with the reference's message;
    the kernel records the status and returns."""
    params, tables, _ = load_case("column_3x3")
    gpu = CdetIntegrand(params, tables)
    sites = params.n1 * params.n2
    chains = McmcmcChains(gpu, 1, 2, 4, [1, 2], [0, 1, 1, 0, 0])
    chains.set_histogram(2, np.full(4, -0.5), np.full(sites * sites, 1.0 / sites), np.full(4, 0.5))
    with pytest.raises(RuntimeError, match="seed density is negative or non-finite"):
        chains.run(1)
    with pytest.raises(ValueError):
        chains.set_histogram(2, np.full(3, 0.5), np.full(sites * sites, 1.0 / sites), np.full(4, 0.5))
    chains.close()
    with pytest.raises(RuntimeError, match="UNIFORM_MIX must lie in"):
        learn_histogram(gpu, 1, 2, 4, 2, 4, 1.5, 0.0, 1)
