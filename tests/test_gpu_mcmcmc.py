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


X87 = np.finfo(np.longdouble).nmant == 63  # the fixtures' long double format
CKPT = os.path.join(GOLDEN, "mcmcmc_checkpoints")


def _ld(pair):
    return np.longdouble(pair[..., 0]) + np.longdouble(pair[..., 1])


def _same_ld(a, b, rtol=1e-15):
    """Exact where this host's long double is the fixtures' x87 format; else
    to rtol (the reference's aarch64 build rounds its long doubles in quad)."""
    a, b = np.asarray(a, dtype=np.longdouble), np.asarray(b, dtype=np.longdouble)
    if X87:
        return np.array_equal(a, b)
    return bool(np.all(np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b))))


def _welford(values):
    count, mean, m2 = 0, np.longdouble(0), np.longdouble(0)
    for v in values:
        count += 1
        delta = np.longdouble(v) - mean
        mean += delta / np.longdouble(count)
        m2 += delta * (np.longdouble(v) - mean)
    return count, mean, m2


def _hist_chains(name, gpu):
    run = RUNS[name]
    chains = McmcmcChains(gpu, run["order_min"], run["order_max"], run["envelope"], GOLD[f"{name}.hist.seeds"],
                          run["lambdas"], run["adapt_interval"], run["adapt_rate"])
    chains.set_histogram(run["histogram"]["tau_bins"], GOLD[f"{name}.hist.tau"], GOLD[f"{name}.hist.space"],
                         GOLD[f"{name}.hist.replica"])
    return chains


def _check_results(name, res):
    run = RUNS[name]
    env = run["envelope"]
    u64, stats = GOLD[f"{name}.run.u64"], GOLD[f"{name}.run.stats"]
    assert np.array_equal(res["seed"], u64[:, 0])
    for k, field in enumerate(("warmup_proposed_steps", "warmup_accepted_steps", "production_proposed_steps",
                               "production_accepted_steps")):
        assert np.array_equal(res[field], u64[:, 1 + k]), field
    assert np.array_equal(res["warmup_chosen_counts"][:, :env + 1], u64[:, 5:6 + env])
    assert np.array_equal(res["production_chosen_counts"][:, :env + 1], u64[:, 6 + env:])
    for k, field in enumerate(("warmup_retained_fraction_stats", "production_retained_fraction_stats")):
        assert np.array_equal(res[field]["count"], stats[:, k, 0])
        assert _same_ld(res[field]["mean"], _ld(stats[:, k, 1:3])), field
        assert _same_ld(res[field]["m2"], _ld(stats[:, k, 3:5])), field
    sig = res["order_signal_stats"][:, :env + 1]
    assert np.array_equal(sig["count"], stats[:, 2:, 0])
    assert _same_ld(sig["mean"], _ld(stats[:, 2:, 1:3]))
    assert _same_ld(sig["m2"], _ld(stats[:, 2:, 3:5]))


@pytest.mark.parametrize("name", sorted(RUNS))
def test_chain_results_match_reference(name):
    """MCMCMCChainResult of every chain, the cross-chain summary and the
    absolute estimates, against run_mcmcmc_chains_parallel's, and bit for bit
    against np.longdouble on this host from the chains' own order signals."""
    run = RUNS[name]
    omin, omax, env = run["order_min"], run["order_max"], run["envelope"]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    chains = _hist_chains(name, gpu)
    chains.run(run["warmup"], warmup=True)
    chains.end_warmup()
    p = chains.run(run["production"], warmup=False, record=True)
    _, lams, _ = chains.state()
    res = chains.results()
    _check_results(name, res)
    means = {}
    for o in range(omin, omax + 1):
        means[o] = []
        for c in range(chains.chains):
            count, mean, m2 = _welford(p["signal"][:, c, o] / lams[c, o])
            st = res["order_signal_stats"][c, o]
            assert st["count"] == count and st["mean"] == mean and st["m2"] == m2, (c, o)
            means[o].append(mean)
    cross, ratios = chains.summary(omin)
    for o in range(omin, omax + 1):
        count, mean, m2 = _welford(means[o])
        assert cross[o]["count"] == count and cross[o]["mean"] == mean and cross[o]["m2"] == m2
        assert ratios[o] == mean / _welford(means[omin])[1]
        assert _same_ld(cross[o]["mean"], _ld(GOLD[f"{name}.run.cross"][o, 1:3]))
        assert _same_ld(ratios[o], _ld(GOLD[f"{name}.run.ratios"][o]))
    if omin <= 1:
        est = chains.estimates(0.0625, 0.0)
        c1 = cross[1]
        se1 = np.sqrt(c1["m2"] / np.longdouble(c1["count"] - 1) / np.longdouble(c1["count"]))
        const = np.longdouble(0.0625) / c1["mean"]
        assert est["normalization"] == const
        assert est["normalization_stderr"] == abs(np.longdouble(0.0625) * se1 / (c1["mean"] * c1["mean"]))
        assert est["estimate"][1] == np.longdouble(0.0625)
        for o in range(2, omax + 1):
            assert est["estimate"][o] == const * cross[o]["mean"]
    else:
        with pytest.raises(RuntimeError, match="order 1"):
            chains.estimates(0.0625)
    launches, graph_steps = chains.launch_count()
    # the first step of each (vertex buffer, warmup) kind is direct, the rest are graph replays
    assert graph_steps >= run["warmup"] + run["production"] - 4
    assert launches >= 3 * (run["warmup"] + run["production"])
    chains.close()


@pytest.mark.parametrize("name", sorted(RUNS))
def test_checkpoints_match_reference(name, tmp_path):
    """After half the production steps the chains' checkpoints hold what the
    reference's do (exact state; long double statistics as above)."""
    from cdet_gb300.mcmcmc import read_checkpoint
    run = RUNS[name]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    chains = _hist_chains(name, gpu)
    half = run["checkpoint_production"]
    chains.run_to(run["warmup"], half, run["order_min"], checkpoint_dir=str(tmp_path))
    for fname in sorted(os.listdir(os.path.join(CKPT, name))):
        ref = read_checkpoint(os.path.join(CKPT, name, fname))
        got = read_checkpoint(str(tmp_path / fname))
        for field in ("chain_index", "seed", "order_min", "order_max", "envelope_order", "normalization_order",
                      "lambda_warmup_steps", "production_steps", "seed_mode"):
            assert getattr(got, field) == getattr(ref, field), (fname, field)
        for field in ("rng_state", "lambdas", "warmup_block_counts", "vertices"):
            assert bytes(getattr(got, field)) == bytes(getattr(ref, field)), (fname, field)
        if X87:
            assert bytes(got.result) == bytes(ref.result)
    chains.close()


@pytest.mark.parametrize("name", sorted(RUNS))
def test_resume_from_reference_checkpoints(name):
    """Chains restored from the reference's checkpoint files and run to the
    full length end where the reference's uninterrupted run ends."""
    run = RUNS[name]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    chains = _hist_chains(name, gpu)
    n = chains.load_checkpoints(os.path.join(CKPT, name), run["order_min"], run["warmup"], run["production"],
                                require=True)
    assert n == chains.chains
    chains.run_to(run["warmup"], run["production"], run["order_min"])
    verts, lams, rng = chains.state()
    assert np.array_equal(verts.view(np.uint64), GOLD[f"{name}.hist.vertices"].view(np.uint64))
    for c in range(chains.chains):
        assert np.array_equal(mt64_outputs(rng[c], 8), GOLD[f"{name}.hist.rng"][c]), c
    assert np.array_equal(lams.view(np.uint64), GOLD[f"{name}.run.lambdas"].view(np.uint64))
    _check_results(name, chains.results())
    chains.close()


def test_resume_checks():
    run = RUNS["column_3x3"]
    params, tables, _ = load_case("column_3x3")
    gpu = CdetIntegrand(params, tables)
    chains = _hist_chains("column_3x3", gpu)
    with pytest.raises(RuntimeError, match="does not match current run settings"):
        chains.load_checkpoints(os.path.join(CKPT, "column_3x3"), run["order_min"], run["warmup"] + 1,
                                run["production"])
    with pytest.raises(RuntimeError, match="MCMCMC_RESUME=require but checkpoint is missing for chain 0"):
        chains.load_checkpoints(os.path.join(CKPT, "physical_2x2", "none"), run["order_min"], run["warmup"],
                                run["production"], require=True)
    chains.close()


def test_graphs_follow_context_changes():
    """The step graphs are dropped and captured again when the context's
    buffers change between steps (a larger evaluation on the same context
    reallocates its scratch); the chains still follow the reference's."""
    name = "column_3x3"
    run = RUNS[name]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    seeds = GOLD[f"{name}.seeds"]
    chains = McmcmcChains(gpu, run["order_min"], run["order_max"], run["envelope"], seeds, run["lambdas"],
                          run["adapt_interval"], run["adapt_rate"])
    first = chains.run(7, warmup=True, record=True)
    rng = np.random.default_rng(3)
    gpu.integrand_batch(rng.random((3000, 8, 4)), [8] * 3000)
    rest = chains.run(run["warmup"] - 7, warmup=True, record=True)
    chains.end_warmup()
    p = chains.run(run["production"], warmup=False, record=True)
    chosen = np.concatenate([first["chosen"], rest["chosen"], p["chosen"]]).T
    assert np.array_equal(chosen, GOLD[f"{name}.chosen"])
    verts, _, _ = chains.state()
    assert np.array_equal(verts.view(np.uint64), GOLD[f"{name}.vertices"].view(np.uint64))
    chains.close()


@pytest.mark.parametrize("hist", [False, True])
def test_large_batch_step_path(hist):
    """From 2048 chains the step runs one thread per chain (after the
    warp-per-chain conditional probabilities for the histogram seed); chains
    are independent, so the first 8 chains of a 2048-chain batch seeded like
    the reference's must still be the reference's chains."""
    name = "column_3x3"
    run = RUNS[name]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    key = f"{name}.hist" if hist else name
    seeds = np.concatenate([GOLD[f"{key}.seeds"], np.arange(1, 2041, dtype=np.uint64) * np.uint64(7919)])
    chains = McmcmcChains(gpu, run["order_min"], run["order_max"], run["envelope"], seeds, run["lambdas"],
                          run["adapt_interval"], run["adapt_rate"])
    if hist:
        chains.set_histogram(run["histogram"]["tau_bins"], GOLD[f"{key}.tau"], GOLD[f"{key}.space"],
                             GOLD[f"{key}.replica"])
    w = chains.run(run["warmup"], warmup=True, record=True)
    chains.end_warmup()
    p = chains.run(run["production"], warmup=False, record=True)
    verts, _, rng = chains.state()
    chosen = np.concatenate([w["chosen"], p["chosen"]]).T[:8]
    assert np.array_equal(chosen, GOLD[f"{key}.chosen"])
    assert np.array_equal(verts[:8].view(np.uint64), GOLD[f"{key}.vertices"].view(np.uint64))
    for c in range(8):
        assert np.array_equal(mt64_outputs(rng[c], 8), GOLD[f"{key}.rng"][c]), c
    assert _close(p["signal"].transpose(1, 0, 2)[:8], GOLD[f"{key}.signal"])
    chains.close()


def _same_fields(a, b) -> bool:
    if a.dtype.names is None:
        return np.array_equal(a, b)
    return all(_same_fields(a[n], b[n]) for n in a.dtype.names)


def test_ring_wraps_and_call_boundaries():
    """1,100 production steps (the step-output ring holds two halves of 256
    steps for a small batch): one call and eleven calls of 100 steps record the
    same steps, end in the same state and results, and choose the oracle
    chain's masks step for step."""
    from bindings import Oracle
    name = "physical_2x2"
    run = RUNS[name]
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    seeds = GOLD[f"{name}.seeds"][:4]
    steps = 1100
    outs, states, results = [], [], []
    for calls in (1, 11):
        chains = McmcmcChains(gpu, run["order_min"], run["order_max"], run["envelope"], seeds, run["lambdas"],
                              run["adapt_interval"], run["adapt_rate"])
        rec = [chains.run(steps // calls, warmup=False, record=True) for _ in range(calls)]
        outs.append({k: np.concatenate([r[k] for r in rec]) for k in ("chosen", "norms", "signal")})
        states.append(chains.state())
        results.append(chains.results())
        chains.close()
    for k in ("chosen", "norms", "signal"):
        assert np.array_equal(outs[0][k].view(np.uint64) if k != "chosen" else outs[0][k],
                              outs[1][k].view(np.uint64) if k != "chosen" else outs[1][k]), k
    for a, b in zip(states[0], states[1]):
        assert np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))
    assert _same_fields(results[0], results[1])  # field by field: struct padding carries no data
    assert np.all(results[0]["production_proposed_steps"] == steps)
    orc = Oracle(params.runtime_scalars(), tables)
    for c, seed in enumerate(seeds):
        want = orc.mcmcmc_chain(run["order_min"], run["order_max"], run["envelope"], run["lambdas"], 0,
                                run["adapt_interval"], run["adapt_rate"], steps, int(seed))
        assert np.array_equal(outs[0]["chosen"][:, c], want["chosen"]), c


@pytest.mark.parametrize("assembly", ["fp64", "split"])
def test_green_reuse_keeps_chains_bit_identical(assembly):
    """Green-pair reuse across steps (the default) against every pair
    evaluated each step: the same chosen masks, local normalisations and
    order signals at every step, and the same final vertices and generator
    states, bit for bit, for both assemblies."""
    name = "physical_2x2"
    run = RUNS[name]
    params, tables, _ = load_case(name)
    seeds = np.arange(1, 97, dtype=np.uint64) * 7919
    outs = []
    for reuse in (False, True):
        gpu = CdetIntegrand(params, tables)
        gpu.set_assembly(assembly)
        chains = McmcmcChains(gpu, run["order_min"], run["order_max"], run["envelope"], seeds, run["lambdas"],
                              run["adapt_interval"], run["adapt_rate"])
        chains.set_green_reuse(reuse)
        w = chains.run(40, warmup=True, record=True)
        chains.end_warmup()
        p = chains.run(60, warmup=False, record=True)
        verts, lams, rng = chains.state()
        outs.append((w, p, verts, lams, rng))
        chains.close()
    (w0, p0, v0, l0, r0), (w1, p1, v1, l1, r1) = outs
    for key in ("chosen", "norms", "signal"):
        a = np.concatenate([w0[key], p0[key]]) if key != "signal" else p0[key]
        b = np.concatenate([w1[key], p1[key]]) if key != "signal" else p1[key]
        assert np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64)), key
    assert np.array_equal(v0.view(np.uint64), v1.view(np.uint64))
    assert np.array_equal(l0.view(np.uint64), l1.view(np.uint64))
    assert np.array_equal(r0, r1)
    # every step retains the chosen order's vertices (order_min >= 1), so the copies ran
    kept = np.vectorize(lambda m: bin(int(m)).count("1"))(np.asarray(p1["chosen"]))
    assert kept.min() >= run["order_min"] and kept.mean() > 1.0
