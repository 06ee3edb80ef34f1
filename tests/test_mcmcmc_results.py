"""MCMCMC production statistics and checkpoint files, on the CPU.

mcmcmc_chains.npz holds, per golden parameter set, the result of the
reference's run_mcmcmc_chains_parallel (mcmcmc_sampler.h:1090-1150) over 8
histogram-seeded chains: per-chain MCMCMCChainResult (chosen counts, running
statistics of the retained fraction and of order_signal / lambda in long
double), the cross-chain statistics and the ratios to the normalisation
order. The long doubles are stored as exact (hi, lo) pairs of the x86-64
80-bit values. Recomputing the statistics in np.longdouble from the oracle's
chains (the same chains, step for step) must give them bit for bit where
numpy's long double is that 80-bit format, and to 1e-15 elsewhere.

tests/golden/mcmcmc_checkpoints/<name>/ holds the reference's V1 checkpoint
files after half the production steps; the library's host-only reader and
writer (cdet_read_mcmcmc_checkpoint / cdet_write_mcmcmc_checkpoint) must read
them and write them back byte for byte.
"""
import filecmp
import json
import os

import numpy as np
import pytest

from bindings import Oracle
from helpers import GOLDEN, load_case

with open(os.path.join(GOLDEN, "mcmcmc_chains.json")) as f:
    RUNS = json.load(f)
GOLD = np.load(os.path.join(GOLDEN, "mcmcmc_chains.npz"))
X87 = np.finfo(np.longdouble).nmant == 63  # numpy's long double is the format the fixtures were written in
CKPT = os.path.join(GOLDEN, "mcmcmc_checkpoints")


def ld(pair):
    """An exact (hi, lo) pair as np.longdouble."""
    return np.longdouble(pair[..., 0]) + np.longdouble(pair[..., 1])


def welford(values):
    count, mean, m2 = 0, np.longdouble(0), np.longdouble(0)
    for v in values:
        count += 1
        delta = np.longdouble(v) - mean
        mean += delta / np.longdouble(count)
        m2 += delta * (np.longdouble(v) - mean)
    return count, mean, m2


def same(a, b, rtol=1e-15):
    a, b = np.asarray(a, dtype=np.longdouble), np.asarray(b, dtype=np.longdouble)
    if X87:
        return np.array_equal(a, b)
    return bool(np.all(np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b))))


@pytest.mark.parametrize("name", sorted(RUNS))
def test_chain_statistics_match_reference(name):
    run = RUNS[name]
    params, tables, _ = load_case(name)
    orc = Oracle(params.runtime_scalars(), tables)
    env, omin, omax = run["envelope"], run["order_min"], run["order_max"]
    hist = (run["histogram"]["tau_bins"], GOLD[f"{name}.hist.tau"], GOLD[f"{name}.hist.space"],
            GOLD[f"{name}.hist.replica"])
    u64, stats = GOLD[f"{name}.run.u64"], GOLD[f"{name}.run.stats"]
    means = {o: [] for o in range(omin, omax + 1)}
    for c, seed in enumerate(GOLD[f"{name}.hist.seeds"]):
        assert int(u64[c, 0]) == int(seed)
        got = orc.mcmcmc_chain(omin, omax, env, run["lambdas"], run["warmup"], run["adapt_interval"],
                               run["adapt_rate"], run["production"], int(seed), histogram=hist)
        orders = np.array([bin(int(m)).count("1") for m in got["chosen"]])
        w, p = orders[:run["warmup"]], orders[run["warmup"]:]
        assert list(u64[c, 1:5]) == [run["warmup"], run["warmup"], run["production"], run["production"]]
        assert np.array_equal(u64[c, 5:5 + env + 1], np.bincount(w, minlength=env + 1))
        assert np.array_equal(u64[c, 5 + env + 1:], np.bincount(p, minlength=env + 1))
        for k, seq in ((0, w), (1, p)):
            count, mean, m2 = welford(np.longdouble(seq) / np.longdouble(env))
            assert stats[c, k, 0] == count
            assert same(mean, ld(stats[c, k, 1:3])) and same(m2, ld(stats[c, k, 3:5])), (c, k)
        for o in range(omin, omax + 1):
            count, mean, m2 = welford(got["signal"][:, o] / got["lambdas"][o])
            assert stats[c, 2 + o, 0] == count
            assert same(mean, ld(stats[c, 2 + o, 1:3])) and same(m2, ld(stats[c, 2 + o, 3:5])), (c, o)
            means[o].append(mean)
    cross, ratios = GOLD[f"{name}.run.cross"], GOLD[f"{name}.run.ratios"]
    for o in range(omin, omax + 1):
        count, mean, m2 = welford(means[o])
        assert cross[o, 0] == count
        assert same(mean, ld(cross[o, 1:3])) and same(m2, ld(cross[o, 3:5]))
        ref_mean = welford(means[omin])[1]
        assert same(mean / ref_mean, ld(ratios[o]))


def _checkpoint_files():
    return sorted((name, f) for name in sorted(RUNS) for f in os.listdir(os.path.join(CKPT, name)))


@pytest.mark.parametrize("name,fname", _checkpoint_files())
def test_checkpoint_round_trip(name, fname, tmp_path):
    from cdet_gb300.mcmcmc import read_checkpoint, write_checkpoint
    src = os.path.join(CKPT, name, fname)
    ck = read_checkpoint(src)
    run = RUNS[name]
    c = int(fname[6:12])
    assert ck.chain_index == c and ck.seed == int(GOLD[f"{name}.hist.seeds"][c])
    assert (ck.order_min, ck.order_max, ck.envelope_order) == (run["order_min"], run["order_max"], run["envelope"])
    assert ck.seed_mode == b"histogram" and ck.production_steps == run["checkpoint_production"]
    assert ck.result.production_proposed_steps == run["checkpoint_production"]
    assert ck.result.warmup_proposed_steps == run["warmup"]
    dst = str(tmp_path / fname)
    write_checkpoint(dst, ck)
    assert not os.path.exists(dst + ".tmp")
    if X87:
        assert filecmp.cmp(src, dst, shallow=False)
    else:
        back = read_checkpoint(dst)
        assert bytes(back.rng_state) == bytes(ck.rng_state) and bytes(back.vertices) == bytes(ck.vertices)


def test_checkpoint_reader_errors(tmp_path):
    from cdet_gb300.mcmcmc import read_checkpoint
    src = os.path.join(CKPT, "column_3x3", "chain_000000.chk")
    text = open(src).read()
    bad = tmp_path / "bad.chk"
    bad.write_text(text.replace("warmup_block_counts", "warmup_blocks"))
    with pytest.raises(RuntimeError, match="expected label warmup_block_counts but found warmup_blocks"):
        read_checkpoint(str(bad))
    bad.write_text(text.replace("CDET_MCMCMC_CHAIN_CHECKPOINT_V1", "CDET_MCMCMC_CHAIN_CHECKPOINT_V0"))
    with pytest.raises(RuntimeError, match="Unsupported MCMCMC checkpoint format"):
        read_checkpoint(str(bad))
    bad.write_text(text.replace("\nEND\n", "\nFIN\n"))
    with pytest.raises(RuntimeError, match="Malformed MCMCMC checkpoint footer"):
        read_checkpoint(str(bad))
    with pytest.raises(RuntimeError, match="Could not open MCMCMC checkpoint"):
        read_checkpoint(str(tmp_path / "missing.chk"))
