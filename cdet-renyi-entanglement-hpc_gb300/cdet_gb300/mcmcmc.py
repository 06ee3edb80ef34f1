"""MCMCMC chains resident on the GPU (uniform or factorized histogram seed).

The batch counterpart of run_single_mcmcmc_chain (mcmcmc_sampler.h:994-1088):
every step evaluates the all-subset integrand of each chain's envelope on the
GPU and runs run_mcmcmc_step (:524-577) in one thread per chain, with each
chain's std::mt19937_64 stream reproduced on the device. With the FP64
assembly the chains are the reference's chains, step for step.
`learn_histogram` is learn_factorized_histogram_seed (:607-664) and
`McmcmcChains.set_histogram` switches the chains to that seed kernel
(MCMCMC_SEED_MODE=histogram). Every step also updates each chain's
MCMCMCChainResult (`results`); `summary` and `estimates` are the reference's
cross-chain aggregation (:1118-1146) and absolute estimates (main.cpp:831-870);
`save_checkpoints` / `load_checkpoints` read and write the reference's V1
checkpoint files, and `run_to` is run_single_mcmcmc_chain's loop (:994-1088)
for the whole batch.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import lib as L
from .integrand import CdetIntegrand

STREAM_TAG = 0x4D434D434D435348  # run_mcmcmc_chains_parallel's seed stream (mcmcmc_sampler.h:1102)


class McmcmcChains:
    def __init__(self, integrand: CdetIntegrand, order_min: int, order_max: int, envelope: int,
                 seeds: Sequence[int], lambdas: Sequence[float], adapt_interval: int = 1000,
                 adapt_rate: float = 0.25):
        self._lib = integrand._lib
        self._integrand = integrand  # keeps the context alive
        self.envelope = int(envelope)
        self.chains = len(seeds)
        cfg = L.McmcmcConfig(order_min, order_max, envelope, adapt_interval, adapt_rate)
        s = np.ascontiguousarray(seeds, dtype=np.uint64)
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        if lam.size != envelope + 1:
            raise ValueError("lambdas needs envelope + 1 entries (index = order)")
        self._h = C.c_void_p()
        L.check(self._lib.cdet_mcmcmc_create(integrand._ctx, C.byref(cfg), self.chains,
                                             s.ctypes.data_as(C.POINTER(C.c_uint64)),
                                             lam.ctypes.data_as(C.POINTER(C.c_double)), C.byref(self._h)))

    def run(self, steps: int, warmup: bool = False, record: bool = False) -> Optional[dict]:
        """Advances every chain `steps` steps; with record=True returns the
        per-step chosen masks [steps][chains], local normalisations and raw
        order signals [steps][chains][envelope + 1]."""
        up, dp = C.POINTER(C.c_uint64), C.POINTER(C.c_double)
        if record:
            chosen = np.zeros((steps, self.chains), dtype=np.uint64)
            norms = np.zeros((steps, self.chains))
            signal = np.zeros((steps, self.chains, self.envelope + 1))
            L.check(self._lib.cdet_mcmcmc_run(self._h, int(warmup), steps, chosen.ctypes.data_as(up),
                                              norms.ctypes.data_as(dp), signal.ctypes.data_as(dp)))
            return dict(chosen=chosen, norms=norms, signal=signal)
        L.check(self._lib.cdet_mcmcmc_run(self._h, int(warmup), steps, None, None, None))
        return None

    def set_histogram(self, tau_bins: int, tau, space, replica) -> None:
        """Seed later steps with the FactorizedHistogramSeed of these row
        probabilities: tau [bins][bins], space [N1 N2][N1 N2], replica [2][2]."""
        sites = self._integrand.params.n1 * self._integrand.params.n2
        arrs = []
        for x, n in ((tau, tau_bins * tau_bins), (space, sites * sites), (replica, 4)):
            a = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
            if a.size != n:
                raise ValueError("histogram probabilities have the wrong size")
            arrs.append(a)
        dp = C.POINTER(C.c_double)
        L.check(self._lib.cdet_mcmcmc_set_histogram(self._h, int(tau_bins), *(a.ctypes.data_as(dp) for a in arrs)))

    def results(self) -> np.ndarray:
        """Every chain's MCMCMCChainResult as a structured array (fields as in
        cdet_mcmcmc_chain_result; running statistics with count, mean, m2 in
        the host's long double)."""
        arr = (L.ChainResult * self.chains)()
        for c in range(self.chains):
            L.check(self._lib.cdet_mcmcmc_result(self._h, c, C.byref(arr[c])))
        return np.frombuffer(arr, dtype=result_dtype()).copy()

    def summary(self, normalization_order: int):
        """(cross-chain running statistics [envelope + 1], ratios to the
        normalisation order [envelope + 1] as np.longdouble)."""
        e1 = self.envelope + 1
        cross = (L.RunningStats * e1)()
        ratios = (C.c_longdouble * e1)()
        L.check(self._lib.cdet_mcmcmc_summary(self._h, int(normalization_order), cross, ratios))
        return (np.frombuffer(cross, dtype=stats_dtype()).copy(),
                np.frombuffer(ratios, dtype=np.longdouble).copy())

    def estimates(self, order1_hi: float, order1_lo: float = 0.0) -> dict:
        """Absolute estimates normalised by the deterministic order-1 value."""
        e1 = self.envelope + 1
        const, const_err = C.c_longdouble(), C.c_longdouble()
        est, err = (C.c_longdouble * e1)(), (C.c_longdouble * e1)()
        L.check(self._lib.cdet_mcmcmc_estimates(self._h, float(order1_hi), float(order1_lo), C.byref(const),
                                                C.byref(const_err), est, err))
        return dict(normalization=_ld(const), normalization_stderr=_ld(const_err),
                    estimate=np.frombuffer(est, dtype=np.longdouble).copy(),
                    stderr=np.frombuffer(err, dtype=np.longdouble).copy())

    def save_checkpoints(self, directory: str, normalization_order: int, lambda_warmup_steps: int,
                         production_steps: int) -> None:
        info = L.RunInfo(normalization_order, lambda_warmup_steps, production_steps)
        L.check(self._lib.cdet_mcmcmc_save_checkpoints(self._h, os.fsencode(directory), C.byref(info)))

    def load_checkpoints(self, directory: str, normalization_order: int, lambda_warmup_steps: int,
                         production_steps: int, require: bool = False) -> int:
        """Restores the chains that have a checkpoint in `directory`; returns
        how many did."""
        info = L.RunInfo(normalization_order, lambda_warmup_steps, production_steps)
        restored = C.c_int64()
        L.check(self._lib.cdet_mcmcmc_load_checkpoints(self._h, os.fsencode(directory), C.byref(info),
                                                       int(require), C.byref(restored)))
        return restored.value

    def set_green_reuse(self, enable: bool) -> None:
        """Green-pair reuse across steps (default on): pairs of retained
        vertices are copied from the previous step's Green matrices; the
        chains are the same bit for bit either way."""
        L.check(self._lib.cdet_mcmcmc_set_green_reuse(self._h, int(bool(enable))))

    def launch_count(self) -> tuple:
        """(kernels launched by the runs so far, steps replayed from a CUDA graph)."""
        n, g = C.c_int64(), C.c_int64()
        L.check(self._lib.cdet_mcmcmc_launch_count(self._h, C.byref(n), C.byref(g)))
        return n.value, g.value

    def run_to(self, lambda_warmup_steps: int, production_steps: int, normalization_order: int,
               checkpoint_dir: Optional[str] = None, checkpoint_interval: int = 0) -> None:
        """run_single_mcmcmc_chain's loop for the batch: the remaining warmup
        steps, the adaptation of a partial last block, the remaining
        production steps; with checkpoint_dir, checkpoints whenever the
        completed steps reach a multiple of checkpoint_interval (if > 0) and at
        the end."""
        res = self.results()
        done = int(res["warmup_proposed_steps"][0] + res["production_proposed_steps"][0])

        def save():
            if checkpoint_dir:
                self.save_checkpoints(checkpoint_dir, normalization_order, lambda_warmup_steps, production_steps)

        def advance(steps: int, warmup: bool) -> None:
            nonlocal done
            while steps > 0:
                chunk = steps
                if checkpoint_dir and checkpoint_interval > 0:
                    chunk = min(chunk, checkpoint_interval - done % checkpoint_interval)
                self.run(chunk, warmup=warmup)
                done += chunk
                steps -= chunk
                if checkpoint_dir and checkpoint_interval > 0 and done % checkpoint_interval == 0:
                    save()

        advance(max(0, lambda_warmup_steps - int(res["warmup_proposed_steps"][0])), True)
        self.end_warmup()
        advance(max(0, production_steps - int(res["production_proposed_steps"][0])), False)
        save()

    def end_warmup(self) -> None:
        L.check(self._lib.cdet_mcmcmc_end_warmup(self._h))

    def state(self):
        """(vertices [chains][envelope][4], lambdas [chains][envelope + 1],
        rng_state [chains][313]: mt19937_64 words and position)."""
        v = np.zeros((self.chains, self.envelope, 4))
        lam = np.zeros((self.chains, self.envelope + 1))
        rng = np.zeros((self.chains, 313), dtype=np.uint64)
        L.check(self._lib.cdet_mcmcmc_state(self._h, v.ctypes.data_as(C.POINTER(C.c_double)),
                                            lam.ctypes.data_as(C.POINTER(C.c_double)),
                                            rng.ctypes.data_as(C.POINTER(C.c_uint64))))
        return v, lam, rng

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.cdet_mcmcmc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ld(x: C.c_longdouble) -> np.longdouble:
    """A ctypes long double as np.longdouble, every bit kept."""
    return np.frombuffer(bytes(x), dtype=np.longdouble)[0]


def stats_dtype() -> np.dtype:
    """cdet_running_stats as a numpy structured type."""
    if np.dtype(np.longdouble).itemsize != C.sizeof(C.c_longdouble):
        raise RuntimeError("numpy's long double does not match the C long double")
    R = L.RunningStats
    return np.dtype({"names": ["count", "mean", "m2"], "formats": [np.uint64, np.longdouble, np.longdouble],
                     "offsets": [R.count.offset, R.mean.offset, R.m2.offset], "itemsize": C.sizeof(R)})


def result_dtype() -> np.dtype:
    """cdet_mcmcmc_chain_result as a numpy structured type."""
    R, st, e = L.ChainResult, stats_dtype(), L.MAX_ENVELOPE + 1
    names = ["seed", "warmup_proposed_steps", "warmup_accepted_steps", "production_proposed_steps",
             "production_accepted_steps", "warmup_chosen_counts", "production_chosen_counts",
             "warmup_retained_fraction_stats", "production_retained_fraction_stats", "order_signal_stats"]
    formats = [np.uint64] * 5 + [(np.uint64, (e,)), (np.uint64, (e,)), st, st, (st, (e,))]
    return np.dtype({"names": names, "formats": formats, "offsets": [getattr(R, n).offset for n in names],
                     "itemsize": C.sizeof(R)})


def read_checkpoint(path: str, lib=None) -> L.Checkpoint:
    """One CDET_MCMCMC_CHAIN_CHECKPOINT_V1 file (host only)."""
    lib = lib or L.load()
    ck = L.Checkpoint()
    L.check(lib.cdet_read_mcmcmc_checkpoint(os.fsencode(path), C.byref(ck)))
    return ck


def write_checkpoint(path: str, ck: L.Checkpoint, lib=None) -> None:
    lib = lib or L.load()
    L.check(lib.cdet_write_mcmcmc_checkpoint(os.fsencode(path), C.byref(ck)))


def learn_histogram(integrand: CdetIntegrand, order_min: int, order_max: int, envelope: int, learning_steps: int,
                    tau_bins: int = 16, uniform_mix: float = 0.05, pseudo_count: float = 0.0,
                    base_seed: int = 0):
    """learn_factorized_histogram_seed on the integrand's tables: (tau, space,
    replica, total pair weight), the probabilities as flat rows."""
    sites = integrand.params.n1 * integrand.params.n2
    tau, space, rep = np.zeros(tau_bins * tau_bins), np.zeros(sites * sites), np.zeros(4)
    total = C.c_double()
    cfg = L.McmcmcConfig(order_min, order_max, envelope, 1, 0.0)
    hcfg = L.HistogramConfig(learning_steps, tau_bins, uniform_mix, pseudo_count)
    dp = C.POINTER(C.c_double)
    L.check(integrand._lib.cdet_mcmcmc_learn_histogram(integrand._ctx, C.byref(cfg), C.byref(hcfg),
                                                        int(base_seed), tau.ctypes.data_as(dp),
                                                        space.ctypes.data_as(dp), rep.ctypes.data_as(dp),
                                                        C.byref(total)))
    return tau, space, rep, total.value


def jackknife_ratios(results: np.ndarray, order_min: int, order_max: int, normalization_order: int) -> dict:
    """Chain-level jackknife of the per-order ratios the reference reports
    (run_mcmcmc_chains_parallel, mcmcmc_sampler.h:1118-1146): each chain's
    production mean of the order signal is one sample, the ratio of order n
    is mean over chains at n / mean over chains at the normalisation order.
    Leaving out one chain at a time gives the jackknife estimates R_(c);
    the error is sqrt((C - 1)/C sum_c (R_(c) - mean R_(.))^2). Returns
    {"ratio": [envelope + 1], "error": [envelope + 1]} (NaN outside the
    sampled orders), from `results` = McmcmcChains.results()."""
    means = np.asarray(results["order_signal_stats"]["mean"], dtype=np.float64)  # [chains][max envelope + 1]
    counts = np.asarray(results["order_signal_stats"]["count"])
    chains = means.shape[0]
    e1 = means.shape[1]
    ratio = np.full(e1, np.nan)
    error = np.full(e1, np.nan)
    ref = normalization_order
    for n in range(order_min, order_max + 1):
        use = (counts[:, n] > 0) & (counts[:, ref] > 0)
        m, r = means[use, n], means[use, ref]
        k = m.size
        if k < 2 or r.sum() == 0.0:
            continue
        ratio[n] = m.sum() / r.sum()
        loo = (m.sum() - m) / (r.sum() - r)
        error[n] = float(np.sqrt((k - 1) / k * np.sum((loo - loo.mean()) ** 2)))
    return {"ratio": ratio, "error": error, "chains": chains}


def mt64_outputs(state: np.ndarray, count: int) -> np.ndarray:
    """The next `count` outputs of an mt19937_64 from its [313] state (312
    words and position), without changing it."""
    mt = [int(x) for x in state[:312]]
    index = int(state[312])
    out = []
    m64 = (1 << 64) - 1
    for _ in range(count):
        if index >= 312:
            for i in range(312):
                x = (mt[i] & 0xFFFFFFFF80000000) | (mt[(i + 1) % 312] & 0x7FFFFFFF)
                mt[i] = mt[(i + 156) % 312] ^ (x >> 1) ^ (0xB5026F5AA96619E9 if x & 1 else 0)
            index = 0
        y = mt[index]
        index += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000 & m64
        y ^= (y << 37) & 0xFFF7EEE000000000 & m64
        y ^= y >> 43
        out.append(y & m64)
    return np.array(out, dtype=np.uint64)
