"""MCMCMC chains resident on the GPU (uniform or factorized histogram seed).

The batch counterpart of run_single_mcmcmc_chain (mcmcmc_sampler.h:994-1088):
every step evaluates the all-subset integrand of each chain's envelope on the
GPU and runs run_mcmcmc_step (:524-577) in one thread per chain, with each
chain's std::mt19937_64 stream reproduced on the device. With the FP64
assembly the chains are the reference's chains, step for step.
`learn_histogram` is learn_factorized_histogram_seed (:607-664) and
`McmcmcChains.set_histogram` switches the chains to that seed kernel
(MCMCMC_SEED_MODE=histogram).
"""
from __future__ import annotations

import ctypes as C
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
