"""Chains driven by the split (tensor-core) assembly against chains driven by
the FP64 assembly (which are the reference's chains step for step).

The MCMCMC configuration of the benchmark: 6x6 lattice, U=2, beta=6, mu=0,
3x6 half-lattice subsystem, Chebyshev degree 96, orders 1..8 in envelope 9,
128 chains on the factorized histogram seed learned on the GPU, lambda
adaptation during warmup. The split form's integrand values differ from the
FP64 form's at the round-off floor of each order, so its chains diverge from
the FP64 chains after a few steps; they must sample the same distribution:
per order, the ratios to order 1 (the reference's cross-chain summary,
mcmcmc_sampler.h:1118-1146) agree within three chain-level jackknife
standard errors (run lengths here are shortened from the production 10^5
steps).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.mcmcmc import STREAM_TAG, McmcmcChains, jackknife_ratios, learn_histogram  # noqa: E402
from cdet_gb300.params import CdetParams, half_lattice_mask  # noqa: E402
from cdet_gb300.synthetic import derive_seed  # noqa: E402
from cdet_gb300.tables import build_tables  # noqa: E402


def test_split_chains_agree_with_fp64_chains():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    params = CdetParams(n1=6, n2=6, beta="6", mu="0", u="2", alpha_up="0", alpha_down="0",
                        mask_sites=half_lattice_mask(6, 6), cheb_nu=96, cheb_nv=96)
    env, omin, omax = 9, 1, 8
    lambdas = [0.0] + [1.0] * 8 + [0.0]
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    gpu.set_assembly("fp64")
    tau, space, rep, _ = learn_histogram(gpu, omin, omax, env, 64, 16, 0.05, 0.0, 20261203)
    est = {}
    for path in ("fp64", "split"):
        gpu.set_assembly(path)
        seeds = [derive_seed(20261207, STREAM_TAG, i) for i in range(128)]
        chains = McmcmcChains(gpu, omin, omax, env, seeds, lambdas, adapt_interval=50)
        chains.set_histogram(16, tau, space, rep)
        chains.run(400, warmup=True)
        chains.end_warmup()
        chains.run(3000)
        est[path] = jackknife_ratios(chains.results(), omin, omax, 1)
        chains.close()
    for n in range(2, omax + 1):
        a, b = est["split"], est["fp64"]
        sigma = np.hypot(a["error"][n], b["error"][n])
        assert np.isfinite(sigma) and sigma > 0, n
        assert abs(a["ratio"][n] - b["ratio"][n]) <= 3.0 * sigma, (n, a["ratio"][n], b["ratio"][n], sigma)
    gpu.close()
