"""Host-side logic: runtime scalars, masks, the reference's vertex stream."""
import numpy as np

from cdet_gb300.params import CdetParams, half_lattice_mask, named_mask
from cdet_gb300.synthetic import MT19937_64, derive_seed, splitmix64, truncated_geometric_orders
from helpers import GOLDEN


def test_vertex_stream_matches_reference():
    """sample_uniform_unit_vertex (mcmcmc_sampler.h:187-190) from
    std::mt19937_64, as recorded from the reference build."""
    data = np.load(f"{GOLDEN}/vertex_samples.npz")
    for seed in (1, 12345, 2026101401):
        got = MT19937_64(seed).uniform01(200 * 4).reshape(200, 4)
        assert np.array_equal(got, data[f"mt{seed}"])


def test_seed_derivation():
    assert splitmix64(0) == 0xE220A8397B1DCDAF  # first SplitMix64 output of state 0
    a = derive_seed(2026101401, 3, 0)
    assert a == derive_seed(2026101401, 3, 0) and a != derive_seed(2026101401, 3, 1)


def test_runtime_scalars():
    p = CdetParams(n1=8, n2=8, beta="8", u="4", alpha_up="0.55", alpha_down="0.4")
    s = p.runtime_scalars()
    assert s["scale"] == float(np.sqrt(4 * 64 * 8))
    assert s["diag_up_shift"] == 0.4 / 4 and s["diag_down_shift"] == 0.55 / 4
    assert s["fpm_shift"] == -1.0 and s["z_eps0"] == 2e-16 and s["z_safety"] == 1e4
    assert not p.alpha_equal


def test_masks():
    assert len(named_mask("origin_square", 8, 8, 2)) == 16  # the 4x4 corner block
    assert named_mask("first_column", 3, 3) == (0, 3, 6)
    assert named_mask("first_row", 3, 3) == (0, 1, 2)
    assert len(half_lattice_mask(6, 6)) == 18 and len(half_lattice_mask(12, 12)) == 72


def test_truncated_geometric_orders():
    o = truncated_geometric_orders(5, 200000, 0.3, 10)
    assert o.min() == 1 and o.max() == 10
    freq = np.bincount(o, minlength=11)[1:] / o.size
    w = 0.3 * 0.7 ** np.arange(10)
    assert np.allclose(freq, w / w.sum(), atol=0.005)
