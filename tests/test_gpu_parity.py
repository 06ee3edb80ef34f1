"""Parity of the GB300 kernels (through the C ABI) with the reference.

* Golden vectors: on the reference-built tables the GPU values must equal the
  reference's outputs bit for bit (single-order, all-subset, filter off,
  forced LU fallback), and the reference entry points must raise the
  reference's errors.
* Oracle at larger sizes: tables from the in-tree precompute, GPU against the
  C oracle, bit for bit, at the 3x3/d=64 configuration (4096 configurations
  per order 1..6), 8x8/d=128 at order 10, and high orders on a small lattice.
* Size-independent properties at full batch: permutation invariance,
  determinism, all-subset vs single-order consistency.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from bindings import Oracle  # noqa: E402
from cdet_gb300 import lib as L  # noqa: E402
from cdet_gb300.integrand import CdetIntegrand, UnitVertex, subset_vertices  # noqa: E402
from cdet_gb300.params import CdetParams, named_mask  # noqa: E402
from cdet_gb300.synthetic import truncated_geometric_orders, uniform_configurations  # noqa: E402
from cdet_gb300.tables import build_tables  # noqa: E402
from helpers import bits_equal, load_case  # noqa: E402

CASES = ("physical_2x2", "column_3x3")
THREADS = 16


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


@pytest.mark.parametrize("name", CASES)
def test_golden_single_order(name):
    params, tables, data = load_case(name)
    gpu = CdetIntegrand(params, tables)
    out, st = gpu.integrand_batch(data["single.vertices"], data["single.orders"])
    assert (st & ~L.CONFIG_FPM_FALLBACK).max() == 0
    assert bits_equal(out, data["single.values"])
    # the reference entry point, one configuration at a time
    for v, n, want in list(zip(data["single.vertices"], data["single.orders"], data["single.values"]))[::7]:
        got = gpu.evaluate_cdet_density_integrand_double([UnitVertex(*row) for row in v[:n]])
        assert bits_equal([got], [want])


@pytest.mark.parametrize("name", CASES)
def test_golden_all_subsets(name):
    params, tables, data = load_case(name)
    gpu = CdetIntegrand(params, tables)
    for env in range(2, 8):
        out, st = gpu.all_subsets_batch(data[f"all{env}.vertices"])
        assert st.max() == 0
        assert bits_equal(out, data[f"all{env}.values"]), env
    values = []
    gpu.evaluate_cdet_density_all_subset_integrands_double_into(data["audit6.vertices"][0], values)
    assert len(values) == 64 and bits_equal(values, data["audit6.values"][0])


@pytest.mark.parametrize("name", CASES)
def test_golden_filter_off_and_fallback(name):
    import dataclasses
    params, tables, data = load_case(name)
    v, n = data["single.vertices"], data["single.orders"]
    gpu = CdetIntegrand(dataclasses.replace(params, z_safety="0"), tables)
    out, _ = gpu.integrand_batch(v, n)
    assert bits_equal(out, data["nofilter.values"])
    gpu = CdetIntegrand(dataclasses.replace(params, tol_fpm="1"), tables)
    out, st = gpu.integrand_batch(v, n)
    assert bits_equal(out, data["fallback.values"])
    assert np.all((st[n >= 2] & L.CONFIG_FPM_FALLBACK) != 0)
    calls, fallbacks = gpu.counters()
    assert calls == len(n) and fallbacks == int((n >= 2).sum())


def test_reference_errors():
    params, tables, _ = load_case("column_3x3")
    gpu = CdetIntegrand(params, tables)
    with pytest.raises(RuntimeError, match="order >= 1"):
        gpu.evaluate_cdet_density_integrand_double([])
    with pytest.raises(RuntimeError, match="envelope order >= 2"):
        gpu.evaluate_cdet_density_all_subset_integrands_double([UnitVertex(0.1, 0.2, 0.3, 0.4)])
    with pytest.raises(RuntimeError):
        gpu.evaluate_cdet_density_integrand_double([UnitVertex(float("nan"), 0.2, 0.3, 0.4)] * 2)
    # ragged batch: orders outside 1..max_order are flagged, the rest evaluated
    v = uniform_configurations(5, 4, 3)
    out, st = gpu.integrand_batch(v, [3, 0, 2, 4])
    assert st[1] & L.CONFIG_BAD_INPUT and st[3] & L.CONFIG_BAD_INPUT
    assert st[0] == 0 and st[2] == 0


def _column_3x3(d):
    return CdetParams(n1=3, n2=3, beta="4", mu="0", u="2",
                      mask_sites=named_mask("first_column", 3, 3), cheb_nu=d, cheb_nv=d)


def test_oracle_3x3_d64_full_batch():
    """The 3x3 one-column configuration at Chebyshev degree 64: 4096 seeded
    configurations per order n = 1..6, GPU against the oracle bit for bit."""
    params = _column_3x3(64)
    tables = build_tables(params, device="cuda")
    gpu = CdetIntegrand(params, tables)
    orc = Oracle(params.runtime_scalars(), tables)
    for n in range(1, 7):
        v = uniform_configurations(1000 + n, 4096, n)
        orders = np.full(4096, n, dtype=np.int32)
        got, st = gpu.integrand_batch(v, orders)
        want, wst = orc.integrand_batch(v, orders, threads=THREADS)
        assert np.array_equal(st, wst)
        assert bits_equal(got, want), n


def test_oracle_mixed_orders_and_high_orders():
    params = _column_3x3(8)
    tables = build_tables(params, device="cuda")
    gpu = CdetIntegrand(params, tables)
    orc = Oracle(params.runtime_scalars(), tables)
    # uneven orders 1..10 in one batch (truncated geometric, p = 0.3)
    orders = truncated_geometric_orders(11, 2048, 0.3, 10)
    v = uniform_configurations(12, 2048, 10)
    got, st = gpu.integrand_batch(v, orders)
    want, wst = orc.integrand_batch(v, orders, threads=THREADS)
    assert np.array_equal(st, wst) and bits_equal(got, want)
    # high orders 11..14 (one block per configuration): fixed orders, and a
    # batch of orders 1..13 whose slots are sorted by order
    for n, count in ((11, 64), (12, 64), (13, 32), (14, 16)):
        v = uniform_configurations(100 + n, count, n)
        orders = np.full(count, n, dtype=np.int32)
        got, st = gpu.integrand_batch(v, orders)
        want, wst = orc.integrand_batch(v, orders, threads=THREADS)
        assert np.array_equal(st, wst) and bits_equal(got, want), n
    v = uniform_configurations(113, 96, 13)
    orders = np.random.default_rng(114).integers(1, 14, size=96).astype(np.int32)
    orders[5] = 0  # flagged, its value unspecified
    got, st = gpu.integrand_batch(v, orders)
    want, wst = orc.integrand_batch(v, orders, threads=THREADS)
    ok = orders > 0
    assert np.array_equal(st, wst) and st[5] & L.CONFIG_BAD_INPUT
    assert bits_equal(got[ok], want[ok])
    # orders 1..14 in one batch: the order-14 kernel (512 threads, the top
    # levels' serial sums on separate warps) also runs the lower orders
    v = uniform_configurations(115, 32, 14)
    orders = np.random.default_rng(116).integers(1, 15, size=32).astype(np.int32)
    orders[:4] = (14, 13, 12, 11)
    got, st = gpu.integrand_batch(v, orders)
    want, wst = orc.integrand_batch(v, orders, threads=THREADS)
    assert np.array_equal(st, wst) and bits_equal(got, want)
    # all-subsets at envelope 9
    v = uniform_configurations(13, 64, 9)
    got, _ = gpu.all_subsets_batch(v)
    want, _ = orc.all_subsets_batch(v, threads=THREADS)
    assert bits_equal(got, want)


def test_oracle_high_orders_two_spins_fallback_and_envelope():
    """Orders 11..14, whose minors run the chunked Schur recursion (top levels
    in the global workspace, subtrees in shared memory), on tables with
    distinct up and down spins, with the LU fallback forced (TOL_FPM = 1) and
    as an all-subsets envelope of 12: bit for bit the oracle's."""
    import dataclasses
    params, tables, _ = load_case("physical_2x2")
    for over in ({}, {"tol_fpm": "1"}):
        p2 = dataclasses.replace(params, **over)
        gpu = CdetIntegrand(p2, tables)
        orc = Oracle(p2.runtime_scalars(), tables)
        for n, count in ((11, 24), (12, 16), (13, 8), (14, 6)):
            v = uniform_configurations(300 + n, count, n)
            orders = np.full(count, n, dtype=np.int32)
            got, st = gpu.integrand_batch(v, orders)
            want, wst = orc.integrand_batch(v, orders, threads=THREADS)
            assert np.array_equal(st, wst) and bits_equal(got, want), (over, n)
            if over:
                assert np.all(st & L.CONFIG_FPM_FALLBACK)
    gpu = CdetIntegrand(params, tables)
    orc = Oracle(params.runtime_scalars(), tables)
    v = uniform_configurations(399, 4, 12)
    got, _ = gpu.all_subsets_batch(v)
    want, _ = orc.all_subsets_batch(v, threads=THREADS)
    assert bits_equal(got, want)


def test_oracle_8x8_d128_order10():
    """The 8x8 / 4x4-corner / degree-128 configuration at order 10 on a
    512-configuration sample, GPU against the oracle bit for bit."""
    params = CdetParams(n1=8, n2=8, beta="8", mu="0", u="4",
                        mask_sites=named_mask("origin_square", 8, 8, 2), cheb_nu=128, cheb_nv=128)
    tables = build_tables(params, device="cuda")
    gpu = CdetIntegrand(params, tables)
    orc = Oracle(params.runtime_scalars(), tables)
    v = uniform_configurations(810, 512, 10)
    orders = np.full(512, 10, dtype=np.int32)
    got, st = gpu.integrand_batch(v, orders)
    want, wst = orc.integrand_batch(v, orders, threads=THREADS)
    assert np.array_equal(st, wst) and bits_equal(got, want)


def test_properties_full_batch():
    """Size-independent properties on a 65,536-configuration batch: the
    result of a configuration does not depend on its position in the batch,
    and repeated runs are bit-identical."""
    params = _column_3x3(16)
    tables = build_tables(params, device="cuda")
    gpu = CdetIntegrand(params, tables)
    v = uniform_configurations(99, 65536, 6)
    orders = np.full(65536, 6, dtype=np.int32)
    first, st = gpu.integrand_batch(v, orders)
    again, _ = gpu.integrand_batch(v, orders)
    assert bits_equal(first, again)
    perm = np.random.default_rng(3).permutation(65536)
    permuted, _ = gpu.integrand_batch(v[perm], orders[perm])
    assert bits_equal(permuted, first[perm])
    assert np.all(np.isfinite(first))


def test_all_subsets_against_single_order():
    """tests/test_integrand_all_subsets.cpp:36-50 on the GPU path: every subset
    of the all-subset integrand equals the single-order integrand of that
    subset within 2e-9 (absolute + relative, the audit's tolerance)."""
    params, tables, data = load_case("physical_2x2")
    gpu = CdetIntegrand(params, tables)
    env = data["audit6.vertices"]
    allv, _ = gpu.all_subsets_batch(env)
    subsets = []
    for v in env:
        for mask in range(1, 64):
            subsets.append(np.pad(subset_vertices(v, mask), ((0, 6 - bin(mask).count("1")), (0, 0))))
    orders = np.array([bin(m).count("1") for _ in env for m in range(1, 64)], dtype=np.int32)
    single, _ = gpu.integrand_batch(np.array(subsets), orders)
    combined = allv[:, 1:].reshape(-1)
    scale = np.maximum(1.0, np.maximum(np.abs(single), np.abs(combined)))
    assert np.all(np.abs(single - combined) <= 2e-9 + 2e-9 * scale)


@pytest.mark.parametrize("assembly", ["fp64", "split"])
def test_all_subsets_forms_identical(assembly):
    """The lane and warp forms of the all-subsets CDet recursion give the same
    values bit for bit (orders 2..11, batches not a multiple of the warp or
    block), and the automatic choice is one of them."""
    params = _column_3x3(64)
    tables = build_tables(params, device="cuda")
    gpu = CdetIntegrand(params, tables)
    gpu.set_assembly(assembly)
    for n, count in ((2, 37), (5, 70), (9, 129), (11, 45)):
        v = uniform_configurations(500 + n, count, n)
        out = {}
        for form in ("lane", "warp", "auto"):
            gpu.set_all_subsets_form(form)
            out[form] = gpu.all_subsets_batch(v)
        assert bits_equal(out["lane"][0], out["warp"][0]), n
        assert np.array_equal(out["lane"][1], out["warp"][1]), n
        assert bits_equal(out["auto"][0], out["warp"][0]), n
        assert gpu.all_subsets_form_tuned(n, count) in ("lane", "warp")  # measured by the "auto" call
    if assembly == "fp64":
        orc = Oracle(params.runtime_scalars(), tables)
        v = uniform_configurations(611, 40, 11)
        gpu.set_all_subsets_form("warp")
        got, _ = gpu.all_subsets_batch(v)
        want, _ = orc.all_subsets_batch(v, threads=THREADS)
        assert bits_equal(got, want)
