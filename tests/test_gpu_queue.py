"""The persistent queue form and the integrand autotuner (through the C ABI).

A single-top batch of order <= 10 runs after its Green matrices either
staged (minors kernel, a[] in HBM, CDet kernel) or as one persistent kernel
that takes configurations from order-sorted slots through an atomic queue
head. Every form and launch shape performs the same operations per
configuration, so the values and status bits must be the staged form's bit
for bit: FP64 and split assemblies, mixed and single orders, one-spin and
two-spin tables, the forced LU fallback, and the autotuner's choice.
"""
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from bindings import Oracle  # noqa: E402
from cdet_gb300 import lib as L  # noqa: E402
from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.params import CdetParams, half_lattice_mask  # noqa: E402
from cdet_gb300.synthetic import truncated_geometric_orders, uniform_configurations  # noqa: E402
from cdet_gb300.tables import build_tables  # noqa: E402
from helpers import bits_equal, load_case  # noqa: E402

SHAPES = [dict(), dict(pair=True), dict(grab=4), dict(warps_per_sm=4), dict(warps_per_sm=2, pair=True, grab=3)]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


def _evaluate(gpu, v, o, form, **shape):
    gpu.set_integrand_form(form, **shape)
    out, st = gpu.integrand_batch(v, o)
    return out, st


@pytest.mark.parametrize("name", ["physical_2x2", "column_3x3"])
@pytest.mark.parametrize("assembly", ["fp64", "split"])
def test_queue_equals_staged_golden_tables(name, assembly):
    """Reference-built tables (the 2x2 case has distinct up and down tables,
    so both spins run), mixed orders 1..10 with uneven counts."""
    params, tables, _ = load_case(name)
    gpu = CdetIntegrand(params, tables)
    gpu.set_assembly(assembly)
    v = uniform_configurations(31 + len(name), 700, 10)
    o = truncated_geometric_orders(32, 700, 0.3, 10)
    want, wst = _evaluate(gpu, v, o, "staged")
    for shape in SHAPES:
        got, st = _evaluate(gpu, v, o, "queue", **shape)
        assert bits_equal(got, want), (assembly, shape)
        assert np.array_equal(st, wst), (assembly, shape)
    if assembly == "fp64":  # and the FP64 queue form is the oracle's (the reference's) value
        oracle = Oracle(params.runtime_scalars(), tables)
        ref, _ = oracle.integrand_batch(v[:200], o[:200])
        got, _ = _evaluate(gpu, v[:200], o[:200], "queue")
        assert bits_equal(got, ref)


@pytest.mark.parametrize("assembly", ["fp64", "split"])
def test_queue_forced_fallback_and_filter_off(assembly):
    params, tables, _ = load_case("physical_2x2")
    v = uniform_configurations(77, 300, 9)
    o = truncated_geometric_orders(78, 300, 0.25, 9)
    for over in (dict(tol_fpm="1"), dict(z_safety="0")):
        gpu = CdetIntegrand(dataclasses.replace(params, **over), tables)
        gpu.set_assembly(assembly)
        want, wst = _evaluate(gpu, v, o, "staged")
        for shape in (dict(), dict(pair=True)):
            got, st = _evaluate(gpu, v, o, "queue", **shape)
            assert bits_equal(got, want) and np.array_equal(st, wst), (over, shape)
        if "tol_fpm" in over:
            assert np.all((wst[o >= 2] & L.CONFIG_FPM_FALLBACK) != 0)


@pytest.mark.parametrize("assembly", ["fp64", "split"])
def test_queue_mixed_batch_half_lattice(assembly):
    """The batching workload's shape at reduced size: 6x6 half lattice,
    degree 32, orders 1..10 truncated geometric (p = 0.3), and a single-order
    batch at order 10; under the autotuner the kept form gives the same values."""
    params = CdetParams(n1=6, n2=6, beta="5", mu="0", u="4", mask_sites=half_lattice_mask(6, 6),
                        cheb_nu=32, cheb_nv=32)
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    gpu.set_assembly(assembly)
    for seed, orders in ((5, None), (6, 10)):
        batch = 4096
        v = uniform_configurations(seed, batch, 10)
        o = (truncated_geometric_orders(seed + 100, batch, 0.3, 10) if orders is None
             else np.full(batch, orders, dtype=np.int32))
        want, wst = _evaluate(gpu, v, o, "staged")
        got, st = _evaluate(gpu, v, o, "queue")
        assert bits_equal(got, want) and np.array_equal(st, wst)
        gpu.set_integrand_form("auto")
        if seed == 5:  # nothing measured yet for (order 10, this assembly, 4096 configurations)
            assert gpu.integrand_form_tuned(10, batch) == {"form": "auto"}
        for _ in range(2):  # the first call measures, the second runs the kept form
            got, st = gpu.integrand_batch(v, o)
            assert bits_equal(got, want) and np.array_equal(st, wst)
        kept = gpu.integrand_form_tuned(10, batch)
        assert kept["form"] in ("staged", "queue"), kept


def test_queue_device_entry_and_launch_count():
    """Device buffers and the launch count: the queue form launches the sort
    (three kernels) and one persistent kernel after the assembly."""
    params, tables, _ = load_case("column_3x3")
    gpu = CdetIntegrand(params, tables)
    batch = 1000
    v = torch.from_numpy(uniform_configurations(9, batch, 8)).cuda()
    o = torch.from_numpy(truncated_geometric_orders(10, batch, 0.3, 8)).cuda()
    outs = []
    for form in ("staged", "queue"):
        gpu.set_integrand_form(form)
        vals = torch.empty(batch, dtype=torch.float64, device="cuda")
        st = torch.empty(batch, dtype=torch.int32, device="cuda")
        gpu.integrand_device(v, o, vals, st)
        torch.cuda.synchronize()
        outs.append((vals.cpu().numpy(), st.cpu().numpy(), gpu.last_launch_count()))
    assert bits_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert outs[1][2] == 2 + 3  # FP64 assembly, queue kernel, three sort kernels


def test_integrand_form_arguments_checked():
    params, tables, _ = load_case("column_3x3")
    gpu = CdetIntegrand(params, tables)
    with pytest.raises(RuntimeError):
        gpu.set_integrand_form("queue", warps_per_sm=33)
    with pytest.raises(RuntimeError):
        gpu.set_integrand_form("queue", grab=0)
