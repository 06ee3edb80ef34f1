"""The precision contract, per order, on the 8x8 / degree-128 benchmark lattice.

Orders 1..10 of seeded configurations (t=1, U=4, beta=8, mu=0, 4x4 corner
subsystem, Chebyshev degree 128), both assemblies, with the round-off filter
on (the reference default) and off, against the oracle's long double truth
(pinned to the reference's long_double / double_double mode).

Relative error is ill-posed at high order: the connected sums cancel by
factors up to 1e19 at order 10, so any FP64 evaluation (the reference's
included) is off by about a percent there. The contract is stated
normwise against the magnitude of the terms (oracle/precision.py,
``condition_scaled``): <= 1e-10 at every order, for both forms, filter on
and off. Beside it, at each order the split form's median error against
the truth (filter off, where the value is well defined; relative, scaled by
|twisted| + 2 |ordinary| for order 1's cancelling combine) is at most 3x the
FP64 form's, and split and FP64 agree to 1e-12 condition-scaled.
"""
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.params import CdetParams, half_lattice_mask, named_mask  # noqa: E402
from cdet_gb300.synthetic import uniform_configurations  # noqa: E402
from cdet_gb300.tables import build_tables  # noqa: E402
from bindings import Oracle  # noqa: E402
from precision import error_forms  # noqa: E402

CONTRACT = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


def _evaluate(ctx, path, v, o):
    ctx.set_assembly(path)
    dv, do = torch.from_numpy(v).cuda(), torch.from_numpy(o).cuda()
    vals = torch.empty(v.shape[0], dtype=torch.float64, device="cuda")
    st = torch.empty(v.shape[0], dtype=torch.int32, device="cuda")
    ctx.integrand_device(dv, do, vals, st)
    torch.cuda.synchronize()
    return vals.cpu().numpy(), st.cpu().numpy()


def _host(tables):
    host = {k: {kk: vv.cpu().numpy() for kk, vv in t.items()} for k, t in tables.items()}
    for a, b in (("twisted_down", "twisted_up"), ("ordinary_down", "ordinary_up")):
        if tables[a] is tables[b]:
            host[a] = host[b]
    return host


def _check_orders(params, orders, per_order, seed):
    tables = build_tables(params, device="cuda")
    host = _host(tables)
    orc = Oracle(params.runtime_scalars(), host)
    ctxs = {"on": CdetIntegrand(params, tables),
            "off": CdetIntegrand(dataclasses.replace(params, z_safety="0"), tables)}
    report = {}
    for n in orders:
        v = uniform_configurations(seed + n, per_order, n)
        o = np.full(per_order, n, np.int32)
        truth, parts, st = orc.integrand_ld_parts_batch(v, o, threads=8)
        got = {(f, p): _evaluate(ctxs[f], p, v, o) for f in ctxs for p in ("split", "fp64")}
        ok = st == 0
        for _, s in got.values():
            ok &= s == 0
        assert ok.sum() >= per_order // 2, n
        for f in ctxs:
            for p in ("split", "fp64"):
                e = error_forms(got[(f, p)][0], truth, parts, ok)
                report[(n, f, p)] = e
                assert e["condition_scaled"]["max"] <= CONTRACT, (n, f, p, e)
        # the split form is as accurate as the FP64 form (filter off: the
        # value the truth computes; combine-scaled, which is the relative
        # error except at order 1, where twisted - 2 ordinary cancels)
        es, ef = report[(n, "off", "split")], report[(n, "off", "fp64")]
        assert es["combine_scaled"]["median"] <= 3.0 * ef["combine_scaled"]["median"] + 1e-15, (n, es, ef)
        agree = error_forms(got[("on", "split")][0], got[("on", "fp64")][0], parts, ok)
        assert agree["condition_scaled"]["max"] <= 1e-12, (n, agree)
    for ctx in ctxs.values():
        ctx.close()
    return report


def test_precision_contract_8x8_orders_1_to_10():
    params = CdetParams(n1=8, n2=8, beta="8", mu="0", u="4", alpha_up="0", alpha_down="0",
                        mask_sites=named_mask("origin_square", 8, 8, 2), cheb_nu=128, cheb_nv=128)
    _check_orders(params, range(1, 11), 64, 41000)


def test_precision_contract_order_14_degree_192():
    """Order 14 at Chebyshev degree 192 (the split form's sub-block assembly)
    on a 3x3 half-lattice, U=6, beta=10, mu=-0.5."""
    params = CdetParams(n1=3, n2=3, beta="10", mu="-0.5", u="6", alpha_up="0", alpha_down="0",
                        mask_sites=half_lattice_mask(3, 3), cheb_nu=192, cheb_nv=192)
    _check_orders(params, [14], 16, 42000)


def test_double_double_meets_relative_contract_8x8():
    """The literal contract, relative error <= 1e-10 at every order, on the
    benchmark lattice: the double-double recursion (the reference's
    INTEGRAND_REAL=double_double on the FP64 assembly, and the same recursion
    on the split assembly's Green matrices), with the reference's default
    round-off filter, against the long double truth at orders 2..10; at
    order 1, whose twisted - 2 ordinary cancels to the round-off of its
    inputs, scaled by |twisted| + 2 |ordinary|."""
    params = CdetParams(n1=8, n2=8, beta="8", mu="0", u="4", alpha_up="0", alpha_down="0",
                        mask_sites=named_mask("origin_square", 8, 8, 2), cheb_nu=128, cheb_nv=128)
    tables = build_tables(params, device="cuda")
    orc = Oracle(params.runtime_scalars(), _host(tables))
    ctx = CdetIntegrand(params, tables)
    ctx.set_integrand_real("double_double")
    ctx.set_integrand_form("staged")  # the lane layout a large batch runs (lighter steps on the split assembly)
    for n in range(1, 11):
        v = uniform_configurations(43000 + n, 64, n)
        o = np.full(64, n, np.int32)
        truth, parts, st = orc.integrand_ld_parts_batch(v, o, threads=8)
        for path in ("fp64", "split"):
            got, gst = _evaluate(ctx, path, v, o)
            ok = (st == 0) & (gst == 0)
            assert ok.sum() >= 32, (n, path)
            e = error_forms(got, truth, parts, ok)
            form = "combine_scaled" if n == 1 else "relative"
            assert e[form]["max"] <= CONTRACT, (n, path, e[form])
    ctx.close()
