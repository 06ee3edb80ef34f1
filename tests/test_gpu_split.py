"""The split-precision (tcgen05, bf16-slice) Green-matrix assembly.

Its Green matrices must agree with the FP64 Clenshaw assembly to
|G_split - G_fp64| <= 2e-15 * max|G| per matrix set: both are FP64-level
evaluations of the same Chebyshev series. (Against an exact evaluation of the
series the split form's error is 1.4e-16 to 3.8e-16 of the block's largest
coefficient at degrees 16 to 160, below the Clenshaw sum's; see
test_split_arithmetic.py.)

Integrand values are compared only where that is meaningful. Any ulp-level
change of the Green entries re-rolls the round-off of the FP64 minors and
CDet recursion; on the 8x8 lattice a 1e-15 relative perturbation moves the
FP64 integrand by a median 2e-13 at order 2, 3e-10 at order 4 and 3e-7 at
order 6, whatever the perturbation's size. So order 1 (a product of two
diagonal entries) is held to 1e-13, the rest to those noise levels.
"""
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.params import CdetParams, named_mask  # noqa: E402
from cdet_gb300.synthetic import uniform_configurations  # noqa: E402
from cdet_gb300.tables import build_tables  # noqa: E402
from bindings import Oracle  # noqa: E402
from helpers import bits_equal, load_case  # noqa: E402

GREEN_TOL = 2e-15


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


def _green_both(params, tables, v, orders):
    gpu = CdetIntegrand(params, tables)
    dv = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    do = torch.from_numpy(np.ascontiguousarray(orders, dtype=np.int32)).cuda()
    g64, d64, s64 = gpu.assemble(dv, do)
    gpu.set_assembly("split")
    gsp, dsp, ssp = gpu.assemble(dv, do)
    torch.cuda.synchronize()
    assert int(s64.max()) == 0 and int(ssp.max()) == 0
    return gpu, g64.cpu().numpy(), d64.cpu().numpy(), gsp.cpu().numpy(), dsp.cpu().numpy()


def _check_green(g64, gsp, orders, nmax):
    for c, n in enumerate(orders):
        for set_ in range(2):
            for spin in range(2):
                a = g64[c, set_, spin, : n * n]
                b = gsp[c, set_, spin, : n * n]
                scale = max(np.max(np.abs(a)), 1e-300)
                assert np.max(np.abs(a - b)) <= GREEN_TOL * scale, (c, set_, spin)


@pytest.mark.parametrize("d", [16, 64, 128])
def test_split_green_matches_fp64(d):
    params = CdetParams(n1=4, n2=4, beta="6", mu="0", u="2",
                        mask_sites=named_mask("origin_square", 4, 4, 1), cheb_nu=d, cheb_nv=d)
    tables = build_tables(params, device="cuda")
    v = uniform_configurations(300 + d, 256, 8)
    orders = np.full(256, 8, dtype=np.int32)
    _, g64, d64, gsp, dsp = _green_both(params, tables, v, orders)
    _check_green(g64, gsp, orders, 8)
    scale = np.max(np.abs(d64))
    assert np.max(np.abs(d64 - dsp)) <= GREEN_TOL * scale


def test_split_unaliased_padded_and_corners():
    """Four distinct tables (alpha_up != alpha_down: two records per set),
    degree 18 (K and M padding), and vertices at tau = 0 (corner path)."""
    params, tables, data = load_case("physical_2x2")
    v = data["single.vertices"]
    orders = data["single.orders"]
    gpu, g64, d64, gsp, dsp = _green_both(params, tables, v, orders)
    _check_green(g64, gsp, orders, 8)
    # order 1 is a function of the diagonal only: 1e-13; order 2: the FP64
    # noise level of the minors and CDet recursion
    gpu.set_assembly("split")
    split_vals, st = gpu.integrand_batch(v, orders)
    ref = data["single.values"]
    # twisted - 2 * ordinary cancels, so order 1 uses the reference audit's
    # form: |a - b| <= tol * max(1, |a|, |b|) (tests/audit_test_utils.h:17-28)
    close = np.abs(split_vals - ref) / np.maximum(1.0, np.maximum(np.abs(split_vals), np.abs(ref)))
    assert np.max(close[orders == 1]) <= 1e-13
    rel = np.abs(split_vals - ref) / np.maximum(np.abs(ref), 1e-300)
    assert np.median(rel[orders == 2]) <= 1e-11


def test_split_deterministic_and_full_path():
    params = CdetParams(n1=3, n2=3, beta="4", mu="0", u="2",
                        mask_sites=named_mask("first_column", 3, 3), cheb_nu=64, cheb_nv=64)
    tables = build_tables(params, device="cuda")
    gpu = CdetIntegrand(params, tables)
    gpu.set_assembly("split")
    gpu.prepare_split()
    v = uniform_configurations(77, 8192, 4)
    orders = np.full(8192, 4, dtype=np.int32)
    a, st = gpu.integrand_batch(v, orders)
    b, _ = gpu.integrand_batch(v, orders)
    assert st.max() == 0 and bits_equal(a, b)
    gpu.set_assembly("fp64")
    ref, _ = gpu.integrand_batch(v, orders)
    rel = np.abs(a - ref) / np.maximum(np.abs(ref), 1e-300)
    assert np.median(rel) <= 1e-9  # order 4: the FP64 noise level
    # all-subsets through the split assembly
    gpu.set_assembly("split")
    env = uniform_configurations(78, 64, 6)
    sa, _ = gpu.all_subsets_batch(env)
    gpu.set_assembly("fp64")
    fa, _ = gpu.all_subsets_batch(env)
    singles = [1 << i for i in range(6)]
    a_, b_ = sa[:, singles], fa[:, singles]
    close = np.abs(a_ - b_) / np.maximum(1.0, np.maximum(np.abs(a_), np.abs(b_)))
    assert np.max(close) <= 1e-13


@pytest.mark.parametrize("nu,nv", [(160, 160), (192, 192), (256, 256), (136, 200), (200, 100), (96, 160),
                                   (129, 129)])
def test_split_sub_blocks_match_fp64(nu, nv):
    """Degrees above 128: each coefficient block is assembled as sub-blocks
    of at most 128 rows x 128 columns whose exact parts are added before one
    rounding. Non-square degrees cut rows and columns differently. The FP64
    Clenshaw sum's own round-off grows with the degree, so the bound scales
    with it."""
    params = CdetParams(n1=3, n2=3, beta="6", mu="0", u="2",
                        mask_sites=named_mask("first_column", 3, 3), cheb_nu=nu, cheb_nv=nv)
    tables = build_tables(params, device="cuda")
    v = uniform_configurations(900 + nu + nv, 192, 7)
    v[::11, 0, 0] = 0.0  # vertex 0 at tau = 0: its pairs take the corner path
    orders = np.full(192, 7, dtype=np.int32)
    orders[::5] = 1
    gpu, g64, d64, gsp, dsp = _green_both(params, tables, v, orders)
    tol = GREEN_TOL * max(nu, nv) / 128
    worst = 0.0
    for c, n in enumerate(orders):
        for set_ in range(2):
            for spin in range(2):
                a = g64[c, set_, spin, : n * n]
                b = gsp[c, set_, spin, : n * n]
                scale = max(np.max(np.abs(a)), 1e-300)
                worst = max(worst, np.max(np.abs(a - b)) / scale)
    print(f"degree {nu}x{nv}: max |G_split - G_fp64| / max|G| = {worst:.3e}")
    assert worst <= tol
    gpu.set_assembly("split")
    split_vals, st = gpu.integrand_batch(v, orders)
    gpu.set_assembly("fp64")
    ref, st64 = gpu.integrand_batch(v, orders)
    assert st.max() == 0 and st64.max() == 0
    close = np.abs(split_vals - ref) / np.maximum(1.0, np.maximum(np.abs(split_vals), np.abs(ref)))
    assert np.max(close[orders == 1]) <= 1e-13
    if (nu, nv) == (192, 192):
        # the all-subsets (MCMCMC envelope) path through the sub-blocks: the
        # singletons are order-1 values, functions of the diagonal only
        env = uniform_configurations(77 + nu, 32, 6)
        gpu.set_assembly("split")
        sa, sst = gpu.all_subsets_batch(env)
        gpu.set_assembly("fp64")
        fa, fst = gpu.all_subsets_batch(env)
        assert sst.max() == 0 and fst.max() == 0
        singles = [1 << i for i in range(6)]
        a_, b_ = sa[:, singles], fa[:, singles]
        assert np.max(np.abs(a_ - b_) / np.maximum(1.0, np.maximum(np.abs(a_), np.abs(b_)))) <= 1e-13


def test_split_refuses_degree_above_256():
    params = CdetParams(n1=2, n2=2, beta="2", mu="0", u="2",
                        mask_sites=named_mask("first_column", 2, 2), cheb_nu=264, cheb_nv=32)
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    with pytest.raises(Exception, match="<= 256"):
        gpu.set_assembly("split")


def test_split_high_order_block_cdet():
    """Orders 11..14 run the CDet recursion one block per configuration. With
    the split assembly its pair updates are FMAs and a level with few masks
    splits each mask's submask sum over a lane group; on a well-conditioned
    case (beta = 1, U = 1) the values stay within the FP64 noise of the
    reference-order FP64 form, and repeat bit for bit."""
    params = CdetParams(n1=3, n2=3, beta="1", mu="0", u="1",
                        mask_sites=named_mask("first_column", 3, 3), cheb_nu=16, cheb_nv=16)
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    for n in (11, 12, 13, 14):
        v = uniform_configurations(1400 + n, 48, n)
        orders = np.full(48, n, dtype=np.int32)
        orders[::7] = n - 9  # lower orders in the same sorted batch
        gpu.set_assembly("fp64")
        ref, st64 = gpu.integrand_batch(v, orders)
        gpu.set_assembly("split")
        a, st = gpu.integrand_batch(v, orders)
        b, _ = gpu.integrand_batch(v, orders)
        assert st.max() == 0 and st64.max() == 0 and bits_equal(a, b)
        rel = np.abs(a - ref) / np.maximum(np.abs(ref), 1e-300)
        print(f"order {n}: split vs FP64 median rel {np.median(rel):.3e}, max {rel.max():.3e}")
        assert np.median(rel) <= 1e-6, n


def _errors_against_truth(params, tables, v, orders, threads=16):
    """Per-configuration relative errors of the split and FP64 forms against
    the oracle's long double truth."""
    gpu = CdetIntegrand(params, tables)
    fp64, st64 = gpu.integrand_batch(v, orders)
    gpu.set_assembly("split")
    split, st = gpu.integrand_batch(v, orders)
    host = {k: {kk: (vv.cpu().numpy() if hasattr(vv, "cpu") else vv) for kk, vv in t.items()}
            for k, t in tables.items()}
    truth, tst = Oracle(params.runtime_scalars(), host).integrand_ld_batch(v, orders, threads=threads)
    assert st.max() == 0 and st64.max() == 0 and tst.max() == 0
    den = np.maximum(np.abs(truth), 1e-300)
    return np.abs(split - truth) / den, np.abs(fp64 - truth) / den


def test_split_error_against_long_double_truth():
    """Against the long double truth (pinned to the reference's own
    high-precision mode) the split form is as accurate as the FP64 form,
    order by order: the split Green matrices are closer to the exact series
    than the FP64 Clenshaw sums, and the minors and CDet are FP64 in both."""
    params, tables, data = load_case("column_3x3")
    v, orders = data["single.vertices"], data["single.orders"]
    e_split, e_fp64 = _errors_against_truth(params, tables, v, orders)
    for n in range(1, 9):
        sel = orders == n
        ms, mf = np.median(e_split[sel]), np.median(e_fp64[sel])
        print(f"column 3x3 order {n}: median rel error vs truth split {ms:.2e} fp64 {mf:.2e}")
        assert ms <= 3.0 * mf + 1e-15, n
    params = CdetParams(n1=4, n2=4, beta="6", mu="0", u="2",
                        mask_sites=named_mask("origin_square", 4, 4, 1), cheb_nu=64, cheb_nv=64)
    tables = build_tables(params, device="cuda")
    v = uniform_configurations(4242, 256, 8)
    orders = np.full(256, 8, dtype=np.int32)
    e_split, e_fp64 = _errors_against_truth(params, tables, v, orders)
    print(f"4x4 degree 64 order 8: median rel error vs truth split {np.median(e_split):.2e} "
          f"fp64 {np.median(e_fp64):.2e}")
    assert np.median(e_split) <= 3.0 * np.median(e_fp64) + 1e-15


def test_split_sub_blocks_unaliased():
    """Degree above 128 with four distinct tables (alpha_up != alpha_down:
    two records per set, each cut into sub-blocks)."""
    params = CdetParams(n1=2, n2=2, beta="2.5", mu="0.3", u="1.7", alpha_up="0.55", alpha_down="0.4",
                        mask_sites=named_mask("first_row", 2, 2), cheb_nu=144, cheb_nv=144)
    tables = build_tables(params, device="cuda")
    v = uniform_configurations(1444, 128, 6)
    v[::9, 0, 0] = 0.0
    orders = np.full(128, 6, dtype=np.int32)
    orders[::4] = 1
    _, g64, d64, gsp, dsp = _green_both(params, tables, v, orders)
    _check_green(g64, gsp, orders, 6)
    assert np.max(np.abs(d64 - dsp)) <= GREEN_TOL * np.max(np.abs(d64))
