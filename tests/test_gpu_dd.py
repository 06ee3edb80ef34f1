"""The double-double integrand mode (INTEGRAND_REAL=double_double with
VECTOR_REAL=double) on the GPU, through the C ABI, against the reference's
own values of that mode (dd_mode.npz, written by make_dd_golden.py from the
reference build): bit for bit at orders 1..10 on the 2x2 tables (distinct up
and down spins, U = 1.7 with a DoubleDouble low part) and the 3x3 tables, with
the round-off filter on and off and with the LU fallback forced. The
parameters' DoubleDouble values are taken as the quad-precision MP_Real of
that build gives them (they agree with the 100-digit ones for these literals).
"""
import dataclasses
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300 import lib as L  # noqa: E402
from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.params import dd_of_literal  # noqa: E402
from cdet_gb300.synthetic import uniform_configurations  # noqa: E402
from helpers import GOLDEN, bits_equal, load_case  # noqa: E402

DD = np.load(os.path.join(GOLDEN, "dd_mode.npz"))
VARIANTS = {"default": {}, "nofilter": {"z_safety": "0"}, "fallback": {"tol_fpm": "1"}}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


@pytest.mark.parametrize("case", ["physical_2x2", "column_3x3"])
@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_dd_mode_equals_reference(case, variant):
    params, tables, _ = load_case(case)
    params = dataclasses.replace(params, **VARIANTS[variant])
    gpu = CdetIntegrand(params, tables)
    gpu.set_integrand_real("double_double", significand_bits=113)
    v, o = DD[f"{case}.vertices"], DD[f"{case}.orders"]
    want = DD[f"{case}.{variant}.values"]
    for form in ("auto", "staged", "queue"):  # every layout gives the reference's values on the FP64 assembly
        gpu.set_integrand_form(form)
        got, st = gpu.integrand_batch(v, o)
        assert (st & ~L.CONFIG_FPM_FALLBACK).max() == 0
        bad = np.flatnonzero(got.view(np.uint64) != want.view(np.uint64))
        assert bad.size == 0, (form, bad[:8], o[bad[:8]], got[bad[:8]], want[bad[:8]])
    gpu.set_integrand_form("auto")
    if variant == "fallback":
        assert np.all(st[o >= 2] & L.CONFIG_FPM_FALLBACK)
    # back to the FP64 drop-in: the FP64 values again
    gpu.set_integrand_real("double")
    fp64, _ = gpu.integrand_batch(v[:, :8][o <= 8], o[o <= 8])
    gpu2 = CdetIntegrand(params, tables)
    want64, _ = gpu2.integrand_batch(v[:, :8][o <= 8], o[o <= 8])
    assert bits_equal(fp64, want64)


@pytest.mark.parametrize("case", ["physical_2x2", "column_3x3"])
@pytest.mark.parametrize("variant", ["default", "fallback"])
def test_dd_lane_form_equals_reference(case, variant):
    """A batch large enough for the lane form (minors by warps into
    lane-interleaved arrays, the recursion one lane per configuration over
    order-sorted slots): the golden configurations repeated to 6,300, every
    value the reference's bit for bit."""
    params, tables, _ = load_case(case)
    params = dataclasses.replace(params, **VARIANTS[variant])
    gpu = CdetIntegrand(params, tables)
    gpu.set_integrand_real("double_double", significand_bits=113)
    v, o = DD[f"{case}.vertices"], DD[f"{case}.orders"]
    reps = 50
    got, st = gpu.integrand_batch(np.tile(v, (reps, 1, 1)), np.tile(o, reps))
    want = np.tile(DD[f"{case}.{variant}.values"], reps)
    assert (st & ~L.CONFIG_FPM_FALLBACK).max() == 0
    assert bits_equal(got, want)


@pytest.mark.parametrize("case", ["physical_2x2", "column_3x3"])
def test_dd_on_split_assembly_and_what_it_rejects(case):
    """The double-double recursion on the tensor-core Green matrices: not
    the reference's mode, but its values stay within 1e-12 relative of it at
    every order 1..10 (the Green entries agree to ~1e-15; the FP64 recursion
    is off by up to 1e-7 on these cases); all-subsets calls and orders above
    10 are refused."""
    params, tables, _ = load_case(case)
    gpu = CdetIntegrand(params, tables)
    gpu.set_integrand_real("double_double", significand_bits=113)
    gpu.set_assembly("split")
    v, o = DD[f"{case}.vertices"], DD[f"{case}.orders"]
    want = DD[f"{case}.default.values"]
    for form in ("queue", "staged"):  # the warp layout (exact steps) and the lane layout (lighter ones)
        gpu.set_integrand_form(form)
        got, st = gpu.integrand_batch(v, o)
        assert st.max() == 0
        scale = np.maximum(np.abs(want), 1e-300)
        rel = np.abs(got - want) / scale
        big = o >= 2  # order 1 cancels to round-off residue (compare absolutely)
        assert rel[big].max() <= 1e-12, (form, rel[big].max(), o[big][np.argmax(rel[big])])
        assert np.abs(got - want)[o == 1].max() <= 1e-13
    with pytest.raises(RuntimeError, match="order <= 10"):
        gpu.all_subsets_batch(uniform_configurations(3, 4, 5))
    with pytest.raises(RuntimeError, match="order <= 10"):
        gpu.integrand_batch(uniform_configurations(4, 2, 11), np.full(2, 11, dtype=np.int32))


def test_dd_literals_quad_and_exact_agree_here():
    for lit in ("1.7", "0.55", "0.4", "2.5", "1e-7", "1e-31", "1e4", "-1", "4", "2", "0"):
        assert dd_of_literal(lit) == dd_of_literal(lit, 113), lit
