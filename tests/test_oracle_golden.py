"""The C oracle against golden vectors produced by the reference build.

Pins oracle/cdet_oracle.c to the reference: on the reference's own tables and
inputs every value must be bit-identical (the oracle restates the reference's
operations in order, without FMA contraction, like an x86-64 build of it).
The known-answer checks of the reference audit (tests/test_fpm_cdet.cpp) are
repeated on the oracle with the audit's own tolerances.
"""
import dataclasses
import os
from fractions import Fraction
import itertools

import numpy as np
import pytest

from bindings import (Oracle, oracle_mat2pm, oracle_minors_by_lu, oracle_prefactors,
                      oracle_ztransform, oracle_ztransform_all)
from helpers import GOLDEN, bits_equal, load_case

CASES = ("physical_2x2", "column_3x3")


def _oracle(name, **scalar_overrides):
    params, tables, data = load_case(name)
    scalars = params.runtime_scalars()
    scalars.update(scalar_overrides)
    return Oracle(scalars, tables), data


@pytest.mark.parametrize("name", CASES)
def test_single_order_bit_identical(name):
    orc, data = _oracle(name)
    v, n = data["single.vertices"], data["single.orders"]
    out, st = orc.integrand_batch(v, n, threads=2)
    assert (st & ~2).max() == 0
    assert bits_equal(out, data["single.values"])


@pytest.mark.parametrize("name", CASES)
def test_all_subsets_bit_identical(name):
    orc, data = _oracle(name)
    for env in range(2, 8):
        out, st = orc.all_subsets_batch(data[f"all{env}.vertices"], threads=2)
        assert st.max() == 0
        assert bits_equal(out, data[f"all{env}.values"]), env
    out, _ = orc.all_subsets_batch(data["audit6.vertices"])
    assert bits_equal(out, data["audit6.values"])


@pytest.mark.parametrize("name", CASES)
def test_filter_off_and_forced_fallback(name):
    orc, data = _oracle(name, z_safety=0.0)
    v, n = data["single.vertices"], data["single.orders"]
    out, _ = orc.integrand_batch(v, n)
    assert bits_equal(out, data["nofilter.values"])
    orc, data = _oracle(name, tol_fpm=1.0)
    out, st = orc.integrand_batch(v, n)
    assert bits_equal(out, data["fallback.values"])
    # every configuration of order >= 2 takes the LU fallback at TOL_FPM = 1
    assert np.all((st[n >= 2] & 2) == 2)
    assert int(data["fallback.count"]) > 0


def test_all_subset_matches_single_order_within_audit_tolerance():
    """tests/test_integrand_all_subsets.cpp:36-50: every subset of the
    all-subset path equals an independent single-order call within 2e-9."""
    orc, data = _oracle("physical_2x2")
    for v, all_values in zip(data["audit6.vertices"], data["audit6.values"]):
        for mask in range(1, 64):
            sub = v[[i for i in range(6) if (mask >> i) & 1]]
            direct, _ = orc.integrand(sub)
            scale = max(1.0, abs(direct), abs(all_values[mask]))
            assert abs(all_values[mask] - direct) <= 2e-9 + 2e-9 * scale


def test_fpm_known_answers():
    kats = np.load(f"{GOLDEN}/fpm_cdet_kats.npz")
    for n in range(1, 9):
        m = kats[f"fpm{n}.matrix"]
        for tag, tol, shift in (("auto", 0.0, -1.0), ("shift", 0.0, 0.37), ("tol", 1e-5, -1.0)):
            pm, _ = oracle_mat2pm(m, tol, shift)
            assert bits_equal(pm, kats[f"fpm{n}.{tag}"])
            # the audit's own check: fast minors vs pivoted determinants, 2e-10
            lu = oracle_minors_by_lu(m)
            assert bits_equal(lu, kats[f"fpm{n}.lu"])
            scale = np.maximum(1.0, np.maximum(np.abs(pm), np.abs(lu)))
            assert np.all(np.abs(pm - lu) <= 2e-10 + 2e-10 * scale)
    pm, fell_back = oracle_mat2pm(kats["pathology.matrix"], 1e-5, 0.0)
    assert fell_back == 1
    assert bits_equal(pm, kats["pathology.minors"])
    assert np.all(np.abs(pm - kats["pathology.lu"]) <= 2e-13)


def _partition_cumulant(mask, moments, blocks=0, product=1.0):
    """Independent set-partition cumulant (test_fpm_cdet.cpp:11-43)."""
    if mask == 0:
        k = blocks - 1
        return (-1) ** k * float(np.prod(np.arange(2, k + 1))) * product if k >= 0 else product
    anchor = mask & -mask
    rest = mask ^ anchor
    total = 0.0
    sub = rest
    while True:
        block = anchor | sub
        total += _partition_cumulant(mask ^ block, moments, blocks + 1, product * moments[block])
        if sub == 0:
            break
        sub = (sub - 1) & rest
    return total


def test_ztransform_known_answers():
    kats = np.load(f"{GOLDEN}/fpm_cdet_kats.npz")
    for order in range(1, 10):
        up, down = kats[f"z{order}.up"], kats[f"z{order}.down"]
        assert bits_equal(oracle_ztransform_all(up, down, order, 0.0, 0.0), kats[f"z{order}.all"])
        assert bits_equal(oracle_ztransform_all(up, down, order, 2e-16, 1e4),
                          kats[f"z{order}.all_filter"])
        assert bits_equal(oracle_ztransform(up, down, order, 2e-16, 1e4), kats[f"z{order}.single"])
        ones = np.ones_like(up)
        const = oracle_ztransform_all(ones, ones, order, 2e-16, 1e4)
        assert bits_equal(const, kats[f"z{order}.const"])
        if order >= 2:
            assert abs(const[-1]) < 1e-14  # the filter cancels a constant moment
        if order <= 7:
            moments = np.concatenate([[0.0], up * down])
            connected = oracle_ztransform_all(up, down, order, 0.0, 0.0)
            for mask in range(1, 1 << order):
                ref = _partition_cumulant(mask, moments)
                assert abs(connected[mask] - ref) <= 2e-11 + 2e-11 * max(1.0, abs(ref))


def test_descriptor_corner_routing():
    import ctypes as C
    from bindings import Oracle as _O
    lib = _O._lib()
    kats = np.load(f"{GOLDEN}/fpm_cdet_kats.npz")
    lib.oracle_lookup_descriptor.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double] + \
        [C.c_int] * 4 + [C.c_double, C.c_double] + [C.c_int] * 5 + \
        [C.POINTER(C.c_int), C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    for probe, expect in zip(kats["descriptor.probes"], kats["descriptor.values"]):
        ra, rb, t1, t2, upper = probe
        corner, index, u, v = C.c_int(), C.c_uint64(), C.c_double(), C.c_double()
        lib.oracle_lookup_descriptor(int(ra), int(rb), t1, t2, 0, 1, 2, 0, 8.0, 1e-13, 25, 25, 3,
                                     3, int(upper), C.byref(corner), C.byref(index), C.byref(u),
                                     C.byref(v))
        assert (corner.value, index.value) == (int(expect[0]), int(expect[1]))
        assert bits_equal([u.value, v.value], expect[2:])


@pytest.mark.parametrize("order,sites,r",
                         list(itertools.product(range(1, 17), (4, 9, 36, 64, 144), (1, 2))))
def test_prefactors(order, sites, r):
    hi, lo, ld = oracle_prefactors(order, sites, 1, r)
    exact = Fraction((-r) ** order, sites * int(np.prod(np.arange(1, order + 1, dtype=object))))
    assert abs(Fraction(hi) + Fraction(lo) - exact) <= abs(exact) * Fraction(1, 2 ** 100)
    if order >= 2:
        assert abs(Fraction(ld) - exact) <= abs(exact) * Fraction(1, 2 ** 52)


def test_long_double_truth_against_reference_high_precision():
    """The oracle's long double integrand (the truth the FP64 and split forms
    are measured against) agrees with the reference's own high-precision mode
    (VECTOR_REAL=long_double, INTEGRAND_REAL=double_double; golden values of
    precision_3x3.npz) about a hundred times more closely than the FP64
    integrand does, order by order. The residual is the reference forming
    (u, v) from double-double vertices, which the truth takes in double as
    both GPU forms do."""
    params, tables, _ = load_case("column_3x3")
    d = np.load(os.path.join(GOLDEN, "precision_3x3.npz"))
    orc = Oracle(params.runtime_scalars(), tables)
    truth, st = orc.integrand_ld_batch(d["vertices"], d["orders"], threads=4)
    fp64, _ = orc.integrand_batch(d["vertices"], d["orders"], threads=4)
    assert st.max() == 0
    assert bits_equal(fp64, d["values_double"])
    high, orders = d["values_high"], d["orders"]
    den = np.maximum(np.abs(high), 1e-300)
    for n in range(1, 9):
        sel = orders == n
        truth_err = np.median(np.abs(truth - high)[sel] / den[sel])
        fp64_err = np.median(np.abs(fp64 - high)[sel] / den[sel])
        assert truth_err <= max(1e-15, 0.01 * fp64_err), (n, truth_err, fp64_err)
