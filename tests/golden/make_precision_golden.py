"""Golden values of the reference's high-precision integrand mode.

Run from the repository root with the environment variable REFERENCE set
to the reference checkout, after make_golden.py:

    REFERENCE=<reference checkout> python tests/golden/make_precision_golden.py

It loads the 3x3 one-column tables of column_3x3.npz into the reference's
own integrand (oracle/_ref/libcdet_ref.so), selects VECTOR_REAL=long_double
and INTEGRAND_REAL=double_double (precision_config.h:15-26; the error-floor
mode of cdet_integrand_evaluator.h:431-465), evaluates the fixture's
single-order configurations (orders 1..8 and the edge cases) and writes
precision_3x3.npz. The oracle's long double truth (oracle_integrand_ld) is
checked against these values; no test needs the reference at run time.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import bindings  # noqa: E402
from make_golden import CASES  # noqa: E402

REFERENCE = os.environ.get("REFERENCE", "")
if not REFERENCE:
    raise SystemExit("set REFERENCE to the reference checkout (the generator compiles its headers)")


def main() -> None:
    bindings.build(REFERENCE)
    data = np.load(os.path.join(HERE, "column_3x3.npz"))
    tables = {kind: {key: data[f"table.{kind}.{key}"] for key in
                     ("upper", "lower", "upper_corners", "lower_corners")} for kind in bindings.KINDS}
    ref = bindings.Reference()
    ref.configure(**CASES["column_3x3"])
    ref.set_tables(tables)
    vertices, orders = data["single.vertices"], data["single.orders"]
    fp64 = np.array([ref.integrand(v[:n]) for v, n in zip(vertices, orders)])
    ref.set_tables(tables, long_double=True)
    ref.set_precision("long_double", "double_double")
    high = np.array([ref.integrand(v[:n]) for v, n in zip(vertices, orders)])
    np.savez(os.path.join(HERE, "precision_3x3.npz"), vertices=vertices, orders=orders,
             values_double=fp64, values_high=high)
    rel = np.abs(fp64 - high) / np.maximum(np.abs(high), 1e-300)
    print("double vs high precision, median relative difference per order:",
          [float(np.median(rel[orders == n])) for n in range(1, 9)])


if __name__ == "__main__":
    main()
