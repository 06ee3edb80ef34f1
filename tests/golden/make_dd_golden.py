"""Golden values of the reference's double-double integrand mode.

Run from the repository root with the environment variable REFERENCE set
to the reference checkout, after make_golden.py:

    REFERENCE=<reference checkout> python tests/golden/make_dd_golden.py

It loads the reference-built tables of physical_2x2.npz (distinct up and down
tables, U = 1.7 whose DoubleDouble has a low part) and column_3x3.npz into the
reference's own integrand (oracle/_ref/libcdet_ref.so), selects
VECTOR_REAL=double and INTEGRAND_REAL=double_double (precision_config.h:15-26,
cdet_integrand_evaluator.h:431-465) and evaluates seeded configurations of
orders 1..10 (the fixture's orders 1..8 with their edge cases, then uniform
ones at orders 9 and 10): with the default settings, with the round-off
filter off (ZTRANSFORM_SAFETY_FACTOR = 0) and with the LU fallback forced
(TOL_FPM = 1). It writes dd_mode.npz; no test needs the reference at run time.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "cdet-renyi-entanglement-hpc_gb300"))

import bindings  # noqa: E402
from cdet_gb300.synthetic import uniform_configurations  # noqa: E402
from make_golden import CASES  # noqa: E402

REFERENCE = os.environ.get("REFERENCE", "")
if not REFERENCE:
    raise SystemExit("set REFERENCE to the reference checkout (the generator compiles its headers)")

VARIANTS = {"default": {}, "nofilter": {"z_safety": "0"}, "fallback": {"tol_fpm": "1"}}


def main() -> None:
    bindings.build(REFERENCE)
    ref = bindings.Reference()
    out = {}
    for case in ("physical_2x2", "column_3x3"):
        data = np.load(os.path.join(HERE, f"{case}.npz"))
        tables = {kind: {key: data[f"table.{kind}.{key}"] for key in
                         ("upper", "lower", "upper_corners", "lower_corners")} for kind in bindings.KINDS}
        v8, n8 = data["single.vertices"], data["single.orders"]
        v10 = uniform_configurations(910 + len(case), 24, 10)
        n10 = np.array([9] * 12 + [10] * 12, dtype=np.int32)
        vertices = np.zeros((len(n8) + len(n10), 10, 4))
        vertices[:len(n8), :8] = v8
        vertices[len(n8):] = v10
        orders = np.concatenate([n8, n10]).astype(np.int32)
        for variant, over in VARIANTS.items():
            ref.configure(**dict(CASES[case], **over))
            ref.set_tables(tables)
            ref.set_precision("double", "double_double")
            values = np.array([ref.integrand(v[:n]) for v, n in zip(vertices, orders)])
            out[f"{case}.{variant}.values"] = values
            print(case, variant, "orders 1..10:", len(values), "values")
        out[f"{case}.vertices"] = vertices
        out[f"{case}.orders"] = orders
    np.savez(os.path.join(HERE, "dd_mode.npz"), **out)


if __name__ == "__main__":
    main()
