"""Golden values of the order-1 diagonal observable, from the reference itself.

Run from the repository root with the environment variable REFERENCE set
to the reference checkout, after make_golden.py:

    REFERENCE=<reference checkout> python tests/golden/make_diagonal_golden.py

For each golden parameter set it loads the reference-built tables stored in
<name>.npz into the reference build (oracle/_ref/libcdet_ref.so), evaluates
normalized_log_partition_first_order_density_dd and its twisted and ordinary
parts (diagonal_green_observable.h:237-327), and writes them as exact hex
floats to diagonal_order1.json.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import bindings  # noqa: E402
from make_golden import CASES, REFERENCE  # noqa: E402

KINDS = ("twisted_up", "twisted_down", "ordinary_up", "ordinary_down")
KEYS = ("upper", "lower", "upper_corners", "lower_corners")


def main():
    bindings.build(REFERENCE)
    ref = bindings.Reference()
    out = {}
    for name, args in CASES.items():
        data = np.load(os.path.join(HERE, f"{name}.npz"))
        ref.configure(**args)
        ref.set_tables({k: {key: data[f"table.{k}.{key}"] for key in KEYS} for k in KINDS})
        vals = ref.diagonal_order1()
        out[name] = {"normalized": float(vals[0]).hex(), "normalized_lo": float(vals[3]).hex(),
                     "twisted": float(vals[1]).hex(), "ordinary": float(vals[2]).hex()}
    with open(os.path.join(HERE, "diagonal_order1.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
