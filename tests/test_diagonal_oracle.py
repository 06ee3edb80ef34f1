"""The order-1 diagonal observable's C restatement against the reference.

diagonal_order1.json holds the reference build's
normalized_log_partition_first_order_density_dd and its twisted and ordinary
parts (diagonal_green_observable.h:237-327) on the golden tables, as exact hex
floats (tests/golden/make_diagonal_golden.py). The oracle must reproduce them
bit for bit, including the unaliased 2x2 set (ALPHA_UP != ALPHA_DOWN).
"""
import json
import os

import numpy as np
import pytest

from bindings import Oracle
from helpers import GOLDEN, load_case

with open(os.path.join(GOLDEN, "diagonal_order1.json")) as f:
    GOLD = json.load(f)


@pytest.mark.parametrize("name", sorted(GOLD))
def test_diagonal_order1_bit_identical(name):
    params, tables, _ = load_case(name)
    orc = Oracle(params.runtime_scalars(), tables)
    got = orc.diagonal_order1(float(params.alpha_up), float(params.alpha_down))
    want = np.array([float.fromhex(GOLD[name][k]) for k in ("normalized", "twisted", "ordinary")])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    assert float.fromhex(GOLD[name]["normalized_lo"]) == 0.0  # a double cast to DoubleDouble


def test_diagonal_order1_rejects_zero_u():
    params, tables, _ = load_case("column_3x3")
    scalars = params.runtime_scalars()
    scalars["u"] = 0.0
    with pytest.raises(RuntimeError, match="U = 0"):
        Oracle(scalars, tables).diagonal_order1(0.0, 0.0)
