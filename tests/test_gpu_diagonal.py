"""cdet_diagonal_order1_density: the deterministic order-1 diagonal observable
(diagonal_green_observable.h:237-366) on the GPU.

Bit-identical to the reference on the golden tables (values written by the
reference build, tests/golden/make_diagonal_golden.py), and to the oracle on a
4x4 / degree-32 parameter set with unequal ALPHA_UP and ALPHA_DOWN (four
distinct tables built on the GPU by the in-tree precompute). U = 0 is refused
with the reference's message.
"""
import dataclasses
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from bindings import Oracle  # noqa: E402
from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.params import CdetParams, named_mask  # noqa: E402
from cdet_gb300.tables import build_tables  # noqa: E402
from helpers import GOLDEN, load_case  # noqa: E402

with open(os.path.join(GOLDEN, "diagonal_order1.json")) as f:
    GOLD = json.load(f)


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


def _bits(a):
    return np.asarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", sorted(GOLD))
def test_golden_bit_identical(name):
    params, tables, _ = load_case(name)
    got = CdetIntegrand(params, tables).diagonal_order1_density()
    want = [float.fromhex(GOLD[name][k]) for k in ("normalized", "twisted", "ordinary")]
    assert np.array_equal(_bits(got), _bits(want))


def test_unaliased_4x4_matches_oracle():
    params = CdetParams(n1=4, n2=4, beta="5", mu="0.2", u="3", alpha_up="0.55", alpha_down="0.4",
                        mask_sites=named_mask("origin_square", 4, 4, 1), cheb_nu=32, cheb_nv=32)
    tables = build_tables(params, device="cuda")
    got = CdetIntegrand(params, tables).diagonal_order1_density()
    host = {k: {kk: vv.cpu().numpy() for kk, vv in t.items()} for k, t in tables.items()}
    want = Oracle(params.runtime_scalars(), host).diagonal_order1(0.55, 0.4)
    assert np.array_equal(_bits(got), _bits(want))
    assert np.all(np.isfinite(got))


def test_zero_u_refused():
    @dataclasses.dataclass(frozen=True)
    class ZeroU(CdetParams):
        def runtime_scalars(self):
            s = super().runtime_scalars()
            s["u"] = 0.0
            return s

    params, tables, _ = load_case("column_3x3")
    zero = ZeroU(**{f.name: getattr(params, f.name) for f in dataclasses.fields(CdetParams)})
    with pytest.raises(RuntimeError, match="undefined for U = 0"):
        CdetIntegrand(zero, tables).diagonal_order1_density()
