"""The Green-table precompute run on the GPU, against the reference's tables.

The same restatement as test_precompute.py, with every batched solve and
transform on the CUDA device (cuSOLVER and cuBLAS through torch): the tables
must match the reference-built golden tables to 1e-14 absolute on
coefficients and corners, and the direct kernel solves of the reference's
Chebyshev audit configuration to 1e-13.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300.params import CdetParams, named_mask  # noqa: E402
from cdet_gb300.tables import ReplicaGreenCalculator, build_tables  # noqa: E402
from helpers import GOLDEN, KEYS, KINDS, load_case  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


@pytest.mark.parametrize("name", ["physical_2x2", "column_3x3"])
def test_gpu_tables_match_reference(name):
    params, ref_tables, _ = load_case(name)
    mine = build_tables(params, device="cuda")
    for kind in KINDS:
        for key in KEYS:
            a = np.asarray(ref_tables[kind][key])
            t = mine[kind][key]
            assert t.is_cuda
            b = t.cpu().numpy()
            assert a.shape == b.shape
            assert np.max(np.abs(a - b)) <= 1e-14, (kind, key, np.max(np.abs(a - b)))
    if params.alpha_equal:
        assert mine["twisted_down"] is mine["twisted_up"]


def test_gpu_chebyshev_audit_configuration():
    """3x3, beta = 8, mu = -0.4, first_row, degree 25 (the reference's
    tests/test_chebyshev_accuracy.cpp:61-64), built on the GPU."""
    data = np.load(f"{GOLDEN}/precompute_3x3.npz")
    p = CdetParams(n1=3, n2=3, beta="8", mu="-0.4", u="2", mask_sites=named_mask("first_row", 3, 3),
                   cheb_nu=25, cheb_nv=25)
    mine = build_tables(p, device="cuda")
    for kind in ("twisted_up", "ordinary_up"):
        for key in ("upper", "lower"):
            idx = data[f"pre.{kind}.{key}.idx"]
            got = mine[kind][key].cpu().numpy()[idx]
            assert np.max(np.abs(got - data[f"pre.{kind}.{key}.val"])) <= 1e-14
        for key in ("upper_corners", "lower_corners"):
            assert np.max(np.abs(mine[kind][key].cpu().numpy() - data[f"pre.{kind}.{key}"])) <= 1e-13
    calc = ReplicaGreenCalculator(3, 3, 8.0, -0.4, True, named_mask("first_row", 3, 3), device="cuda")
    for (ra, rb, t, tp, upper), want in zip(((0, 1, 3.1, 1.2, 1), (1, 1, 0.7, 5.5, 0), (0, 0, 6.0, 2.0, 1)),
                                            data["pre.direct"]):
        g0 = calc.green_sector(0, np.array([t]), np.array([tp]), bool(upper))[0]
        g1 = calc.green_sector(1, np.array([t]), np.array([tp]), bool(upper))[0]
        if ra == rb:
            got = ((g0 + g1) / 2).real
        elif ra == 0:
            got = (1j * (g0 - g1) / 2).real
        else:
            got = (-1j * (g0 - g1) / 2).real
        assert np.max(np.abs(got.cpu().numpy() - want)) <= 1e-13
