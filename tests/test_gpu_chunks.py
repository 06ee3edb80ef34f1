"""cdet_load_chunks: the four tables streamed from a chunk directory of the
reference's workflow straight into HBM (tests/golden/chunks_2x2, written and
loaded back by the reference in tests/golden/make_chunk_golden.py).

On the loaded tables the FP64 integrand must equal the reference's integrand
on the same directory bit for bit, and so must the diagonal observable; the
directory's precomputed order-1 value is returned. A manifest that does not
match the context, or a directory without READY, is refused.
"""
import json
import os
import shutil

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from helpers import GOLDEN, params_from_reference_args  # noqa: E402

FIXTURE = os.path.join(GOLDEN, "chunks_2x2")
with open(os.path.join(GOLDEN, "chunks_2x2.json")) as f:
    META = json.load(f)


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield


def _bits(a):
    return np.asarray(a, dtype=np.float64).view(np.uint64)


def test_loaded_tables_reproduce_reference():
    params = params_from_reference_args(META["args"])
    gpu = CdetIntegrand(params, None)
    order1 = gpu.load_chunks(FIXTURE)
    assert order1 == (0.015857633184457098, 0.0)
    gold = np.load(os.path.join(GOLDEN, "physical_2x2.npz"))
    values, status = gpu.integrand_batch(gold["single.vertices"], gold["single.orders"])
    want = np.array([float.fromhex(x) for x in META["integrand"]])
    assert int(status.max()) & 1 == 0
    assert np.array_equal(_bits(values), _bits(want))
    diag = gpu.diagonal_order1_density()
    assert np.array_equal(_bits(diag), _bits([float.fromhex(x) for x in META["diagonal"]]))


def test_manifest_and_ready_checks(tmp_path):
    params = params_from_reference_args(dict(META["args"], beta="3"))
    with pytest.raises(RuntimeError, match="mismatch for BETA"):
        CdetIntegrand(params, None).load_chunks(FIXTURE)
    params = params_from_reference_args(dict(META["args"], nu=10, nv=10))
    with pytest.raises(RuntimeError, match="mismatch for CHEB_NU"):
        CdetIntegrand(params, None).load_chunks(FIXTURE)
    copy = tmp_path / "no_ready"
    shutil.copytree(FIXTURE, copy)
    os.remove(copy / "READY")
    with pytest.raises(RuntimeError, match="missing READY"):
        CdetIntegrand(params_from_reference_args(META["args"]), None).load_chunks(str(copy))
