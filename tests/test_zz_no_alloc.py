"""cdet_integrand_device_noalloc: the FP64 integrand on fixed static scratch.

For callers that must not let the library allocate device memory (a process
that has handed HBM to its tables or to a pool allocator of its own). Through
the C ABI, two calls in a row must equal the ordinary entry point bit for bit
(the FP64 form's tolerance in every other test), at a mixed-order batch whose
minors run from shared memory and at orders 12 and 14, whose minors use the
workspace carved from the array. The first call on a device is the set-up
call: it looks up the array's device address, which loads the library's
module holding the array (the 64 MiB then stays with the GPU until exit). The
calls after it must leave the device's free memory unchanged, also when one
is captured into a CUDA graph and replayed. A batch too large for the fixed
scratch must be refused with a message. This file sorts
last so that a run stopping at the first failure has already run every other
test.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300 import lib as L  # noqa: E402
from cdet_gb300.integrand import CdetIntegrand  # noqa: E402
from cdet_gb300.params import CdetParams, named_mask  # noqa: E402
from cdet_gb300.synthetic import truncated_geometric_orders, uniform_configurations  # noqa: E402
from cdet_gb300.tables import build_tables  # noqa: E402


def test_noalloc_matches_device_entry_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    params = CdetParams(n1=4, n2=4, beta="6", mu="0", u="2",
                        mask_sites=named_mask("origin_square", 4, 4, 1), cheb_nu=32, cheb_nv=32)
    tables = build_tables(params, device="cuda")  # device tables: bound, not copied
    gpu = CdetIntegrand(params, tables)
    batch, nmax = 512, 8
    v = torch.from_numpy(uniform_configurations(4242, batch, nmax)).cuda()
    o = torch.from_numpy(truncated_geometric_orders(4243, batch, 0.3, nmax)).cuda()
    ref_values = torch.empty(batch, dtype=torch.float64, device="cuda")
    ref_status = torch.empty(batch, dtype=torch.int32, device="cuda")
    gpu.integrand_device(v, o, ref_values, ref_status)
    values = [torch.full((batch,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(3)]
    status = [torch.full((batch,), -1, dtype=torch.int32, device="cuda") for _ in range(3)]
    # set-up call (first on this device)
    assert gpu.integrand_device_noalloc(v, o, values[0], status[0]) == L.CDET_OK, L.last_error()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for k in (1, 2):
        rc = gpu.integrand_device_noalloc(v, o, values[k], status[k])
        assert rc == L.CDET_OK, L.last_error()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before  # the calls allocate nothing on the device
    want = ref_values.cpu().numpy().view(np.uint64)
    for k in range(3):
        assert np.array_equal(values[k].cpu().numpy().view(np.uint64), want)
        assert np.array_equal(status[k].cpu().numpy(), ref_status.cpu().numpy())


def test_noalloc_in_a_cuda_graph():
    """The use the entry exists for: after the set-up call (outside any
    capture), one call captured into a CUDA graph on a side stream and
    replayed twice; every replay gives the ordinary entry point's values and
    statuses bit for bit and leaves the device's free memory as it was."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    params = CdetParams(n1=4, n2=4, beta="6", mu="0", u="2",
                        mask_sites=named_mask("origin_square", 4, 4, 1), cheb_nu=32, cheb_nv=32)
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    batch, nmax = 384, 8
    v = torch.from_numpy(uniform_configurations(5252, batch, nmax)).cuda()
    o = torch.from_numpy(truncated_geometric_orders(5253, batch, 0.3, nmax)).cuda()
    ref_values = torch.empty(batch, dtype=torch.float64, device="cuda")
    ref_status = torch.empty(batch, dtype=torch.int32, device="cuda")
    gpu.integrand_device(v, o, ref_values, ref_status)
    values = torch.full((batch,), float("nan"), dtype=torch.float64, device="cuda")
    status = torch.full((batch,), -1, dtype=torch.int32, device="cuda")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        assert gpu.integrand_device_noalloc(v, o, values, status, side) == L.CDET_OK, L.last_error()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        rc = gpu.integrand_device_noalloc(v, o, values, status, torch.cuda.current_stream())
    assert rc == L.CDET_OK, L.last_error()
    values.fill_(float("nan"))
    status.fill_(-1)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    want_v, want_s = ref_values.cpu().numpy().view(np.uint64), ref_status.cpu().numpy()
    for _ in range(2):
        graph.replay()
        torch.cuda.synchronize()
        assert np.array_equal(values.cpu().numpy().view(np.uint64), want_v)
        assert np.array_equal(status.cpu().numpy(), want_s)
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_noalloc_rejects_oversized_batch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    params = CdetParams(n1=3, n2=3, beta="4", mu="0", u="2",
                        mask_sites=named_mask("first_column", 3, 3), cheb_nu=8, cheb_nv=8)
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    batch, nmax = 65536, 10
    v = torch.zeros((batch, nmax, 4), dtype=torch.float64, device="cuda")
    o = torch.full((batch,), nmax, dtype=torch.int32, device="cuda")
    out = torch.empty(batch, dtype=torch.float64, device="cuda")
    st = torch.empty(batch, dtype=torch.int32, device="cuda")
    rc = gpu.integrand_device_noalloc(v, o, out, st)
    assert rc == L.CDET_ERR_INVALID
    assert "split the batch" in L.last_error()


@pytest.mark.parametrize("order,batch", [(12, 256), (14, 96)])
def test_noalloc_high_order_matches_device_entry(order, batch):
    """Orders whose minors keep their workspace in global memory: the
    workspace and the LU-fallback scratch are carved from what the batch
    leaves of the array."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    params = CdetParams(n1=3, n2=3, beta="4", mu="0", u="2",
                        mask_sites=named_mask("first_column", 3, 3), cheb_nu=16, cheb_nv=16)
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    v = torch.from_numpy(uniform_configurations(5150 + order, batch, order)).cuda()
    o = torch.full((batch,), order, dtype=torch.int32, device="cuda")
    ref_values = torch.empty(batch, dtype=torch.float64, device="cuda")
    ref_status = torch.empty(batch, dtype=torch.int32, device="cuda")
    gpu.integrand_device(v, o, ref_values, ref_status)
    values = [torch.full((batch,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)]
    status = [torch.full((batch,), -1, dtype=torch.int32, device="cuda") for _ in range(2)]
    assert gpu.integrand_device_noalloc(v, o, values[0], status[0]) == L.CDET_OK, L.last_error()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    assert gpu.integrand_device_noalloc(v, o, values[1], status[1]) == L.CDET_OK, L.last_error()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    want = ref_values.cpu().numpy().view(np.uint64)
    assert int(ref_status.max()) == 0
    for k in range(2):
        assert np.array_equal(values[k].cpu().numpy().view(np.uint64), want)
        assert np.array_equal(status[k].cpu().numpy(), ref_status.cpu().numpy())


def test_noalloc_limits_by_order():
    """The documented limits: 224 configurations of order 14 are accepted,
    232 refused; order 16 is refused at any batch."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    params = CdetParams(n1=3, n2=3, beta="4", mu="0", u="2",
                        mask_sites=named_mask("first_column", 3, 3), cheb_nu=8, cheb_nv=8)
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    for order, batch, ok in ((14, 224, True), (14, 232, False), (16, 1, False)):
        v = torch.from_numpy(uniform_configurations(77 + batch, batch, order)).cuda()
        o = torch.full((batch,), order, dtype=torch.int32, device="cuda")
        out = torch.empty(batch, dtype=torch.float64, device="cuda")
        st = torch.empty(batch, dtype=torch.int32, device="cuda")
        rc = gpu.integrand_device_noalloc(v, o, out, st)
        if ok:
            assert rc == L.CDET_OK, L.last_error()
            torch.cuda.synchronize()
        else:
            assert rc == L.CDET_ERR_INVALID
            assert "split the batch" in L.last_error()
