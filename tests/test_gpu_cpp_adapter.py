"""The C++20 drop-in adapter (include/cdet_gb300.hpp) on the GPU.

Builds tests/cpp/adapter_check.cpp against the in-tree library, feeds it the
golden 2x2 parameter set (four distinct tables), and checks that the
reference-named C++ entry points return the reference's values bit for bit.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300 import lib as L  # noqa: E402
from cdet_gb300.build import INCLUDE, LIB_DIR  # noqa: E402
from helpers import bits_equal, load_case  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def test_cpp_adapter_matches_golden(tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    params, tables, data = load_case("physical_2x2")
    sc = params.runtime_scalars()
    rs = L.RuntimeScalars(**{k: sc[k] for k, _ in L.RuntimeScalars._fields_})
    (tmp_path / "scalars.bin").write_bytes(bytes(rs))
    kinds = ["twisted_up", "twisted_down", "ordinary_up", "ordinary_down"]
    alias = []
    for i, k in enumerate(kinds):
        src = next((j for j in range(i) if tables[kinds[j]] is tables[k]), -1)
        alias.append(src)
        if src < 0:
            for part in ("upper", "lower", "upper_corners", "lower_corners"):
                np.asarray(tables[k][part], dtype=np.float64).tofile(tmp_path / f"{k}.{part}.bin")
    np.array(alias, dtype=np.int32).tofile(tmp_path / "alias.bin")
    np.ascontiguousarray(data["single.vertices"]).tofile(tmp_path / "vertices.bin")
    np.ascontiguousarray(data["single.orders"], dtype=np.int32).tofile(tmp_path / "orders.bin")
    np.ascontiguousarray(data["audit6.vertices"]).tofile(tmp_path / "envelopes.bin")
    exe = tmp_path / "adapter_check"
    subprocess.run(["g++", "-std=c++20", "-O2", f"-I{INCLUDE}", os.path.join(HERE, "cpp", "adapter_check.cpp"),
                    f"-L{LIB_DIR}", "-lcdet_gb300", f"-Wl,-rpath,{LIB_DIR}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    single = np.fromfile(tmp_path / "single_out.bin")
    assert bits_equal(single, data["single.values"])
    allv = np.fromfile(tmp_path / "all_out.bin").reshape(-1, 64)
    assert bits_equal(allv, data["audit6.values"])
