"""The C-ABI library loads and exports every symbol include/cdet_gb300.h
declares (no GPU needed: nothing is called)."""
import ctypes as C
import os
import re

from cdet_gb300 import build as cuda_build
from cdet_gb300 import lib as L


def test_header_symbols_exported():
    cuda_build.build()
    lib = C.CDLL(cuda_build.LIB_PATH)
    with open(os.path.join(cuda_build.INCLUDE, "cdet_gb300.h")) as f:
        header = f.read()
    declared = set(re.findall(r"^(?:int|void|const char\*)\s+(cdet_\w+)\(", header, re.M))
    assert declared == set(L.EXPORTED)
    for name in declared:
        assert hasattr(lib, name), name


def test_no_cpu_fallback_when_library_missing(tmp_path):
    import pytest
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        L._LIB = None
        try:
            L.load(str(tmp_path / "missing.so"))
        finally:
            L._LIB = None
