"""The compact minors workspace's placement rules, checked on the host.

tests/cpp/arena_check.cu includes cdet_kernels.cuh (the functions the minors
kernels, the queue kernel and the double-double kernels use to place their
level lists inside the shifted minors' arena) and checks, for every batch
order up to 10 and every matrix order up to it, that no list covers a live
shifted minor or the other list of its level and that everything stays inside
the arena. The GPU tests then show the values bit for bit; this pins the
layout arithmetic without a GPU.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "cdet-renyi-entanglement-hpc_gb300", "csrc")


def test_compact_arena_placement(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc")
                                    else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = tmp_path / "arena_check"
    subprocess.run([nvcc, "-std=c++17", "-O1", f"-I{CSRC}", f"-I{os.path.join(ROOT, 'include')}",
                    os.path.join(HERE, "cpp", "arena_check.cu"), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "0 violations" in out.stdout
