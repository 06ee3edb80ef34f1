"""Pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the in-tree libcdet_gb300.so; the
rest run on the CPU (the C oracle against golden vectors, host logic, and the
library's exported symbols).
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("cdet-renyi-entanglement-hpc_gb300", "oracle", "tests"):
    path = os.path.join(ROOT, sub)
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
