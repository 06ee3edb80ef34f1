"""The N-GPU host logic on the CPU: two ranks under torchrun with the gloo
backend (127.0.0.1), as the benchmark runs under torchrun with NCCL.

Each rank must see its own RANK / LOCAL_RANK / WORLD_SIZE, draw a batch of
configurations distinct from the other rank's and reproducible from its seed
stream, and both ranks must agree on the maximum of their times; the
whole-job rate is every rank's configurations over that time. The reference
arm under torchrun runs on rank 0 alone: another rank exits 0 without output.
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

pytest.importorskip("torch")

from cdet_gb300 import replicas  # noqa: E402
from cdet_gb300.synthetic import uniform_configurations  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks(tmp_path):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}",
           os.path.join(HERE, "replica_worker.py"), str(tmp_path)]
    proc = subprocess.run(cmd, capture_output=True, text=True, timeout=240)
    assert proc.returncode == 0, proc.stderr[-2000:]
    seen = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r, s in enumerate(seen):
        assert (s["world"], s["rank"], s["local_rank"]) == (2, r, r)
        assert s["slowest"] == 1.5
        assert s["throughput"] == pytest.approx(65536 * 5 * 2 / 1.5)
        for q in range(2):
            want = uniform_configurations(replicas.batch_seed(q, 0), 4, 3)
            assert np.array_equal(np.array(s["batches"][q]), want)
    assert not np.array_equal(np.array(seen[0]["batches"][0]), np.array(seen[0]["batches"][1]))


def test_reference_arm_other_ranks_exit(tmp_path):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    proc = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                           "--warmup", "3"], capture_output=True, text=True, env=env, timeout=240)
    assert proc.returncode == 0, proc.stderr[-2000:]
    assert proc.stdout.strip() == ""


def test_single_rank_defaults(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.rank_info() == (1, 0, 0)
    assert replicas.max_over_ranks(3.25, 1) == 3.25
    assert replicas.batch_seed(0, 0) != replicas.batch_seed(1, 0)
    assert replicas.batch_seed(0, 1) != replicas.batch_seed(0, 0)
