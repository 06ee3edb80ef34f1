"""The C++20 drop-in adapter (include/cdet_gb300.hpp) on the GPU.

Builds tests/cpp/adapter_check.cpp against the in-tree library, feeds it the
golden 2x2 parameter set (four distinct tables), and checks that the
reference-named C++ entry points return the reference's values bit for bit,
and that McmcmcChains runs the reference's histogram-seeded chains of that set
(final vertices, lambdas, generator states and chosen counts bit for bit,
statistics to 1e-15, half-way checkpoints with the reference's state).
"""
import ctypes as C
import json
import os
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cdet_gb300 import lib as L  # noqa: E402
from cdet_gb300.build import INCLUDE, LIB_DIR  # noqa: E402
from cdet_gb300.mcmcmc import mt64_outputs, read_checkpoint  # noqa: E402
from helpers import GOLDEN, bits_equal, load_case  # noqa: E402

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
    # MCMCMC inputs: the golden histogram-seeded chains of this parameter set
    with open(os.path.join(GOLDEN, "mcmcmc_chains.json")) as f:
        run = json.load(f)["physical_2x2"]
    gold = np.load(os.path.join(GOLDEN, "mcmcmc_chains.npz"))
    h = run["histogram"]
    np.array([run["order_min"], run["order_max"], run["envelope"], run["adapt_interval"], run["warmup"],
              run["production"], run["checkpoint_production"], h["tau_bins"]], dtype=np.int32).tofile(
        tmp_path / "mc_ints.bin")
    np.array([run["adapt_rate"]]).tofile(tmp_path / "mc_rate.bin")
    np.array(run["lambdas"], dtype=np.float64).tofile(tmp_path / "mc_lambdas.bin")
    gold["physical_2x2.hist.seeds"].astype(np.uint64).tofile(tmp_path / "mc_seeds.bin")
    for key in ("tau", "space", "replica"):
        np.asarray(gold[f"physical_2x2.hist.{key}"], dtype=np.float64).tofile(tmp_path / f"mc_{key}.bin")
    exe = tmp_path / "adapter_check"
    subprocess.run(["g++", "-std=c++20", "-O2", f"-I{INCLUDE}", os.path.join(HERE, "cpp", "adapter_check.cpp"),
                    f"-L{LIB_DIR}", "-lcdet_gb300", f"-Wl,-rpath,{LIB_DIR}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    single = np.fromfile(tmp_path / "single_out.bin")
    assert bits_equal(single, data["single.values"])
    allv = np.fromfile(tmp_path / "all_out.bin").reshape(-1, 64)
    assert bits_equal(allv, data["audit6.values"])
    # the chains are the reference's chains; their results its results
    env, chains = run["envelope"], len(gold["physical_2x2.hist.seeds"])
    verts = np.fromfile(tmp_path / "mc_vertices_out.bin").reshape(chains, env, 4)
    assert bits_equal(verts, gold["physical_2x2.hist.vertices"])
    rng = np.fromfile(tmp_path / "mc_rng_out.bin", dtype=np.uint64).reshape(chains, 313)
    for c in range(chains):
        assert np.array_equal(mt64_outputs(rng[c], 8), gold["physical_2x2.hist.rng"][c]), c
    lams = np.fromfile(tmp_path / "mc_lambdas_out.bin").reshape(chains, env + 1)
    assert bits_equal(lams, gold["physical_2x2.run.lambdas"])
    counts = np.fromfile(tmp_path / "mc_counts_out.bin", dtype=np.uint64).reshape(chains, -1)
    assert np.array_equal(counts, gold["physical_2x2.run.u64"])
    means = np.fromfile(tmp_path / "mc_means_out.bin").reshape(chains, env + 1)
    want = gold["physical_2x2.run.stats"][:, 2:, 1] + gold["physical_2x2.run.stats"][:, 2:, 2]
    assert np.allclose(means, want, rtol=1e-15, atol=0)
    ratios = np.fromfile(tmp_path / "mc_ratios_out.bin")
    want_r = gold["physical_2x2.run.ratios"][:, 0] + gold["physical_2x2.run.ratios"][:, 1]
    o = slice(run["order_min"], run["order_max"] + 1)
    assert np.allclose(ratios[o], want_r[o], rtol=1e-15, atol=0)
    ck_dir = os.path.join(GOLDEN, "mcmcmc_checkpoints", "physical_2x2")
    for fname in sorted(os.listdir(ck_dir)):
        got, ref = read_checkpoint(str(tmp_path / "ck_half" / fname)), read_checkpoint(os.path.join(ck_dir, fname))
        for field in ("rng_state", "lambdas", "vertices", "warmup_block_counts"):
            assert bytes(getattr(got, field)) == bytes(getattr(ref, field)), (fname, field)
