"""Generates the golden vectors in this directory from the reference itself.

Run from the repository root with the environment variable REFERENCE set
to the reference checkout:

    REFERENCE=<reference checkout> python tests/golden/make_golden.py

It builds oracle/_ref/libcdet_ref.so (the reference's own headers compiled
with the quad-precision Boost stand-in) and records, for a few small
parameter sets, the reference-built Green tables together with the
reference's outputs on seeded inputs. The known-answer inputs follow the
reference's audit tests (tests/test_fpm_cdet.cpp, test_integrand_all_subsets.cpp,
test_chebyshev_accuracy.cpp). Tests read only the .npz files written here; no
test needs the reference at run time.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import bindings  # noqa: E402

REFERENCE = os.environ.get("REFERENCE", "")
if not REFERENCE:
    raise SystemExit("set REFERENCE to the reference checkout (the generator compiles its headers)")

# Parameter sets: name -> reference configure() arguments.
CASES = {
    # tests/test_integrand_all_subsets.cpp:11-28 (alpha_up != alpha_down: four tables)
    "physical_2x2": dict(n1=2, n2=2, beta="2.5", mu="0.3", u="1.7", alpha_up="0.55",
                         alpha_down="0.4", pbc=True, mask_name="first_row", radius=0, nu=18, nv=18),
    # the 3x3 one-column configuration at a small Chebyshev degree (aliased tables)
    "column_3x3": dict(n1=3, n2=3, beta="4", mu="0", u="2", alpha_up="0", alpha_down="0",
                       pbc=True, mask_name="first_column", radius=0, nu=10, nv=10),
}


def table_arrays(tables, prefix):
    out = {}
    for kind, t in tables.items():
        for key, arr in t.items():
            out[f"{prefix}{kind}.{key}"] = arr
    return out


def make_case(ref, name, args, rng):
    ref.configure(**args)
    ref.build_tables(4)
    tables = ref.get_tables()
    data = table_arrays(tables, "table.")
    # single-order integrand, orders 1..8, uniform vertices plus edge cases
    singles_v, singles_n, singles_out = [], [], []
    for n in range(1, 9):
        for _ in range(12):
            v = rng.random((n, 4))
            singles_v.append(np.pad(v, ((0, 8 - n), (0, 0))))
            singles_n.append(n)
            singles_out.append(ref.integrand(v))
    # edge cases: tau exactly 0 (corner path), coordinates at the top of [0, 1),
    # repeated vertices (equal times), tau ties between different sites
    edge = [
        np.array([[0.0, 0.2, 0.7, 0.1], [0.5, 0.5, 0.5, 0.9], [0.25, 0.9, 0.1, 0.6]]),
        np.array([[0.999999999, 0.999999999, 0.999999999, 0.999999999],
                  [0.0, 0.0, 0.0, 0.0], [0.3, 0.3, 0.3, 0.3]]),
        np.array([[0.4, 0.1, 0.1, 0.2], [0.4, 0.1, 0.1, 0.2], [0.7, 0.8, 0.3, 0.7],
                  [0.4, 0.6, 0.9, 0.8]]),
        np.array([[0.0, 0.3, 0.3, 0.3], [0.0, 0.6, 0.6, 0.6]]),
        np.array([[0.0, 0.3, 0.3, 0.3]]),
        np.array([[1e-15, 0.5, 0.5, 0.5], [0.9, 0.1, 0.2, 0.3]]),
    ]
    for v in edge:
        singles_v.append(np.pad(v, ((0, 8 - v.shape[0]), (0, 0))))
        singles_n.append(v.shape[0])
        singles_out.append(ref.integrand(v))
    data["single.vertices"] = np.array(singles_v)
    data["single.orders"] = np.array(singles_n, dtype=np.int32)
    data["single.values"] = np.array(singles_out)
    # all-subset integrand, envelopes 2..7
    for env in range(2, 8):
        vs = rng.random((6, env, 4))
        data[f"all{env}.vertices"] = vs
        data[f"all{env}.values"] = np.array([ref.all_subsets(v) for v in vs])
    # the reference audit's 6-vertex envelopes, U(0.01, 0.99) (test_integrand_all_subsets.cpp:29-33)
    vs = 0.01 + 0.98 * rng.random((5, 6, 4))
    data["audit6.vertices"] = vs
    data["audit6.values"] = np.array([ref.all_subsets(v) for v in vs])
    # roundoff filter off (ZTRANSFORM_SAFETY_FACTOR = 0)
    ref.configure(**dict(args, z_safety="0"))
    ref.set_tables(tables)
    data["nofilter.values"] = np.array([ref.integrand(v[:n]) for v, n in
                                        zip(data["single.vertices"], data["single.orders"])])
    # forced whole-matrix LU fallback (TOL_FPM = 1: every pivot is "tiny")
    ref.configure(**dict(args, tol_fpm="1"))
    ref.set_tables(tables)
    ref.lib.ref_reset_counters()
    data["fallback.values"] = np.array([ref.integrand(v[:n]) for v, n in
                                        zip(data["single.vertices"], data["single.orders"])])
    data["fallback.count"] = np.array(ref.fpm_fallbacks())
    ref.configure(**args)
    ref.set_tables(tables)
    return data


def make_kats(ref, rng):
    """Known-answer inputs of tests/test_fpm_cdet.cpp with reference outputs."""
    data = {}
    for n in range(1, 9):
        m = rng.uniform(-0.8, 0.8, (n, n))
        m[np.diag_indices(n)] += 1.2 + 0.1 * np.arange(n)
        data[f"fpm{n}.matrix"] = m
        for tag, tol, shift in (("auto", 0.0, -1.0), ("shift", 0.0, 0.37), ("tol", 1e-5, -1.0)):
            data[f"fpm{n}.{tag}"] = ref.mat2pm(m, tol, shift)
        data[f"fpm{n}.lu"] = ref.minors_by_lu(m)
    path = np.array([[0.0, 1.0, 0.2], [1.0, 0.3, -0.1], [0.2, -0.1, 1.4]])
    data["pathology.matrix"] = path
    data["pathology.minors"] = ref.mat2pm(path, 1e-5, 0.0)
    data["pathology.lu"] = ref.minors_by_lu(path)
    for order in range(1, 10):
        up = 0.6 + 0.08 * rng.uniform(-0.8, 0.8, (1 << order) - 1)
        down = 0.7 + 0.08 * rng.uniform(-0.8, 0.8, (1 << order) - 1)
        data[f"z{order}.up"] = up
        data[f"z{order}.down"] = down
        data[f"z{order}.all"] = ref.ztransform_all(up, down, order, 0.0, 0.0)
        data[f"z{order}.all_filter"] = ref.ztransform_all(up, down, order, 2e-16, 1e4)
        data[f"z{order}.single"] = np.array(ref.ztransform(up, down, order, 2e-16, 1e4))
        ones = np.ones((1 << order) - 1)
        data[f"z{order}.const"] = ref.ztransform_all(ones, ones, order, 2e-16, 1e4)
    # BRANCH_EPSILON corner routing (test_fpm_cdet.cpp:116-128)
    probes = [(0, 1, 0.5e-13, 0.25e-13, 1), (0, 1, 2.0e-13, 1.0e-13, 1), (0, 1, 0.25e-13, 0.5e-13, 0),
              (1, 0, 3.0, 1.5, 1), (1, 1, 2.0, 6.0, 0)]
    desc = []
    for ra, rb, t1, t2, upper in probes:
        desc.append(ref.lookup_descriptor(ra, rb, t1, t2, 0, 1, 2, 0, 8.0, 1e-13, 25, 25, 3, 3, upper))
    data["descriptor.probes"] = np.array(probes, dtype=np.float64)
    data["descriptor.values"] = np.array(desc, dtype=np.float64)
    return data


def make_vertex_samples(ref):
    data = {}
    for seed in (1, 12345, 2026101401):
        data[f"mt{seed}"] = ref.sample_vertices(seed, 200)
    return data


def make_precompute(ref):
    """Sampled table entries and direct kernel solves of the Chebyshev audit
    configuration (tests/test_chebyshev_accuracy.cpp:61-64)."""
    args = dict(n1=3, n2=3, beta="8", mu="-0.4", u="2", alpha_up="0", alpha_down="0", pbc=True,
                mask_name="first_row", radius=0, nu=25, nv=25)
    ref.configure(**args)
    ref.build_tables(4)
    tables = ref.get_tables()
    rng = np.random.default_rng(7)
    data = {}
    for kind in ("twisted_up", "ordinary_up"):
        for key in ("upper", "lower"):
            idx = rng.choice(tables[kind][key].size, 4000, replace=False)
            data[f"pre.{kind}.{key}.idx"] = idx
            data[f"pre.{kind}.{key}.val"] = tables[kind][key][idx]
        for key in ("upper_corners", "lower_corners"):
            data[f"pre.{kind}.{key}"] = tables[kind][key]
    direct = []
    for ra, rb, t, tp, upper in ((0, 1, 3.1, 1.2, 1), (1, 1, 0.7, 5.5, 0), (0, 0, 6.0, 2.0, 1)):
        direct.append(ref.green_replica(3, 3, 8.0, -0.4, True, "first_row", 0, ra, rb, t, tp, upper))
    data["pre.direct"] = np.array(direct)
    return data


def main():
    bindings.build(REFERENCE)
    ref = bindings.Reference()
    rng = np.random.default_rng(0x4DCD173B)
    meta = {}
    for name, args in CASES.items():
        data = make_case(ref, name, args, rng)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **data)
        meta[name] = {k: v for k, v in args.items()}
    kats = make_kats(ref, np.random.default_rng(0x8AC341EE))
    np.savez_compressed(os.path.join(HERE, "fpm_cdet_kats.npz"), **kats)
    np.savez_compressed(os.path.join(HERE, "vertex_samples.npz"), **make_vertex_samples(ref))
    np.savez_compressed(os.path.join(HERE, "precompute_3x3.npz"), **make_precompute(ref))
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    for fname in sorted(os.listdir(HERE)):
        print(fname, os.path.getsize(os.path.join(HERE, fname)))


if __name__ == "__main__":
    main()
