"""The reference's chunked load-data directory format, on the host.

`read_chunks` assembles the four tables of a chunk directory in host memory
exactly as load_chunked_table_for_kind does (chunked_load_data.h:1372-1425);
`write_chunks` writes tables (for example from the GPU precompute) in the same
layout: manifest.txt (key=value, sorted), transform_jobs.tsv, corner_jobs.tsv,
node_jobs.tsv, coeffs/<kind>/<branch>/sitepairs_<begin>_<end>.bin (raw float64,
[sitepair][u][v]), corners/<kind>/<branch>.bin, diagonal_observable.txt
(optional) and READY, with the job numbering of the reference's planner
(run_chunked_plan_for_real, :755-882). The device loader is the library's
cdet_load_chunks (CdetIntegrand.load_chunks).
"""
from __future__ import annotations

import os
from typing import Dict, Optional

import numpy as np

KINDS = ("twisted_up", "twisted_down", "ordinary_up", "ordinary_down")
BRANCHES = ("upper", "lower")


def _token(begin: int, end: int) -> str:
    return f"{begin:010d}_{end:010d}"


def read_manifest(directory: str) -> Dict[str, str]:
    out = {}
    with open(os.path.join(directory, "manifest.txt")) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line or line.startswith("#") or "=" not in line:
                continue
            key, value = line.split("=", 1)
            out[key] = value
    return out


def read_transform_jobs(directory: str):
    jobs = []
    with open(os.path.join(directory, "transform_jobs.tsv")) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line or line.startswith("#"):
                continue
            tok = line.split("\t")
            jobs.append((int(tok[0]), tok[1], tok[2], int(tok[3]), int(tok[4])))
    return jobs


def read_chunks(directory: str) -> Dict[str, Dict[str, np.ndarray]]:
    m = read_manifest(directory)
    sitepairs, nodes = int(m["replica_sitepair_count"]), int(m["node_count"])
    tables = {k: {"upper": np.zeros(sitepairs * nodes), "lower": np.zeros(sitepairs * nodes),
                  "upper_corners": np.zeros(sitepairs), "lower_corners": np.zeros(sitepairs)} for k in KINDS}
    for _, kind, branch, begin, end in read_transform_jobs(directory):
        path = os.path.join(directory, "coeffs", kind, branch, f"sitepairs_{_token(begin, end)}.bin")
        data = np.fromfile(path, dtype="<f8")
        if data.size != (end - begin) * nodes:
            raise ValueError(f"Unexpected file size for {path}")
        tables[kind][branch][begin * nodes:end * nodes] = data
    for kind in KINDS:
        for branch in BRANCHES:
            path = os.path.join(directory, "corners", kind, f"{branch}.bin")
            data = np.fromfile(path, dtype="<f8")
            if data.size != sitepairs:
                raise ValueError(f"Unexpected file size for {path}")
            tables[kind][f"{branch}_corners"][:] = data
    return tables


def write_chunks(directory: str, manifest: Dict[str, str], tables: Dict[str, Dict], sitepair_chunk_size: int,
                 order1: Optional[tuple] = None) -> None:
    """Writes `tables` as a chunk directory. `manifest` holds the run's
    parameter strings (BETA, MU, ALPHA_UP, ALPHA_DOWN, PBC, SUBREGION_MASK,
    SUBREGION_SQUARE_RADIUS, N1, N2, CHEB_NU, CHEB_NV, node_chunk_size); the
    derived entries are filled in."""
    n1, n2 = int(manifest["N1"]), int(manifest["N2"])
    nu, nv = int(manifest["CHEB_NU"]), int(manifest["CHEB_NV"])
    sites = n1 * n2
    sitepairs, nodes = 4 * sites * sites, nu * nv
    m = dict(manifest)
    m.update({"layout_version": "1", "n_sites": str(sites), "replica_sitepair_count": str(sitepairs),
              "node_count": str(nodes), "sitepair_chunk_size": str(sitepair_chunk_size),
              "LOAD_DATA_REAL": "double", "VECTOR_REAL": "double"})
    m.setdefault("node_chunk_size", str(sitepair_chunk_size))
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "manifest.txt"), "w") as f:
        for key in sorted(m):
            f.write(f"{key}={m[key]}\n")
    node_chunk = int(m["node_chunk_size"])
    with open(os.path.join(directory, "node_jobs.tsv"), "w") as f:
        f.write("#index\ttable\tbranch\tnode_begin\tnode_end\n")
        index = 1
        for kind in KINDS:
            for branch in BRANCHES:
                for b in range(0, nodes, node_chunk):
                    f.write(f"{index}\t{kind}\t{branch}\t{b}\t{min(nodes, b + node_chunk)}\n")
                    index += 1
    with open(os.path.join(directory, "transform_jobs.tsv"), "w") as f:
        f.write("#index\ttable\tbranch\tsitepair_begin\tsitepair_end\n")
        index = 1
        for kind in KINDS:
            for branch in BRANCHES:
                arr = np.ascontiguousarray(tables[kind][branch], dtype="<f8")
                for b in range(0, sitepairs, sitepair_chunk_size):
                    e = min(sitepairs, b + sitepair_chunk_size)
                    f.write(f"{index}\t{kind}\t{branch}\t{b}\t{e}\n")
                    index += 1
                    d = os.path.join(directory, "coeffs", kind, branch)
                    os.makedirs(d, exist_ok=True)
                    arr[b * nodes:e * nodes].tofile(os.path.join(d, f"sitepairs_{_token(b, e)}.bin"))
    with open(os.path.join(directory, "corner_jobs.tsv"), "w") as f:
        f.write("#index\ttable\tbranch\n")
        index = 1
        for kind in KINDS:
            for branch in BRANCHES:
                f.write(f"{index}\t{kind}\t{branch}\n")
                index += 1
                d = os.path.join(directory, "corners", kind)
                os.makedirs(d, exist_ok=True)
                np.ascontiguousarray(tables[kind][f"{branch}_corners"], dtype="<f8").tofile(
                    os.path.join(d, f"{branch}.bin"))
    if order1 is not None:
        with open(os.path.join(directory, "diagonal_observable.txt"), "w") as f:
            # std::setprecision(max_digits10) of write_chunked_diagonal_observable_value (:1303-1318)
            f.write(f"layout_version=1\norder1_hi={float(order1[0]):.17g}\norder1_lo={float(order1[1]):.17g}\n")
    with open(os.path.join(directory, "READY"), "w") as f:
        f.write("ready\n")
