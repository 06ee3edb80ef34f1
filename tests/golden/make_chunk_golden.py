"""A chunked load-data directory written by the reference's own workflow, for
the chunk loader (cdet_load_chunks).

Run from the repository root with the environment variable REFERENCE set
to the reference checkout:

    REFERENCE=<reference checkout> python tests/golden/make_chunk_golden.py

Runs every stage of the reference's chunked load-data workflow (plan, node
samples, corners, sitepair transforms, diagonal reduce, validate;
chunked_load_data.h:1530-1570) for a 2x2 / degree-8 parameter set with four
distinct tables into chunks_2x2/ (without the node samples and diagonal
lines, which loading does not read), then loads it back with the reference's
load_chunked_data_into_resident_tables and records in chunks_2x2.json: the
sha256 of each loaded table array, the reference's diagonal observable on the
loaded tables, and the reference integrand on the golden 2x2 vertices.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import bindings  # noqa: E402
from make_golden import REFERENCE  # noqa: E402

ARGS = dict(n1=2, n2=2, beta="2.5", mu="0.3", u="1.7", alpha_up="0.55", alpha_down="0.4", pbc=True,
            mask_name="first_row", radius=0, nu=8, nv=8)
OUT = os.path.join(HERE, "chunks_2x2")


def main():
    bindings.build(REFERENCE)
    ref = bindings.Reference()
    ref.configure(**ARGS)
    work = tempfile.mkdtemp()
    ref.chunk_workflow(work, 16, 16)
    shutil.rmtree(OUT, ignore_errors=True)
    shutil.copytree(work, OUT, ignore=shutil.ignore_patterns("samples", "diagonal_lines", "*.tmp"))
    shutil.rmtree(work)
    ref.load_chunks(OUT)
    tables = ref.get_tables()
    digests = {f"{k}.{key}": hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
               for k, t in tables.items() for key, v in t.items()}
    diag = ref.diagonal_order1()
    gold = np.load(os.path.join(HERE, "physical_2x2.npz"))
    v, n = gold["single.vertices"], gold["single.orders"]
    values, fails = ref.integrand_batch(v, n, 1)
    meta = {"args": ARGS, "sha256": digests, "diagonal": [float(x).hex() for x in diag[:3]],
            "integrand": [float(x).hex() for x in values], "integrand_failures": int(fails)}
    with open(os.path.join(HERE, "chunks_2x2.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(sum(os.path.getsize(os.path.join(r, f)) for r, _, fs in os.walk(OUT) for f in fs), "bytes")


if __name__ == "__main__":
    main()
