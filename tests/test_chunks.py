"""The chunked load-data format on the host (cdet_gb300/chunks.py) against a
directory written by the reference's own chunk workflow
(tests/golden/make_chunk_golden.py).

read_chunks must assemble exactly the tables the reference's
load_chunked_data_into_resident_tables loads (sha256 of every array), and
write_chunks, given those tables and the directory's manifest, must write the
same directory byte for byte (manifest, job lists, coefficient and corner
files, the diagonal value, READY; not the planner's informational
resource_plan.txt, which no loader reads).
"""
import filecmp
import hashlib
import json
import os

import numpy as np

from cdet_gb300.chunks import read_chunks, read_manifest, write_chunks
from helpers import GOLDEN

FIXTURE = os.path.join(GOLDEN, "chunks_2x2")
with open(os.path.join(GOLDEN, "chunks_2x2.json")) as f:
    META = json.load(f)


def test_reader_matches_reference_loader():
    tables = read_chunks(FIXTURE)
    for kind, t in tables.items():
        for key, arr in t.items():
            digest = hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()
            assert digest == META["sha256"][f"{kind}.{key}"], (kind, key)


def test_writer_reproduces_reference_directory(tmp_path):
    tables = read_chunks(FIXTURE)
    manifest = read_manifest(FIXTURE)
    with open(os.path.join(FIXTURE, "diagonal_observable.txt")) as f:
        kv = dict(line.strip().split("=", 1) for line in f if "=" in line)
    out = str(tmp_path / "chunks")
    write_chunks(out, manifest, tables, int(manifest["sitepair_chunk_size"]),
                 order1=(float(kv["order1_hi"]), float(kv["order1_lo"])))
    written = sorted(os.path.relpath(os.path.join(r, f), out) for r, _, fs in os.walk(out) for f in fs)
    expected = sorted(os.path.relpath(os.path.join(r, f), FIXTURE) for r, _, fs in os.walk(FIXTURE) for f in fs
                      if f != "resource_plan.txt")
    assert written == expected
    for rel in expected:
        assert filecmp.cmp(os.path.join(out, rel), os.path.join(FIXTURE, rel), shallow=False), rel
