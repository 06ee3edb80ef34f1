"""Index bounds of the split path's global and shared-memory accesses, on the CPU.

The index arithmetic of cdet_split.cu, restated for every table shape the
tests run (the 2x2 golden case's degree 18, where rows and K columns are
padded, and the sub-block shapes up to degree 256): each slice, lead and
level-row address slice_blocks writes lies inside the buffer the host sizes
for it (split_slices_bytes, split_leads_bytes, split_level_rows_bytes); every
pass geometry pass_geom can produce keeps the copy warp's bulk copies inside
one K step of the table and inside its ring stage, the MMA's operand rows
inside the copied rows, and the accumulator columns below the sink; the tile
list fits the capacity the scratch carve gives it; the descriptor kernel's
warps take every (configuration, vertex pair) once and shuffle only from
lanes holding that configuration's vertices.
"""
import itertools

import numpy as np
import pytest

ROWS, SUBK, KSTEP, SLICES, LEVELS = 128, 128, 16, 8, 7
SUBKSTEPS = SUBK // KSTEP
STAGE_HALVES = SLICES * ROWS * KSTEP  # kAStageBytes / 2
SINK = 496
TILE_N = 128

SHAPES = [(18, 18), (16, 16), (64, 64), (128, 128), (136, 200), (200, 100), (96, 160), (144, 144),
          (160, 160), (192, 192), (256, 256), (1, 1), (129, 17)]


def geometry(nu, nv):
    """split_geometry."""
    nrb = (nu + ROWS - 1) // ROWS
    nkc = (nv + SUBK - 1) // SUBK
    ksteps_last = (nv - (nkc - 1) * SUBK + KSTEP - 1) // KSTEP
    return nrb, nkc, ksteps_last


def row_ksteps(nkc, ksteps_last):
    return (nkc - 1) * SUBKSTEPS + ksteps_last


def core_offset(row, k):
    return (row >> 3) * 128 + (k >> 3) * 64 + (row & 7) * 8 + (k & 7)


def pass_geom(rows, p):
    """pass_geom: (npass, row0, cols, n[], col[])."""
    total = sum((r + 15) & ~15 for r in rows)
    npass = 1 if total <= SINK else 2
    row0 = 0 if npass == 1 else 64 * p
    span = ROWS if npass == 1 else 64
    n, col, c = [], [], 0
    for r in rows:
        n.append((min(max(r - row0, 0), span) + 15) & ~15)
        col.append(c)
        c += n[-1]
    return npass, row0, max(n), n, col


@pytest.mark.parametrize("nu,nv", SHAPES)
def test_slice_table_writes_in_bounds(nu, nv):
    blocks = 3
    nrb, nkc, ksl = geometry(nu, nv)
    rk = row_ksteps(nkc, ksl)
    slice_halves = blocks * nrb * rk * STAGE_HALVES
    lead_bytes = blocks * nrb * rk
    level_rows = blocks * nrb * nkc
    assert 1 <= ksl <= SUBKSTEPS
    for block, rb, kc in itertools.product(range(blocks), range(nrb), range(nkc)):
        ksteps = ksl if kc == nkc - 1 else SUBKSTEPS
        dst = ((block * nrb + rb) * rk + kc * SUBKSTEPS) * STAGE_HALVES
        # the thread loop's largest (a, b): a = 127, b = ksteps * 16 - 1
        a, b = ROWS - 1, ksteps * KSTEP - 1
        ks, bb = b // KSTEP, b % KSTEP
        k = (bb & 1) * 8 + (bb >> 1)
        assert 0 <= k < KSTEP
        last = dst + ks * SLICES * ROWS * KSTEP + core_offset(a, k) + (SLICES - 1) * ROWS * KSTEP
        assert last < slice_halves
        # every (row, k) of a K step lands on a distinct element of its slice
        assert sorted(core_offset(r, kk) for r in range(ROWS) for kk in range(KSTEP)) == list(range(ROWS * KSTEP))
        assert (block * nrb + rb) * rk + kc * SUBKSTEPS + ksteps - 1 < lead_bytes
        assert block * nrb * nkc + rb * nkc + kc < level_rows
        # coefficient reads are guarded (ag < nu, bg < nv); the guard drops
        # exactly the padding of this sub-block
        rows_real = min(nu - rb * ROWS, ROWS)
        cols_real = min(nv - kc * SUBK, ksteps * KSTEP)
        assert rows_real > 0 and cols_real > 0


def _level_row_vectors(rng):
    """Level-row vectors slice_blocks can record: nondecreasing in the level
    (a digit reaching tau reaches every later level), each <= 128."""
    yield [0] * LEVELS
    yield [128] * LEVELS
    yield [1] * LEVELS
    yield [0, 0, 0, 0, 0, 0, 18]
    yield [18] * LEVELS
    for _ in range(3000):
        v = np.sort(rng.integers(0, 129, LEVELS))
        yield [int(x) for x in v]


def test_pass_geometry_copies_and_columns_in_bounds():
    rng = np.random.default_rng(5)
    for rows in _level_row_vectors(rng):
        npass = pass_geom(rows, 0)[0]
        for p in range(npass):
            _, row0, cols, n, col = pass_geom(rows, p)
            copied = max(cols, 16)  # the copy warp's row count
            assert row0 + copied <= ROWS, (rows, p)
            for lead in range(1, SLICES + 1):
                if row0 == 0 and copied == ROWS:
                    offset = (lead - 1) * ROWS * KSTEP
                    assert offset + (STAGE_HALVES - offset) <= STAGE_HALVES
                else:
                    for t in range(lead, SLICES + 1):
                        offset = (t - 1) * ROWS * KSTEP + row0 * KSTEP
                        assert offset + copied * KSTEP <= STAGE_HALVES
                        assert offset % 8 == 0 and (copied * KSTEP * 2) % 16 == 0  # bulk-copy 16-byte rule
            for lv in range(LEVELS):
                assert n[lv] <= copied  # the MMA's rows were copied
                assert col[lv] + n[lv] <= SINK, (rows, p)


@pytest.mark.parametrize("seed", range(20))
def test_tile_list_capacity(seed):
    rng = np.random.default_rng(seed)
    nblocks = int(rng.integers(1, 300))
    nrec = int(rng.integers(0, 20000))
    counts = np.bincount(rng.integers(0, nblocks, nrec), minlength=nblocks) if nrec else np.zeros(nblocks, int)
    tiles = int(sum((c + TILE_N - 1) // TILE_N for c in counts))
    assert tiles <= nrec // TILE_N + nblocks + 1


def descriptor_configs_per_warp(nmax):
    """descriptor_configs_per_warp: whole configurations' vertices per 32 lanes."""
    return 32 // nmax if 1 <= nmax <= 32 else 1


@pytest.mark.parametrize("nmax", range(1, 25))
def test_descriptor_warp_mapping(nmax):
    """split_descriptors: one warp per K configurations, each vertex on a lane,
    the pairs 32 at a time. Every (configuration, pair) of the batch is taken
    exactly once, and both vertices of a pair are read from lanes holding that
    configuration's vertices (lane < K nmax <= 32)."""
    K = descriptor_configs_per_warp(nmax)
    per_c = nmax * nmax
    for batch in (1, 2, K, K + 1, 3 * K + 2, 97):
        warps = (batch + K - 1) // K
        seen = set()
        for warp in range(warps):
            c0 = warp * K
            assert c0 < batch
            total = K * per_c
            for q0 in range(0, total, 32):
                for lane in range(32):
                    q = q0 + lane
                    valid = q < total
                    cq = q // per_c if valid else 0
                    pair = q - cq * per_c if valid else 0
                    i, j = divmod(pair, nmax)
                    li, lj = cq * nmax + i, cq * nmax + j
                    assert li < 32 and lj < 32 and li // nmax == cq and lj // nmax == cq
                    if valid and c0 + cq < batch:
                        assert (c0 + cq, pair) not in seen
                        seen.add((c0 + cq, pair))
        assert len(seen) == batch * per_c
