"""Wide slab rows: with 1024 lanes or more the batched matrix resets its
seeded, split and in-edge-free rows with bulk copies from shared memory
instead of per-thread stores. Two different source sets alternated on one
graph and one target set must each give the oracle's cells (tolerance 0:
u32 min-plus): a row the reset missed would still hold the other set's
distances, which are smaller in some lanes."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


@pytest.mark.parametrize("S", [1100, 1024 + 8200])
def test_wide_rows_alternating_sources(built, country_small, S):
    import bfphast
    _, cch = country_small
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    rng = np.random.default_rng(21)
    sets = [rng.choice(n, S, replace=True).astype(np.uint32) for _ in range(2)]
    tgt = rng.choice(n, 48, replace=False).astype(np.uint32)
    pick = np.linspace(0, S - 1, 10).astype(np.int64)
    want = [np.stack([c.phast_query(int(s))[tgt] for s in src[pick]]) for src in sets]
    for rep in range(2):
        for i, src in enumerate(sets):
            got = g.matrix(src, tgt)
            assert got.shape == (S, 48)
            assert np.array_equal(got[pick], want[i]), (S, rep, i)
            thr = 2000
            got = g.matrix(src, tgt, threshold=thr)
            assert np.array_equal(got[pick], np.where(want[i] <= thr, want[i], INF)), (S, rep, i)
