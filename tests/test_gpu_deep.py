"""Deep elimination trees: a chain CCH whose ancestor path (depth n - 1) is
longer than the upward pass keeps in shared memory, so the upward pass runs
with per-warp global scratch. Every entry point against the CPU oracle
(bit-exact)."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _chain(n):
    """Ranks 0..n-1 in a line: UP edge i -> i+1, DOWN edge i+1 -> i."""
    up_off = np.minimum(np.arange(n + 1), n - 1).astype(np.uint64)
    up_tgt = np.arange(1, n, dtype=np.uint32)
    up_w = (1 + np.arange(n - 1) % 7).astype(np.uint32)
    down_off = np.concatenate([[0], np.arange(n)]).astype(np.uint64)
    down_tgt = np.arange(0, n - 1, dtype=np.uint32)
    down_w = (2 + np.arange(n - 1) % 5).astype(np.uint32)
    return dict(n=n, up_off=up_off, up_tgt=up_tgt, up_w=up_w, down_off=down_off,
                down_tgt=down_tgt, down_w=down_w)


N = 7000  # ancestor path of rank 0: 7000 entries, past the shared-memory capacity


def test_deep_chain_matrix_both_engines(built):
    import bfphast
    cch = _chain(N)
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    assert g.info()["max_depth"] == N - 1
    src = np.array([0, 1, 17, 3333, N - 2, N - 1, 0], dtype=np.uint32)
    tgt = np.array([N - 1, 0, 5, 4000, 6999, 12], dtype=np.uint32)
    want, _ = c.matrix(src, tgt)
    for eng in (bfphast.ENGINE_BATCHED, bfphast.ENGINE_PLAIN):
        g.set_engine(eng)
        assert np.array_equal(g.matrix(src, tgt), want)
        assert np.array_equal(g.matrix(src, tgt, threshold=5000),
                              np.where(want <= 5000, want, INF))
    assert np.array_equal(g.phast_query(0), c.phast_query(0))


def test_deep_chain_two_channel_global_path(built):
    import bfphast
    cch = _chain(5000)  # 1-channel path fits shared memory, the 2-channel one does not
    c = orc.Cch.from_dict(cch)
    up_l = (cch["up_w"] * 3).astype(np.uint32)
    dn_l = (cch["down_w"] * 5).astype(np.uint32)
    g = bfphast.Graph.from_cch(cch, up_len=up_l, down_len=dn_l)
    for seeds, thr in (([(0, 0, 0)], 4000), ([(2500, 3, 7), (10, 0, 1)], INF)):
        got = g.phast_bounded_seeded_2ch(seeds, thr)
        want = c.bounded_seeded_2ch(seeds, thr, up_l, dn_l)
        for a, b in zip(got, want):
            assert np.array_equal(a, b)


def test_deep_chain_threshold_calls(built):
    # per-lane thresholds and seeded units also run on the global-scratch pass
    import bfphast
    cch = _chain(N)
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    origins = np.array([0, 10, 3500, N - 1], dtype=np.uint32)
    thr = np.array([100, 2000, 9000, 50], dtype=np.uint32)
    bits, counts = g.isochrone_bitsets(origins, thr)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr)
    assert np.array_equal(bits, want_bits) and np.array_equal(counts, want_counts)
    for seeds, t in (([(0, 0)], 100), ([(10, 5), (6000, 0)], 4000)):
        rk, ds = g.phast_bounded_seeded(seeds, t)
        wr, wd = c.bounded_seeded(seeds, t)
        assert np.array_equal(rk, wr) and np.array_equal(ds, wd)
    src = [[(0, 0)], [(100, 3), (200, 1)]]
    tgt = [[(N - 1, 0)], [(50, 2)], [(3000, 0), (3001, 4)]]
    assert np.array_equal(g.matrix_seeded(src, tgt), orc.table_phast_lopsided(c, src, tgt, INF)[0])


def _zigzag(n):
    """Two chains of ranks of one parity (0, 2, 4, ... and 1, 3, 5, ...) that
    meet at the top (n - 2 -> n - 1, n even): every rank's parent is two
    ranks up, so an ancestor path is a run of single ranks, about n / 2 runs."""
    up = {u: [] for u in range(n)}
    for u in range(n - 2):
        up[u].append(u + 2)
    up[n - 2].append(n - 1)
    up_off = np.zeros(n + 1, np.uint64)
    up_off[1:] = np.cumsum([len(up[u]) for u in range(n)])
    up_tgt = np.array([v for u in range(n) for v in up[u]], np.uint32)
    up_w = (3 + np.arange(len(up_tgt)) % 11).astype(np.uint32)
    down = {v: [] for v in range(n)}
    for u in range(n):
        for v in up[u]:
            down[v].append(u)
    down_off = np.zeros(n + 1, np.uint64)
    down_off[1:] = np.cumsum([len(down[v]) for v in range(n)])
    down_tgt = np.array([u for v in range(n) for u in down[v]], np.uint32)
    down_w = (1 + np.arange(len(down_tgt)) % 5).astype(np.uint32)
    return dict(n=n, up_off=up_off, up_tgt=up_tgt, up_w=up_w, down_off=down_off,
                down_tgt=down_tgt, down_w=down_w)


@pytest.mark.parametrize("n", [60, 400])
def test_path_runs_both_upward_forms(built, n):
    """Ancestor paths of at most 32 runs take the run-indexed upward kernel,
    longer ones the path-array kernel: n = 60 gives paths of ~30 runs, n = 400
    of ~200. Both against the oracle, for the matrix engines, per-lane
    thresholds and seeded units."""
    import bfphast
    cch = _zigzag(n)
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    rng = np.random.default_rng(n)
    src = rng.choice(n, 20, replace=False).astype(np.uint32)
    tgt = rng.choice(n, 25, replace=False).astype(np.uint32)
    want, _ = c.matrix(src, tgt)
    for eng in (bfphast.ENGINE_BATCHED, bfphast.ENGINE_PLAIN):
        g.set_engine(eng)
        assert np.array_equal(g.matrix(src, tgt), want), eng
        assert np.array_equal(g.matrix(src, tgt, threshold=150),
                              np.where(want <= 150, want, INF)), eng
    origins = src[:6]
    thr = np.array([10, 40, 90, 200, 500, 3000], dtype=np.uint32)
    bits, counts = g.isochrone_bitsets(origins, thr)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr)
    assert np.array_equal(bits, want_bits) and np.array_equal(counts, want_counts)
    seeds = [(int(src[0]), 3), (int(src[1]), 0)]
    rk, ds = g.phast_bounded_seeded(seeds, 300)
    wr, wd = c.bounded_seeded(seeds, 300)
    assert np.array_equal(rk, wr) and np.array_equal(ds, wd)
