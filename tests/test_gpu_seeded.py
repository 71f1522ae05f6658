"""Phantom-seeded queries on the GPU vs the CPU oracle (bit-exact)."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _graph(d):
    import bfphast
    return bfphast.Graph(d["n"], d["up_off"], d["up_tgt"], d["up_w"], d["down_off"],
                         d["down_tgt"], d["down_w"])


def test_bounded_seeded_matches_oracle(built, grid100, country_small):
    for (_, cch), cases in ((grid100, [([(100, 7), (2000, 0), (31000, 55)], 2500),
                                       ([(5, 0)], 0), ([(5, 0)], INF),
                                       ([(12345, 3), (12346, 9)], 900)]),
                            (country_small, [([(17, 0), (40000, 12)], 6000),
                                             ([(99999, 0)], 1200)])):
        c = orc.Cch.from_dict(cch)
        g = _graph(cch)
        for seeds, thr in cases:
            rk, ds = g.phast_bounded_seeded(seeds, thr)
            wr, wd = c.bounded_seeded(seeds, thr)
            assert np.array_equal(rk, wr) and np.array_equal(ds, wd)


def test_bounded_seeded_empty(built, grid100):
    _, cch = grid100
    g = _graph(cch)
    rk, ds = g.phast_bounded_seeded([], 1000)
    assert len(rk) == 0 and len(ds) == 0


def test_matrix_seeded_matches_lopsided(built, grid100):
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    rng = np.random.default_rng(11)
    n = cch["n"]
    src = [[(int(r), int(rng.integers(0, 40))) for r in rng.integers(0, n, rng.integers(1, 4))]
           for _ in range(37)]
    tgt = [[(int(r), int(rng.integers(0, 40))) for r in rng.integers(0, n, rng.integers(1, 3))]
           for _ in range(45)]
    tgt[3] = [src[5][0]]  # a shared seed rank: a same-edge conflict
    tgt[4] = []           # a target without seeds
    for thr in (INF, 3000, 200):
        got, conf = g.matrix_seeded(src, tgt, thr, with_conflicts=True)
        want, wconf = orc.table_phast_lopsided(c, src, tgt, thr)
        assert np.array_equal(conf, wconf)
        assert 5 * 45 + 3 in conf.tolist()
        assert np.array_equal(got, want)


def test_matrix_seeded_broom(built, kats):
    # bucket_ch.rs:5766-5795 seeded_bounded_equals_unbounded_filtered: every
    # in-bound off-diagonal cell of the bounded run equals the unbounded one
    b = kats["broom"]["12"]
    g = _graph(b["cch"])
    n = 12
    src = [[(i, 0)] for i in range(n)]
    tgt = [[(j, 50 if j % 4 == 3 else 0)] for j in range(n)]
    unb, conf = g.matrix_seeded(src, tgt, INF, with_conflicts=True)
    assert conf.tolist() == [i * n + i for i in range(n)]  # same-rank diagonal
    for thr in (0, 20, 55, 120, 100000):
        bnd = g.matrix_seeded(src, tgt, thr)
        assert np.array_equal(bnd, np.where(unb <= thr, unb, INF))
