"""Two-channel (time, length along the time path) seeded PHAST on the GPU vs
the oracle's restatements of run_phast_bounded_fast_seeded_2ch
(route/src/server/isochrone_handler.rs:500-625) and table_phast_lopsided_2ch
(route/src/matrix/bucket_ch.rs:6381-6521). Bit-exact on both channels
(tolerance 0: u32 saturating arithmetic).

Time weights are coarsened to a few values so that equal-time ties, the
case the lexicographic tie-break exists for, occur everywhere."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _tie_weights(cch, seed, zero_frac=0.0):
    """(time, length) weights per CCH edge: times in {1, 2, 3} (some 0 when
    zero_frac > 0), lengths in [0, 5000); INF kept where the input is INF."""
    rng = np.random.default_rng(seed)
    out = []
    for key in ("up_w", "down_w"):
        w = np.asarray(cch[key], dtype=np.uint32)
        t = rng.integers(1, 4, len(w)).astype(np.uint32)
        if zero_frac:
            t[rng.random(len(w)) < zero_frac] = 0
        ln = rng.integers(0, 5000, len(w)).astype(np.uint32)
        inf = w == INF
        t[inf] = INF
        ln[inf] = INF
        out += [t, ln]
    return out  # up_t, up_l, dn_t, dn_l


def _pair(cch, seed, zero_frac=0.0, **kw):
    import bfphast
    up_t, up_l, dn_t, dn_l = _tie_weights(cch, seed, zero_frac)
    d = dict(cch, up_w=up_t, down_w=dn_t)
    g = bfphast.Graph(d["n"], d["up_off"], d["up_tgt"], up_t, d["down_off"], d["down_tgt"], dn_t,
                      up_len=up_l, down_len=dn_l, **kw)
    return g, orc.Cch.from_dict(d), up_l, dn_l, d


def test_kat_two_channel_tie(built, kats):
    # route/src/server/isochrone_handler.rs:1806-1869
    import bfphast
    for case in kats["two_channel_tie"]["cases"]:
        d = case["cch"]
        g = bfphast.Graph(d["n"], d["up_off"], d["up_tgt"], d["up_w"], d["down_off"],
                          d["down_tgt"], d["down_w"], up_len=case["up_len"],
                          down_len=case["down_len"])
        rk, tm, ln = g.phast_bounded_seeded_2ch([tuple(x) for x in case["seeds"]],
                                                case["threshold"])
        i = rk.tolist().index(case["node"])
        assert (tm[i], ln[i]) == (case["time"], case["len"])


@pytest.mark.parametrize("zero_frac", [0.0, 0.05])
def test_bounded_2ch_grid100_vs_oracle(built, grid100, zero_frac):
    _, cch = grid100
    g, c, up_l, dn_l, d = _pair(cch, 11, zero_frac)
    n = cch["n"]
    seedsets = [
        [(0, 0, 0)],
        [(777, 3, 40), (20000, 1, 9000), (777, 3, 10)],  # same rank, equal time: first kept
        [(5000, 9, 1), (5000, 4, 300), (5001, 0, 0)],    # same rank: smaller time kept
        [(n - 1, 0, 0), (12, 50, 50)],
        [(31000, 7, INF - 3)],                            # length saturates
    ]
    for seeds in seedsets:
        for thr in (0, 8, 25, 60, INF):
            want = c.bounded_seeded_2ch(seeds, thr, up_l, dn_l)
            got = g.phast_bounded_seeded_2ch(seeds, thr)
            for a, b in zip(got, want):
                assert np.array_equal(a, b)


def _seedsets(rng, n, m, max_seeds, cost_hi=8, len_hi=500, ranks=None):
    pool = ranks if ranks is not None else np.arange(n)
    sets = []
    for _ in range(m):
        k = int(rng.integers(1, max_seeds + 1))
        sets.append([(int(rng.choice(pool)), int(rng.integers(0, cost_hi)),
                      int(rng.integers(0, len_hi))) for _ in range(k)])
    return sets


@pytest.mark.parametrize("thr", [INF, 40])
def test_matrix_2ch_grid100_vs_oracle(built, grid100, thr):
    _, cch = grid100
    g, c, up_l, dn_l, _ = _pair(cch, 23)
    rng = np.random.default_rng(5)
    n = cch["n"]
    src = _seedsets(rng, n, 45, 3)
    tgt = _seedsets(rng, n, 60, 3)
    # shared ranks between a source and a target: conflicts
    tgt[3] = [src[0][0], (int(rng.integers(0, n)), 2, 7)]
    tgt[7] = [(src[9][0][0], 1, 1)]
    src[12] = []                      # an empty seed set: an INF row
    g.set_tune(lanes_per_wave=32)     # two waves
    ot, ol, conf = g.matrix_seeded_2ch(src, tgt, threshold=thr, with_conflicts=True)
    wt, wl, wconf = orc.table_phast_lopsided_2ch(c, src, tgt, thr, up_l, dn_l)
    assert np.array_equal(conf, wconf) and len(conf) >= 2
    assert np.array_equal(ot, wt)
    assert np.array_equal(ol, wl)
    assert (ot[12] == INF).all() and (ol[12] == INF).all()


def test_matrix_2ch_country_small_vs_oracle(built, country_small):
    _, cch = country_small
    g, c, up_l, dn_l, _ = _pair(cch, 31)
    rng = np.random.default_rng(9)
    src = _seedsets(rng, cch["n"], 20, 2)
    tgt = _seedsets(rng, cch["n"], 70, 2)
    ot, ol = g.matrix_seeded_2ch(src, tgt)
    wt, wl, _ = orc.table_phast_lopsided_2ch(c, src, tgt, INF, up_l, dn_l)
    assert np.array_equal(ot, wt) and np.array_equal(ol, wl)


def test_length_equal_to_time(built, grid100):
    # with length == time both channels agree, and the time channel is the
    # one-channel seeded matrix of the same graph
    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch, up_len=cch["up_w"], down_len=cch["down_w"])
    rng = np.random.default_rng(2)
    src = _seedsets(rng, cch["n"], 30, 2, cost_hi=200, len_hi=1)
    src = [[(r, t, t) for r, t, _ in ss] for ss in src]
    tgt = _seedsets(rng, cch["n"], 50, 2, cost_hi=200, len_hi=1)
    tgt = [[(r, t, t) for r, t, _ in ss] for ss in tgt]
    ot, ol = g.matrix_seeded_2ch(src, tgt, threshold=30000)
    one = g.matrix_seeded([[(r, t) for r, t, _ in ss] for ss in src],
                          [[(r, t) for r, t, _ in ss] for ss in tgt], threshold=30000)
    assert np.array_equal(ot, ol)
    assert np.array_equal(ot, one)


def _transpose(d, up_l, dn_l):
    """The CCH of the transposed graph (UP' = DOWN in-edges, DOWN' = UP in-edges)."""
    n = d["n"]

    def by_target(off, tgt, w, ln):
        off = np.asarray(off, dtype=np.int64)
        src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off))
        tgt = np.asarray(tgt, dtype=np.uint32)
        order = np.argsort(tgt, kind="stable")
        o = np.zeros(n + 1, dtype=np.uint64)
        o[1:] = np.cumsum(np.bincount(tgt, minlength=n))
        return o, src[order], np.asarray(w, np.uint32)[order], np.asarray(ln, np.uint32)[order]

    uo, ut, uw, ul = by_target(d["down_off"], d["down_tgt"], d["down_w"], dn_l)
    do, dt, dw, dl = by_target(d["up_off"], d["up_tgt"], d["up_w"], up_l)
    return dict(n=n, up_off=uo, up_tgt=ut, up_w=uw, down_off=do, down_tgt=dt, down_w=dw), ul, dl


def test_reverse_2ch_vs_oracle_on_transpose(built, grid100):
    _, cch = grid100
    g, _, up_l, dn_l, d = _pair(cch, 41, reverse=True)
    tr, tul, tdl = _transpose(d, up_l, dn_l)
    c = orc.Cch.from_dict(tr)
    for seeds in ([(99, 0, 0)], [(30001, 2, 5), (411, 0, 17)]):
        for thr in (20, INF):
            want = c.bounded_seeded_2ch(seeds, thr, tul, tdl)
            got = g.phast_bounded_seeded_2ch(seeds, thr)
            for a, b in zip(got, want):
                assert np.array_equal(a, b)


def test_two_channel_errors(built, grid100):
    import bfphast
    _, cch = grid100
    g1 = bfphast.Graph.from_cch(cch)
    with pytest.raises(bfphast.BfError) as e:
        g1.phast_bounded_seeded_2ch([(0, 0, 0)], 100)
    assert e.value.status == bfphast.BF_ERR_UNSUPPORTED
    bad = np.asarray(cch["up_w"], dtype=np.uint32).copy()
    fin = np.flatnonzero(bad != INF)
    up_l = bad.copy()
    up_l[fin[0]] = INF  # INF length on a finite-time edge
    with pytest.raises(bfphast.BfError) as e:
        bfphast.Graph.from_cch(cch, up_len=up_l, down_len=cch["down_w"])
    assert e.value.status == bfphast.BF_ERR_INVALID
    g2 = bfphast.Graph.from_cch(cch, up_len=cch["up_w"], down_len=cch["down_w"])
    with pytest.raises(bfphast.BfError) as e:
        g2.matrix_seeded_2ch([[(cch["n"], 0, 0)]], [[(1, 0, 0)]])
    assert e.value.status == bfphast.BF_ERR_INVALID
    # the graph stays usable
    rk, tm, ln = g2.phast_bounded_seeded_2ch([(5, 0, 0)], 0)
    assert rk.tolist() == [5] and tm.tolist() == [0] and ln.tolist() == [0]
