"""Pins the CPU oracle to the reference's own known-answer tests.

Each case cites the reference test it restates (paths relative to the
butterfly-osm repository). The oracle must reproduce every vector before it
is trusted as the GPU engine's checker.
"""
import numpy as np
import pytest

from oracle import oracle as orc

INF = 0xFFFFFFFF


def _cch(d):
    return orc.Cch(d["n"], d["up_off"], d["up_tgt"], d["up_w"], d["down_off"], d["down_tgt"],
                   d["down_w"])


def test_five_node_forward(built, kats):
    # route/src/range/phast.rs:1307-1312 (fwd_result from 0 == [0,13,10,17,15])
    k = kats["five_node"]
    c = _cch(k["cch"])
    for s, want in k["fwd"].items():
        assert c.phast_query(int(s)).tolist() == want


def test_five_node_reverse_and_cross_identity(built, kats):
    # phast.rs:1375-1389 and test_reverse_phast_vs_forward :1392-1417
    k = kats["five_node"]
    c = _cch(k["cch"])
    ro, rs, rw = orc.down_reverse(c)
    assert c.reverse(0, ro, rs, rw).tolist() == k["rev"]["0"]
    for s in range(5):
        fwd = c.phast_query(s)
        for t in range(5):
            assert fwd[t] == c.reverse(t, ro, rs, rw)[s]


def test_five_node_bounded_reverse_count(built, kats):
    # phast.rs:1420-1445: reverse to 0 within threshold 12 reaches 2 nodes
    k = kats["five_node"]
    c = _cch(k["cch"])
    ro, rs, rw = orc.down_reverse(c)
    rev = c.reverse(0, ro, rs, rw)
    b = k["rev_bounded_count"]
    assert int((rev <= b["threshold"]).sum()) == b["count"]


def test_asymmetric_three_node(built, kats):
    # phast.rs:1508-1560: d_fwd(0) = [0,13,10], d_fwd(1) = [25,0,5], d_rev(0) = [0,25,20]
    k = kats["asym_three_node"]
    c = _cch(k["cch"])
    for s, want in k["fwd"].items():
        assert c.phast_query(int(s)).tolist() == want
    ro, rs, rw = orc.down_reverse(c)
    assert c.reverse(0, ro, rs, rw).tolist() == k["rev"]["0"]
    assert c.phast_query(0)[1] != c.reverse(0, ro, rs, rw)[1]  # asymmetry


def test_inf_edges_are_dropped(built, kats):
    # bucket_ch.rs:4907-4960: 3 finite UP / 3 finite DOWN edges; INF never relaxes
    k = kats["inf_four_node"]
    d = k["cch"]
    assert sum(w != INF for w in d["up_w"]) == k["finite_up"]
    assert sum(w != INF for w in d["down_w"]) == k["finite_down"]
    c = _cch(d)
    # 0 ->2 (10) ->3 (7); 3 ->2 (7) ->1 (3)
    assert c.phast_query(0).tolist() == [0, 13, 10, 17]
    assert c.phast_query(3).tolist() == [17, 10, 7, 0]


@pytest.mark.parametrize("n_leaf", ["5", "12"])
def test_broom_closed_form_and_bounds(built, kats, n_leaf):
    # bucket_ch.rs:5661-5760: d(s,t) = wu[s] + wd[t], bounded == unbounded in-bound
    b = kats["broom"][n_leaf]
    c = _cch(b["cch"])
    n = int(n_leaf)
    m, _ = c.matrix(np.arange(n), np.arange(n))
    assert m.tolist() == b["expect"]
    for thr in b["thresholds"]:
        for s in range(n):
            ranks, dists = c.bounded_seeded([(s, 0)], thr)
            got = dict(zip(ranks.tolist(), dists.tolist()))
            for t in range(n):
                e = b["expect"][s][t]
                if e <= thr:
                    assert got.get(t) == e
                else:
                    assert t not in got


@pytest.mark.parametrize("graph", ["grid100", "country_small"])
def test_batched_equals_single(built, request, graph):
    # bench/main.rs:1393-1414: every batched cell equals the single-source query
    _, cch = request.getfixturevalue(graph)
    c = orc.Cch.from_dict(cch)
    rng = np.random.default_rng(1)
    src = rng.integers(0, c.n, 8)
    batch = c.query_batch(src)
    for lane, s in enumerate(src):
        assert np.array_equal(batch[lane], c.phast_query(s))
    m, _ = c.matrix(src, np.arange(c.n))
    assert np.array_equal(m, batch)
    # the threaded matrix over more sources than one K-lane batch
    src2 = rng.integers(0, c.n, 21)
    tgt = rng.integers(0, c.n, 40)
    m2, _ = c.matrix(src2, tgt, threads=4)
    assert np.array_equal(m2, np.stack([c.phast_query(s)[tgt] for s in src2]))


def test_bounded_agrees_with_unbounded(built, grid100):
    # bench/main.rs:2640-2660: reachability within T agrees between the
    # bounded K-lane sweep and the plain one; values <= T are exact
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    src = np.array([5, 500, 5000, 20000, 30000, 35000, 1, 17], dtype=np.uint32)
    full = c.query_batch(src)
    for thr in (0, 300, 3000, 30000):
        bnd = c.query_batch_bounded(src, thr)
        assert np.array_equal(full <= thr, bnd <= thr)
        assert np.array_equal(np.where(full <= thr, full, 0), np.where(bnd <= thr, bnd, 0))
        for lane, s in enumerate(src):
            rk, ds = c.bounded_seeded([(int(s), 0)], thr)
            want = np.flatnonzero(full[lane] <= thr)
            assert np.array_equal(rk, want)
            assert np.array_equal(ds, full[lane][want])


def test_seeded_multi_source(built, grid100):
    # isochrone_handler.rs:338-373: seeds behave as a super-source with
    # non-negative arcs: field = min over seeds of cost + dist(seed, .)
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    seeds = [(100, 7), (2000, 0), (31000, 55)]
    thr = 2500
    rk, ds = c.bounded_seeded(seeds, thr)
    want = np.full(c.n, INF, dtype=np.uint64)
    for r, cost in seeds:
        d = c.phast_query(r).astype(np.uint64)
        want = np.minimum(want, np.where(d == INF, INF, d + cost))
    sel = np.flatnonzero(want <= thr)
    assert np.array_equal(rk, sel)
    assert np.array_equal(ds, want[sel])


def test_grid100_golden_matches_oracle(built, grid100):
    import pathlib
    g = np.load(pathlib.Path(__file__).parent / "golden" / "grid100_matrix.npz")
    _, cch = grid100
    m, _ = orc.Cch.from_dict(cch).matrix(g["sources"], g["targets"], threads=2)
    assert np.array_equal(m, g["matrix"])


def test_two_channel_lexicographic_tie(built, kats):
    # route/src/server/isochrone_handler.rs:1806-1869 (phast_2ch_lex_tests):
    # node 3 has two time-10 paths; the shorter length (2) wins in both pop orders
    for case in kats["two_channel_tie"]["cases"]:
        c = _cch(case["cch"])
        rk, tm, ln = c.bounded_seeded_2ch([tuple(x) for x in case["seeds"]], case["threshold"],
                                          case["up_len"], case["down_len"])
        i = rk.tolist().index(case["node"])
        assert (tm[i], ln[i]) == (case["time"], case["len"])


def test_two_channel_time_matches_one_channel(built, grid100):
    # the time channel of the 2-channel field is the 1-channel field
    # (isochrone_handler.rs:500-506: "Mirrors run_phast_bounded_fast_seeded
    # exactly on the time side"); with length == time both channels agree
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    seeds = [(17, 0, 0), (4000, 35, 35), (4000, 20, 20)]
    for thr in (900, 5000, INF):
        rk1, d1 = c.bounded_seeded([(r, t) for r, t, _ in seeds], thr)
        rk2, tm, ln = c.bounded_seeded_2ch(seeds, thr, cch["up_w"], cch["down_w"])
        assert np.array_equal(rk1, rk2) and np.array_equal(d1, tm)
        assert np.array_equal(tm, ln)
