"""GPU CCH customization (bf_cch_*) against the oracle, bit for bit:
weights and middles of triangle_relax_parallel, the lexicographic
(time, length) relaxation with its middle election, and the bottom-up pass
(route/src/customization.rs:953-1436)."""
import numpy as np
import pytest

import cchgen
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _gpu(t, **kw):
    import bfphast
    return bfphast.Cch.from_oracle_topo(t, **kw)


def _eq(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x), np.asarray(y))


def test_reference_four_node(built, kats):
    k = kats["cch_customize"]
    tt = k["topo"]
    t = orc.CchTopo(tt["n"], tt["up_off"], tt["up_tgt"], tt["down_off"], tt["down_tgt"],
                    up_short=tt["up_short"], down_short=tt["down_short"], up_mid=tt["up_mid"],
                    down_mid=tt["down_mid"])
    g = _gpu(t)
    for case in k["bottom_up"]:
        up, dn = g.bottom_up(case["orig_up"], case["orig_down"], case["up_mid"], case["down_mid"])
        assert up.tolist() == case["up"] and dn.tolist() == case["down"]
    for case in k["lex"]:
        ut, dt, um, dm = g.relax_lex(case["up_t"], case["down_t"], case["up_l"], case["down_l"],
                                     t.up_mid, t.down_mid)
        assert ut[2] == case["time"] and um[2] == case["middle"]
        _eq((ut, dt, um, dm), t.relax_lex(case["up_t"], case["down_t"], case["up_l"],
                                         case["down_l"])[:4])


@pytest.mark.parametrize("rows,cols,seed,order,w_max", [
    (12, 14, 1, "nd", 60), (15, 15, 2, "nd", 6), (9, 10, 3, "random", 40),
    (20, 24, 4, "nd", 1000), (6, 40, 5, "nd", 3)])
@pytest.mark.parametrize("search", [False, True])
def test_directed_topologies(built, rows, cols, seed, order, w_max, search):
    t, ou, od = cchgen.grid_topology(rows, cols, seed, order=order, w_max=w_max, diagonals=0.2)
    g = _gpu(t, search_targets=search)
    assert g.info()["target_index"] == (0 if search else 1)
    # the union of a directed elimination need not be chordal (two
    # in-neighbours of a node are not joined), so either level kind occurs
    assert g.info()["levels"] > 1
    bu, bd = t.bottom_up(ou, od)
    _eq(g.bottom_up(ou, od), (bu, bd))
    want = t.relax(bu, bd)[:4]
    _eq(g.relax(bu, bd, t.up_mid, t.down_mid), want)
    _eq(g.customize(ou, od), want)
    # length channel: an independent seeded metric
    rng = np.random.default_rng(seed)
    lu = rng.integers(0, 50, len(ou)).astype(np.uint32)
    ld = rng.integers(0, 50, len(od)).astype(np.uint32)
    lbu, lbd = t.bottom_up(lu, ld)
    _eq(g.relax_lex(bu, bd, lbu, lbd, t.up_mid, t.down_mid),
        t.relax_lex(bu, bd, lbu, lbd)[:4])
    # bottom-up through the relaxed (time-optimal) middles
    _, _, um, dm = want
    _eq(g.bottom_up(lu, ld, um, dm), t.bottom_up(lu, ld, um, dm))


@pytest.mark.parametrize("search", [False, True])
def test_arbitrary_and_saturating_seeds(built, search):
    # the reference's fixed point from any seeds: below-optimal seeds,
    # u32::MAX seeds with middles, and legs whose sums saturate (a candidate
    # (u32::MAX, apex) can still lower the middle of a u32::MAX edge)
    t, ou, od = cchgen.grid_topology(11, 13, 9, w_max=30)
    g = _gpu(t, search_targets=search)
    rng = np.random.default_rng(9)
    for trial in range(4):
        su = rng.integers(0, 200, len(ou)).astype(np.uint32)
        sd = rng.integers(0, 200, len(od)).astype(np.uint32)
        if trial >= 2:
            su = np.where(rng.random(len(su)) < 0.5, INF - rng.integers(0, 100, len(su)),
                          su).astype(np.uint32)
            sd = np.where(rng.random(len(sd)) < 0.5, INF - rng.integers(0, 100, len(sd)),
                          sd).astype(np.uint32)
        mu = rng.integers(0, t.n, len(su)).astype(np.uint32)
        md = np.where(rng.random(len(sd)) < 0.3, INF, rng.integers(0, t.n, len(sd))).astype(
            np.uint32)
        _eq(g.relax(su, sd, mu, md), t.relax(su, sd, mu, md)[:4])
        lu = rng.integers(0, 1 << 32, len(su), dtype=np.uint64).astype(np.uint32)
        ld = rng.integers(0, 1 << 32, len(sd), dtype=np.uint64).astype(np.uint32)
        _eq(g.relax_lex(su, sd, lu, ld, mu, md), t.relax_lex(su, sd, lu, ld, mu, md)[:4])


def test_unclosed_topology_uses_longest_path_levels(built):
    # a topology not made by contraction: triangles whose target edge is
    # missing are skipped, and levels fall back to longest paths
    rng = np.random.default_rng(4)
    n = 300
    up = sorted({(u, v) for u, v in rng.integers(0, n, (1500, 2)) if u < v})
    dn = sorted({(u, v) for u, v in rng.integers(0, n, (1500, 2)) if u > v})

    def csr(lst):
        off = np.zeros(n + 1, np.uint64)
        off[1:] = np.cumsum(np.bincount([u for u, _ in lst], minlength=n))
        return off, np.array([v for _, v in lst], np.uint32)

    uo, ut = csr(up)
    do, dt = csr(dn)
    t = orc.CchTopo(n, uo, ut, do, dt)
    su = rng.integers(0, 1000, len(up)).astype(np.uint32)
    sd = rng.integers(0, 1000, len(dn)).astype(np.uint32)
    for search in (False, True):
        g = _gpu(t, with_short=False, search_targets=search)
        assert g.info()["etree_levels"] == 0
        _eq(g.relax(su, sd, t.up_mid, t.down_mid), t.relax(su, sd)[:4])


def test_bottom_up_middle_edge_cases(built):
    import bfphast
    t, ou, od = cchgen.grid_topology(8, 9, 6)
    g = _gpu(t)
    rng = np.random.default_rng(6)
    # middles at or above an endpoint read legs not computed yet: u32::MAX
    mu = np.where(t.up_short == 1, rng.integers(0, t.n, len(ou)), INF).astype(np.uint32)
    md = np.where(t.down_short == 1, rng.integers(0, t.n, len(od)), INF).astype(np.uint32)
    _eq(g.bottom_up(ou, od, mu, md), t.bottom_up(ou, od, mu, md))
    bad = mu.copy()
    bad[np.flatnonzero(t.up_short)[0]] = t.n
    with pytest.raises(bfphast.BfError) as ei:
        g.bottom_up(ou, od, bad, md)
    assert ei.value.status == bfphast.BF_ERR_INVALID
    with pytest.raises(IndexError):
        t.bottom_up(ou, od, bad, md)


def test_tiny_topologies(built):
    # one node; edges without any triangle
    t = orc.CchTopo(1, [0, 0], [], [0, 0], [])
    g = _gpu(t)
    assert all(len(x) == 0 for x in g.customize([], []))
    t = orc.CchTopo(3, [0, 1, 1, 1], [2], [0, 0, 0, 1], [1])
    g = _gpu(t)
    _eq(g.relax([5], [7], [INF], [INF]), t.relax([5], [7])[:4])


def test_fixture_graphs(built):
    # the fixture builder's own customization of its lattice and road CCHs
    import cchbuild
    for kind, r, c in ((cchbuild.KIND_GRID, 100, 100), (cchbuild.KIND_COUNTRY, 200, 250)):
        _, cch = cchbuild.build_synthetic(kind, r, c, seed=42, with_topo=True)
        u = cch["topo"]
        d, order = orc.CchTopo.from_upper(u)
        g = _gpu(d, with_short=False)
        uw, dw, um, dm = g.customize(u["orig_up"], u["orig_down"][order])
        assert np.array_equal(uw, u["cust_up"]) and np.array_equal(dw, u["cust_down"][order])
        if kind == cchbuild.KIND_GRID:
            _eq((uw, dw, um, dm), d.relax(u["orig_up"], u["orig_down"][order])[:4])


def _csr_weights(t, up_w, down_w):
    return dict(n=t.n, up_off=t.up_off, up_tgt=t.up_tgt, up_w=up_w, down_off=t.down_off,
                down_tgt=t.down_tgt, down_w=down_w)


@pytest.mark.parametrize("seed,order", [(21, "nd"), (22, "random")])
def test_customized_weights_answer_queries(built, seed, order):
    # customize on the GPU, build the PHAST engine on the result, and compare
    # the all-pairs matrix with plain Dijkstra on the original arcs
    import bfphast
    t, ou, od = cchgen.grid_topology(12, 13, seed, order=order, one_way=0.3)
    uw, dw, _, _ = _gpu(t).customize(ou, od)
    g = bfphast.Graph.from_cch(_csr_weights(t, uw, dw))
    allr = np.arange(t.n, dtype=np.uint32)
    got = g.matrix(allr, allr)
    want = np.stack([orc.dijkstra_ebg(t.arcs, s) for s in range(t.n)])
    assert np.array_equal(got, want)


def test_two_channel_chain(built):
    # time customization with the (time, length) middle election, then the
    # length along the elected middles, then the 2-channel engine: every stage
    # against the oracle's same chain, and the time channel against Dijkstra
    import bfphast
    t, ou, od = cchgen.grid_topology(11, 12, 31, w_max=4)  # many equal times
    rng = np.random.default_rng(31)
    # a physical length for every arc, also where the time is u32::MAX: a
    # triangle can give such an arc a finite time, and as an original edge it
    # keeps its own length
    lu = rng.integers(1, 90, len(ou)).astype(np.uint32)
    ld = rng.integers(1, 90, len(od)).astype(np.uint32)
    g = _gpu(t)
    bu, bd = g.bottom_up(ou, od)
    lbu, lbd = g.bottom_up(lu, ld)
    tu, td, mu, md = g.relax_lex(bu, bd, lbu, lbd, t.up_mid, t.down_mid)
    wtu, wtd, wmu, wmd, _ = t.relax_lex(*t.bottom_up(ou, od), *t.bottom_up(lu, ld))
    _eq((tu, td, mu, md), (wtu, wtd, wmu, wmd))
    latu, latd = g.bottom_up(lu, ld, mu, md)
    _eq((latu, latd), t.bottom_up(lu, ld, mu, md))
    # the engine takes length weights only where the time weight is finite
    latu = np.where(tu == INF, INF, latu).astype(np.uint32)
    latd = np.where(td == INF, INF, latd).astype(np.uint32)
    cch = _csr_weights(t, tu, td)
    g2 = bfphast.Graph.from_cch(cch, up_len=latu, down_len=latd)
    c = orc.Cch.from_dict(cch)
    for origin in (0, t.n // 3, t.n - 1):
        got = g2.phast_bounded_seeded_2ch([(origin, 0, 0)], INF)
        want = c.bounded_seeded_2ch([(origin, 0, 0)], INF, latu, latd)
        for a, b in zip(got, want):
            assert np.array_equal(a, b)
        dj = orc.dijkstra_ebg(t.arcs, origin)
        rk, tm = got[0], got[1]
        assert np.array_equal(tm, dj[rk])
