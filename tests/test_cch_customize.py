"""CCH customization oracle (route/src/customization.rs:953-1436), pinned by
the reference's own unit tests and checked against the properties the GPU
kernels rely on. CPU only."""
import numpy as np
import pytest

import cchgen
from oracle import oracle as orc

INF = 0xFFFFFFFF


def _four(k):
    t = k["topo"]
    return orc.CchTopo(t["n"], t["up_off"], t["up_tgt"], t["down_off"], t["down_tgt"],
                       up_short=t["up_short"], down_short=t["down_short"], up_mid=t["up_mid"],
                       down_mid=t["down_mid"])


def test_bottom_up_follows_external_middle(built, kats):
    # customization.rs:2302-2350: shortcut 2 -> 3 through apex 0 is 3 + 10,
    # through apex 1 is 5 + 100; original edges do not depend on the middle
    k = kats["cch_customize"]
    t = _four(k)
    for case in k["bottom_up"]:
        up, dn = t.bottom_up(case["orig_up"], case["orig_down"], up_mid=case["up_mid"],
                             down_mid=case["down_mid"])
        assert up.tolist() == case["up"] and dn.tolist() == case["down"]


def test_packed_order(kats):
    # customization.rs:2352-2371: weight in the high word, middle breaks ties
    for (w0, m0), (w1, m1) in kats["cch_customize"]["pack_order"]:
        assert (w0 << 32 | m0) < (w1 << 32 | m1)


def test_lexicographic_middle_election(built, kats):
    # customization.rs:2420-2487: equal times elect the shorter length, then
    # the smallest apex
    k = kats["cch_customize"]
    t = _four(k)
    for case in k["lex"]:
        ut, dt, um, dm, _ = t.relax_lex(case["up_t"], case["down_t"], case["up_l"], case["down_l"])
        assert ut[2] == case["time"] and um[2] == case["middle"]
        assert dt.tolist() == case["down_t"]


def test_relax_matches_builder_customization(built):
    # the fixture builder customizes its CCH with its own triangle pass; the
    # oracle's relaxation of the same topology gives the same weights
    import cchbuild
    _, cch = cchbuild.build_synthetic(cchbuild.KIND_COUNTRY, 60, 80, seed=3, with_topo=True)
    u = cch["topo"]
    d, order = orc.CchTopo.from_upper(u)
    uw, dw, _, _, passes = d.relax(u["orig_up"], u["orig_down"][order])
    assert np.array_equal(uw, u["cust_up"]) and np.array_equal(dw, u["cust_down"][order])
    assert passes >= 2


@pytest.mark.parametrize("seed,order", [(1, "nd"), (2, "nd"), (3, "random")])
def test_shortcut_seeds_do_not_matter(built, seed, order):
    # bottom_up_customize seeds + relax == u32::MAX shortcut seeds + relax
    # (the bottom-up value is dominated by the triangle through its middle)
    t, ou, od = cchgen.grid_topology(9, 11, seed, order=order)
    bu, bd = t.bottom_up(ou, od)
    a = t.relax(bu, bd)
    su = np.where(t.up_short == 1, INF, ou).astype(np.uint32)
    sd = np.where(t.down_short == 1, INF, od).astype(np.uint32)
    b = t.relax(su, sd)
    for x, y in zip(a[:4], b[:4]):
        assert np.array_equal(x, y)
    assert (a[0] != INF).sum() > 0


def test_relax_is_idempotent_and_lex_time_equals_relax(built):
    t, ou, od = cchgen.grid_topology(10, 10, 5, w_max=8)  # small weights: many ties
    uw, dw, um, dm, _ = t.relax(ou, od)
    uw2, dw2, um2, dm2, passes = t.relax(uw, dw, um, dm)
    assert passes == 1
    assert np.array_equal(uw, uw2) and np.array_equal(dw, dw2)
    assert np.array_equal(um, um2) and np.array_equal(dm, dm2)
    bu, bd = t.bottom_up(ou, od)
    lt, ld, _, _, _ = t.relax_lex(bu, bd, bu, bd)
    assert np.array_equal(lt, uw) and np.array_equal(ld, dw)


def test_directed_topology_is_closed(built):
    # every triangle's target edge exists (the contraction's closure), the
    # property under which absent edges never receive a candidate
    t, _, _ = cchgen.grid_topology(8, 8, 11, one_way=0.5)
    up = {(u, int(v)) for u in range(t.n) for v in t.up_tgt[t.up_off[u]:t.up_off[u + 1]]}
    dn = {(u, int(v)) for u in range(t.n) for v in t.down_tgt[t.down_off[u]:t.down_off[u + 1]]}
    for m in range(t.n):
        xs = [x for (x, v) in dn if v == m]
        ys = [int(y) for y in t.up_tgt[t.up_off[m]:t.up_off[m + 1]]]
        for x in xs:
            for y in ys:
                if x != y:
                    assert ((x, y) in up) if y > x else ((x, y) in dn)


def test_parallel_relaxation_matches_sequential(built):
    # the apex-parallel atomic form (the reference's own) reaches the same
    # fixed point, middles included
    for seed in (1, 2):
        t, ou, od = cchgen.grid_topology(14, 14, seed, w_max=5)
        bu, bd = t.bottom_up(ou, od)
        a = t.relax(bu, bd)
        b = t.relax(bu, bd, threads=4)
        for x, y in zip(a[:4], b[:4]):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("seed,order", [(21, "nd"), (23, "random")])
def test_customized_cch_answers_exact_distances(built, seed, order):
    # after customization the CCH's PHAST matrix is the shortest-path matrix
    # of the original directed arcs (plain Dijkstra)
    t, ou, od = cchgen.grid_topology(10, 11, seed, order=order, one_way=0.3)
    uw, dw, _, _, _ = t.relax(ou, od)
    c = orc.Cch(t.n, t.up_off, t.up_tgt, uw, t.down_off, t.down_tgt, dw)
    allr = np.arange(t.n, dtype=np.uint32)
    m, _ = c.matrix(allr, allr)
    assert np.array_equal(m, np.stack([orc.dijkstra_ebg(t.arcs, s) for s in range(t.n)]))
