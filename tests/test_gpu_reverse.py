"""Reverse (all-to-one) PHAST: a graph built with BF_FLAG_REVERSE vs the
oracle's query_block_gated_reverse restatement and the reference's KATs."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _graph(d, **kw):
    import bfphast
    return bfphast.Graph(d["n"], d["up_off"], d["up_tgt"], d["up_w"], d["down_off"],
                         d["down_tgt"], d["down_w"], **kw)


def test_reverse_kats(built, kats):
    # route/src/range/phast.rs:1375-1389, 1508-1560, 1420-1445
    k5 = kats["five_node"]
    g = _graph(k5["cch"], reverse=True)
    assert g.phast_query(0).tolist() == k5["rev"]["0"]
    b = k5["rev_bounded_count"]
    _, counts = g.isochrone_bitsets([b["target"]], [b["threshold"]])
    assert int(counts[0]) == b["count"]
    k3 = kats["asym_three_node"]
    g3 = _graph(k3["cch"], reverse=True)
    assert g3.phast_query(0).tolist() == k3["rev"]["0"]


def test_reverse_matches_oracle_and_transpose(built, grid100):
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    ro, rs, rw = orc.down_reverse(c)
    fwd = _graph(cch)
    rev = _graph(cch, reverse=True)
    for t in (0, 77, 12345, cch["n"] - 1):
        assert np.array_equal(rev.phast_query(t), c.reverse(t, ro, rs, rw))
    src = np.arange(5, cch["n"], 1013, dtype=np.uint32)[:30]
    tgt = np.arange(9, cch["n"], 701, dtype=np.uint32)[:40]
    assert np.array_equal(rev.matrix(tgt, src), fwd.matrix(src, tgt).T)
