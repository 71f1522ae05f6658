"""Target-restricted selection (RPHAST), checked on the CPU.

The matrix engine sweeps only the rows that reach a requested target along
DOWN edges (the set route/src/range/tree_phast.rs:320-417 selects). Its
device builder finds them in two steps: the targets' elimination-tree
ancestor paths give a candidate set, and candidates that are no target and
have no DOWN out-edge into a live candidate are peeled away. This file
restates both steps with plain loops and checks, on the grid and the small
country graph:
- every DOWN edge joins a node to one of its ancestors (so the candidates
  hold every row that reaches a target);
- the peeled set equals the rows from which a target is reachable, found by
  a search backwards from the targets;
- the set is closed under in-edges (every DOWN in-edge source of a selected
  row is selected), which makes the restricted sweep exact;
- the oracle's PHAST with every DOWN edge into an unselected row removed
  gives the full PHAST's distances at the targets (tolerance 0).
"""
import numpy as np
import pytest

from oracle import oracle as orc


def _etree(cch):
    """Parent of each rank in the elimination tree of the undirected union of
    UP and DOWN edges (Liu's algorithm with path compression); -1 at roots."""
    n = cch["n"]
    up_src = np.repeat(np.arange(n, dtype=np.int64), np.diff(cch["up_off"]).astype(np.int64))
    dn_src = np.repeat(np.arange(n, dtype=np.int64), np.diff(cch["down_off"]).astype(np.int64))
    lo = np.concatenate([up_src, cch["down_tgt"].astype(np.int64)])
    hi = np.concatenate([cch["up_tgt"].astype(np.int64), dn_src])
    order = np.argsort(hi, kind="stable")
    lo, hi = lo[order].tolist(), hi[order]
    starts = np.searchsorted(hi, np.arange(n + 1)).tolist()
    parent = [-1] * n
    anc = [-1] * n
    for j in range(n):
        for k in range(starts[j], starts[j + 1]):
            i = lo[k]
            while i != -1 and i < j:
                nxt = anc[i]
                anc[i] = j
                if nxt == -1:
                    parent[i] = j
                i = nxt
    return np.array(parent, dtype=np.int64)


def _candidates(parent, targets):
    mark = np.zeros(len(parent), bool)
    for x in targets:
        x = int(x)
        while x >= 0 and not mark[x]:
            mark[x] = True
            x = int(parent[x])
    return mark


def _peel(cch, cand, targets):
    """Counts of DOWN out-edges into the candidates; rows with none that are
    no target die and decrement their in-edge sources, until nothing dies."""
    n = cch["n"]
    doff, dtgt = cch["down_off"], cch["down_tgt"]
    is_t = np.zeros(n, bool)
    is_t[np.asarray(targets, dtype=np.int64)] = True
    cnt = np.zeros(n, np.int64)
    rin = [[] for _ in range(n)]  # in-edge sources within the candidates
    for u in np.flatnonzero(cand):
        for v in dtgt[doff[u]:doff[u + 1]]:
            if cand[v]:
                cnt[u] += 1
                rin[v].append(u)
    alive = cand.copy()
    front = [int(u) for u in np.flatnonzero(cand) if cnt[u] == 0 and not is_t[u]]
    while front:
        nxt = []
        for v in front:
            alive[v] = False
            for u in rin[v]:
                cnt[u] -= 1
                if cnt[u] == 0 and not is_t[u] and alive[u]:
                    nxt.append(u)
        front = nxt
    return alive


def _reach_backwards(cch, targets):
    """Rows with a DOWN path to a target: a search from the targets along
    reversed DOWN edges."""
    n = cch["n"]
    dn_src = np.repeat(np.arange(n, dtype=np.int64), np.diff(cch["down_off"]).astype(np.int64))
    dtgt = cch["down_tgt"].astype(np.int64)
    order = np.argsort(dtgt, kind="stable")
    src_by_tgt, tg = dn_src[order], dtgt[order]
    starts = np.searchsorted(tg, np.arange(n + 1))
    seen = np.zeros(n, bool)
    stack = [int(t) for t in targets]
    for t in stack:
        seen[t] = True
    while stack:
        v = stack.pop()
        for u in src_by_tgt[starts[v]:starts[v + 1]]:
            if not seen[u]:
                seen[u] = True
                stack.append(int(u))
    return seen


@pytest.mark.parametrize("graph", ["grid100", "country_small"])
def test_restricted_selection(request, graph):
    _, cch = request.getfixturevalue(graph)
    n = cch["n"]
    parent = _etree(cch)

    def is_ancestor(u, v):
        x = int(v)
        while x >= 0 and x < u:
            x = int(parent[x])
        return x == u

    # every DOWN edge u -> v (and every UP edge v -> u) joins v to an
    # ancestor u: a sample of each
    pick = np.random.default_rng(0)
    dn_src = np.repeat(np.arange(n), np.diff(cch["down_off"]).astype(np.int64))
    for e in pick.choice(len(dn_src), min(len(dn_src), 3000), replace=False):
        assert is_ancestor(int(dn_src[e]), int(cch["down_tgt"][e]))
    up_src = np.repeat(np.arange(n), np.diff(cch["up_off"]).astype(np.int64))
    for e in pick.choice(len(up_src), min(len(up_src), 3000), replace=False):
        assert is_ancestor(int(cch["up_tgt"][e]), int(up_src[e]))
    rng = np.random.default_rng(5)
    for T in (1, 16, 200):
        targets = rng.choice(n, T, replace=False)
        cand = _candidates(parent, targets)
        want = _reach_backwards(cch, targets)
        assert not np.any(want & ~cand)  # candidates hold every reaching row
        sel = _peel(cch, cand, targets)
        assert np.array_equal(sel, want)
        # closed under in-edges: a DOWN edge into a selected row starts at one
        into = sel[cch["down_tgt"]]
        assert np.all(sel[dn_src[into]])


def test_restricted_phast_is_exact(country_small):
    _, cch = country_small
    n = cch["n"]
    rng = np.random.default_rng(9)
    targets = rng.choice(n, 64, replace=False)
    sel = _reach_backwards(cch, targets)
    keep = sel[cch["down_tgt"]]
    dn_src = np.repeat(np.arange(n), np.diff(cch["down_off"]).astype(np.int64))
    off = np.zeros(n + 1, np.uint64)
    off[1:] = np.cumsum(np.bincount(dn_src[keep], minlength=n)).astype(np.uint64)
    full = orc.Cch.from_dict(cch)
    restricted = orc.Cch(n, cch["up_off"], cch["up_tgt"], cch["up_w"], off,
                         np.ascontiguousarray(cch["down_tgt"][keep]),
                         np.ascontiguousarray(cch["down_w"][keep]))
    assert 0 < int(sel.sum()) < n
    for s in rng.choice(n, 12, replace=False):
        assert np.array_equal(restricted.phast_query(int(s))[targets],
                              full.phast_query(int(s))[targets])
