"""Directed CCH topologies for the customization tests.

A rows x cols grid whose neighbouring cells are joined by arcs in one or both
directions (one-way streets) with seeded weights, some u32::MAX (filtered
arcs), ranked by nested dissection (or at random), then contracted the way
the reference does (route/src/contraction.rs:240-390): eliminating v adds
u -> w with middle v for every higher in-neighbour u and higher
out-neighbour w of v (u != w) unless that arc exists. The result is the
rank-space topology (formats/cch_topo.rs:250-290) with shortcut flags,
middles and original weights per edge.
"""
import numpy as np

from oracle import oracle as orc

INF = 0xFFFFFFFF


def _nd_order(rows, cols):
    """Nested-dissection elimination order of a grid (separators last)."""
    out = []

    def rec(r0, r1, c0, c1):
        h, w = r1 - r0, c1 - c0
        if h <= 0 or w <= 0:
            return
        if h * w <= 4:
            out.extend(r * cols + c for r in range(r0, r1) for c in range(c0, c1))
            return
        if w >= h:
            m = c0 + w // 2
            rec(r0, r1, c0, m)
            rec(r0, r1, m + 1, c1)
            out.extend(r * cols + m for r in range(r0, r1))
        else:
            m = r0 + h // 2
            rec(r0, m, c0, c1)
            rec(m + 1, r1, c0, c1)
            out.extend(m * cols + c for c in range(c0, c1))

    rec(0, rows, 0, cols)
    return out


def grid_topology(rows, cols, seed, one_way=0.25, w_max=60, p_inf=0.05, order="nd",
                  diagonals=0.0):
    """Returns (oracle.CchTopo with flags and middles, orig_up, orig_down);
    the topology's `arcs` attribute holds the original arcs as a CSR."""
    rng = np.random.default_rng(seed)
    n = rows * cols
    pairs = []
    for r in range(rows):
        for c in range(cols):
            a = r * cols + c
            if c + 1 < cols:
                pairs.append((a, a + 1))
            if r + 1 < rows:
                pairs.append((a, a + cols))
            if diagonals and r + 1 < rows and c + 1 < cols and rng.random() < diagonals:
                pairs.append((a, a + cols + 1))
    arcs = {}
    for a, b in pairs:
        kind = rng.random()
        dirs = [(a, b), (b, a)] if kind >= one_way else [(a, b) if kind < one_way / 2 else (b, a)]
        for u, v in dirs:
            w = INF if rng.random() < p_inf else int(rng.integers(0, w_max))
            arcs[(u, v)] = w
    if order == "nd":
        elim = _nd_order(rows, cols)
    else:
        elim = list(rng.permutation(n))
    rank = np.empty(n, np.int64)
    rank[np.asarray(elim)] = np.arange(n)
    # arcs in rank space: (u, v) -> (original weight, middle)
    edges = {(int(rank[u]), int(rank[v])): (w, INF) for (u, v), w in arcs.items()}
    out_hi = [set() for _ in range(n)]  # higher out-neighbours
    in_hi = [set() for _ in range(n)]   # higher in-neighbours
    for (u, v) in edges:
        if v > u:
            out_hi[u].add(v)
        else:
            in_hi[v].add(u)
    for v in range(n):
        for u in sorted(in_hi[v]):
            for w in sorted(out_hi[v]):
                if u == w or (u, w) in edges:
                    continue
                edges[(u, w)] = (INF, v)
                if w > u:
                    out_hi[u].add(w)
                else:
                    in_hi[w].add(u)
    up = sorted((u, v) for (u, v) in edges if v > u)
    dn = sorted((u, v) for (u, v) in edges if v < u)

    def csr(lst):
        off = np.zeros(n + 1, np.uint64)
        if lst:
            off[1:] = np.cumsum(np.bincount([u for u, _ in lst], minlength=n))
        tgt = np.array([v for _, v in lst], np.uint32)
        short = np.array([edges[e][1] != INF for e in lst], np.uint8)
        mid = np.array([edges[e][1] for e in lst], np.uint32)
        orig = np.array([edges[e][0] for e in lst], np.uint32)
        return off, tgt, short, mid, orig

    uo, ut, us, um, ou = csr(up)
    do, dt, ds, dm, od = csr(dn)
    topo = orc.CchTopo(n, uo, ut, do, dt, up_short=us, down_short=ds, up_mid=um, down_mid=dm)
    # the original arcs in rank space (finite weights), as a CSR for Dijkstra
    fin = sorted((u, v, w) for (u, v), (w, m) in edges.items() if m == INF and w != INF)
    arc_off = np.zeros(n + 1, np.uint64)
    if fin:
        arc_off[1:] = np.cumsum(np.bincount([u for u, _, _ in fin], minlength=n))
    topo.arcs = {"n": n, "arc_off": arc_off, "arc_dst": np.array([v for _, v, _ in fin], np.uint32),
                 "arc_w": np.array([w for _, _, w in fin], np.uint32)}
    return topo, ou, od
