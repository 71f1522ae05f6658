"""ctypes binding of the CPU oracle (phast_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker or the timed CPU baseline,
never as part of the product path.

Parity is pinned by the reference's own known-answer tests (see
tests/golden/reference_kats.json and tests/test_oracle_kat.py) and by plain
Dijkstra over the edge-based graph.
"""
import ctypes
import pathlib

import numpy as np

from .build import build_oracle

INF = 0xFFFFFFFF
_lib = None
_V = ctypes.c_void_p


def load():
    global _lib
    if _lib is None:
        so = build_oracle()
        lib = ctypes.CDLL(str(so))
        csr = [ctypes.c_uint32] + [_V] * 6
        lib.orc_phast_query.argtypes = csr + [ctypes.c_uint32, _V]
        lib.orc_query_batch.argtypes = csr + [_V, ctypes.c_uint32, _V]
        lib.orc_query_batch_bounded.argtypes = csr + [_V, ctypes.c_uint32, ctypes.c_uint32, _V]
        lib.orc_matrix_soa.argtypes = csr + [_V, ctypes.c_uint64, _V, ctypes.c_uint64, _V,
                                             ctypes.c_int]
        lib.orc_phast_bounded_seeded.argtypes = csr + [_V, _V, ctypes.c_uint32, ctypes.c_uint32,
                                                       _V, _V, ctypes.c_uint64]
        lib.orc_phast_bounded_seeded.restype = ctypes.c_uint64
        lib.orc_phast_bounded_seeded_2ch.argtypes = csr + [_V, _V, _V, _V, _V, ctypes.c_uint32,
                                                           ctypes.c_uint32, _V, _V, _V,
                                                           ctypes.c_uint64]
        lib.orc_phast_bounded_seeded_2ch.restype = ctypes.c_uint64
        lib.orc_isochrone_bitsets.argtypes = csr + [_V, _V, ctypes.c_uint64, _V, _V, ctypes.c_int]
        lib.orc_dijkstra_ebg.argtypes = [ctypes.c_uint32, _V, _V, _V, ctypes.c_uint32, _V]
        lib.orc_phast_reverse.argtypes = csr + [ctypes.c_uint32, _V]
        lib.orc_cch_relax.argtypes = [ctypes.c_uint32] + [_V] * 8
        lib.orc_cch_relax.restype = ctypes.c_uint32
        lib.orc_contour_cells.argtypes = [ctypes.c_uint64, _V, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_double, _V, ctypes.c_uint64]
        lib.orc_contour_cells.restype = ctypes.c_uint64
        lib.orc_sparse_contour.argtypes = [ctypes.c_uint32, _V, _V, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int32, ctypes.c_int32, _V, ctypes.c_uint64]
        lib.orc_sparse_contour.restype = ctypes.c_uint64
        lib.orc_sparse_closed.argtypes = [ctypes.c_uint32, _V, _V, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_int32,
                                          ctypes.c_int32, _V, ctypes.c_uint64, _V]
        lib.orc_sparse_closed.restype = ctypes.c_uint64
        lib.orc_contour_config.argtypes = [ctypes.c_int, ctypes.c_uint32] + [_V] * 4
        lib.orc_mercator.argtypes = [ctypes.c_uint64] + [_V] * 4
        lib.orc_inverse_mercator.argtypes = [ctypes.c_uint64] + [_V] * 4
        lib.orc_isochrone_geometry.argtypes = [ctypes.c_uint64, _V, _V, ctypes.c_uint32,
                                               ctypes.c_uint32, _V, _V, _V, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                               _V, ctypes.c_uint64, _V, ctypes.c_uint64, _V, _V,
                                               ctypes.c_uint32]
        lib.orc_isochrone_geometry.restype = ctypes.c_uint64
        lib.orc_cch_relax_par.argtypes = [ctypes.c_uint32] + [_V] * 8 + [ctypes.c_int, _V]
        lib.orc_cch_relax_par.restype = ctypes.c_uint32
        lib.orc_cch_relax_lex.argtypes = [ctypes.c_uint32] + [_V] * 12
        lib.orc_cch_relax_lex.restype = ctypes.c_uint32
        lib.orc_cch_bottom_up.argtypes = [ctypes.c_uint32] + [_V] * 12
        lib.orc_cch_bottom_up.restype = ctypes.c_uint32
        lib.orc_tile_emit.argtypes = ([_V, _V, ctypes.c_uint32, ctypes.c_uint32, _V, _V,
                                       ctypes.c_uint32, _V, _V, ctypes.c_uint32, ctypes.c_int]
                                      + [_V] * 4)
        lib.orc_tile_emit.restype = ctypes.c_uint64
        _lib = lib
    return _lib


def _a(x, dt):
    return np.ascontiguousarray(x, dtype=dt)


class Cch:
    """Rank-aligned CCH (up / down CSR by source) held for oracle calls."""

    def __init__(self, n, up_off, up_tgt, up_w, down_off, down_tgt, down_w):
        self.n = int(n)
        self.arrs = [_a(up_off, np.uint64), _a(up_tgt, np.uint32), _a(up_w, np.uint32),
                     _a(down_off, np.uint64), _a(down_tgt, np.uint32), _a(down_w, np.uint32)]

    @classmethod
    def from_dict(cls, d):
        return cls(d["n"], d["up_off"], d["up_tgt"], d["up_w"], d["down_off"], d["down_tgt"],
                   d["down_w"])

    def _csr(self):
        return [self.n] + [a.ctypes.data for a in self.arrs]

    def phast_query(self, origin):
        out = np.empty(self.n, dtype=np.uint32)
        load().orc_phast_query(*self._csr(), int(origin), out.ctypes.data)
        return out

    def query_batch(self, sources):
        s = _a(sources, np.uint32)
        out = np.empty((len(s), self.n), dtype=np.uint32)
        assert load().orc_query_batch(*self._csr(), s.ctypes.data, len(s), out.ctypes.data) == 0
        return out

    def query_batch_bounded(self, sources, threshold):
        s = _a(sources, np.uint32)
        out = np.empty((len(s), self.n), dtype=np.uint32)
        assert load().orc_query_batch_bounded(*self._csr(), s.ctypes.data, len(s), threshold,
                                              out.ctypes.data) == 0
        return out

    def matrix(self, sources, targets, threads=1):
        """compute_matrix_flat_soa (K = 8); returns (matrix, threads used)."""
        s, t = _a(sources, np.uint32), _a(targets, np.uint32)
        out = np.empty((len(s), len(t)), dtype=np.uint32)
        used = load().orc_matrix_soa(*self._csr(), s.ctypes.data, len(s), t.ctypes.data, len(t),
                                     out.ctypes.data, threads)
        return out, used

    def bounded_seeded(self, seeds, threshold):
        """run_phast_bounded_fast_seeded: (ranks, dists) with dist <= threshold."""
        r = _a([x[0] for x in seeds], np.uint32)
        c = _a([x[1] for x in seeds], np.uint32)
        rk = np.empty(self.n, dtype=np.uint32)
        ds = np.empty(self.n, dtype=np.uint32)
        cnt = load().orc_phast_bounded_seeded(*self._csr(), r.ctypes.data, c.ctypes.data, len(r),
                                              threshold, rk.ctypes.data, ds.ctypes.data, self.n)
        return rk[:cnt].copy(), ds[:cnt].copy()

    def bounded_seeded_2ch(self, seeds, threshold, up_len, down_len):
        """run_phast_bounded_fast_seeded_2ch: (ranks, times, lengths) with
        time <= threshold; seeds are (rank, time cost, length cost)."""
        r = _a([x[0] for x in seeds], np.uint32)
        c = _a([x[1] for x in seeds], np.uint32)
        ln = _a([x[2] for x in seeds], np.uint32)
        ul, dl = _a(up_len, np.uint32), _a(down_len, np.uint32)
        rk = np.empty(self.n, dtype=np.uint32)
        tm = np.empty(self.n, dtype=np.uint32)
        lo = np.empty(self.n, dtype=np.uint32)
        cnt = load().orc_phast_bounded_seeded_2ch(*self._csr(), ul.ctypes.data, dl.ctypes.data,
                                                  r.ctypes.data, c.ctypes.data, ln.ctypes.data,
                                                  len(r), threshold, rk.ctypes.data,
                                                  tm.ctypes.data, lo.ctypes.data, self.n)
        return rk[:cnt].copy(), tm[:cnt].copy(), lo[:cnt].copy()

    def isochrone_bitsets(self, origins, thresholds, threads=0):
        o, t = _a(origins, np.uint32), _a(thresholds, np.uint32)
        words = (self.n + 63) // 64
        bits = np.empty((len(o), words), dtype=np.uint64)
        counts = np.empty(len(o), dtype=np.uint64)
        load().orc_isochrone_bitsets(*self._csr(), o.ctypes.data, t.ctypes.data, len(o),
                                     bits.ctypes.data, counts.ctypes.data, threads)
        return bits, counts

    def reverse(self, target, rev_off, rev_src, rev_w):
        """query_block_gated_reverse with a caller-built DownReverseAdjFlat."""
        ro, rs, rw = _a(rev_off, np.uint64), _a(rev_src, np.uint32), _a(rev_w, np.uint32)
        out = np.empty(self.n, dtype=np.uint32)
        a = self.arrs
        load().orc_phast_reverse(self.n, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data,
                                 ro.ctypes.data, rs.ctypes.data, rw.ctypes.data, int(target),
                                 out.ctypes.data)
        return out


def dijkstra_ebg(ebg, origin_state):
    """Plain Dijkstra over the edge-based graph from one state."""
    off, dst, w = (_a(ebg["arc_off"], np.uint64), _a(ebg["arc_dst"], np.uint32),
                   _a(ebg["arc_w"], np.uint32))
    out = np.empty(ebg["n"], dtype=np.uint32)
    load().orc_dijkstra_ebg(ebg["n"], off.ctypes.data, dst.ctypes.data, w.ctypes.data,
                            int(origin_state), out.ctypes.data)
    return out


def down_reverse(cch):
    """DownReverseAdjFlat::build (bucket_ch.rs:355-418): DOWN edges by target."""
    n = cch.n
    doff, dtg, dw = cch.arrs[3], cch.arrs[4], cch.arrs[5]
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(doff.astype(np.int64)))
    keep = dw != INF
    src, tgt, w = src[keep], dtg[keep], dw[keep]
    order = np.argsort(tgt, kind="stable")
    cnt = np.bincount(tgt, minlength=n)
    off = np.zeros(n + 1, dtype=np.uint64)
    off[1:] = np.cumsum(cnt)
    return off, src[order], w[order]


def table_phast_lopsided(cch, src_seedsets, tgt_seedsets, threshold):
    """table_phast_lopsided (route/src/matrix/bucket_ch.rs:6717-6852), field
    part: per source one run_phast_bounded_fast_seeded field with bound
    T + max source part + max target part (:6741-6758); per target
    min over its seeds (rank, part) of F[rank] - part (saturating, :6785-6808);
    cells above T -> INF (:6800-6803). Pairs sharing a seed rank are the
    reference's bucket-engine conflicts (:6786-6790, :6826-6845): returned as
    cell indices with INF in the matrix."""
    S, T = len(src_seedsets), len(tgt_seedsets)
    out = np.full((S, T), INF, dtype=np.uint32)
    max_tgt = max([p for ss in tgt_seedsets for _, p in ss] or [0])
    conflicts = []
    for s, seeds in enumerate(src_seedsets):
        if not seeds:
            continue
        if threshold == INF:
            bound = INF
        else:
            bound = min(INF, threshold + max(c for _, c in seeds) + max_tgt)
        rk, ds = cch.bounded_seeded(seeds, bound)
        field = dict(zip(rk.tolist(), ds.tolist()))
        src_ranks = {r for r, _ in seeds}
        for t, tseeds in enumerate(tgt_seedsets):
            if not tseeds:
                continue
            if any(r in src_ranks for r, _ in tseeds):
                conflicts.append(s * T + t)
                continue
            best = INF
            for r, part in tseeds:
                f = field.get(r)
                if f is not None and f != INF:
                    best = min(best, f - part if f > part else 0)
            if threshold != INF and best != INF and best > threshold:
                best = INF
            out[s, t] = best
    return out, np.array(sorted(conflicts), dtype=np.uint64)


def table_phast_lopsided_2ch(cch, src_seedsets, tgt_seedsets, threshold, up_len, down_len):
    """table_phast_lopsided_2ch (route/src/matrix/bucket_ch.rs:6381-6521): per
    source one run_phast_bounded_fast_seeded_2ch field (bound as in the
    one-channel form, :6409-6418, from the seeds' time parts); per target,
    over its seeds in order, the first with the strictly smallest
    F_t[rank] - part_t (saturating) also gives F_l[rank] - part_l (:6452-6466);
    time cells above T -> INF in both channels (:6467-6470). Same-rank pairs
    are conflicts (:6460-6463), INF in both matrices."""
    S, T = len(src_seedsets), len(tgt_seedsets)
    out_t = np.full((S, T), INF, dtype=np.uint32)
    out_l = np.full((S, T), INF, dtype=np.uint32)
    max_tgt = max([p for ss in tgt_seedsets for _, p, _ in ss] or [0])
    conflicts = []
    for s, seeds in enumerate(src_seedsets):
        if not seeds:
            continue
        if threshold == INF:
            bound = INF
        else:
            bound = min(INF, threshold + max(c for _, c, _ in seeds) + max_tgt)
        rk, tm, ln = cch.bounded_seeded_2ch(seeds, bound, up_len, down_len)
        field = {int(r): (int(a), int(b)) for r, a, b in zip(rk, tm, ln)}
        src_ranks = {r for r, _, _ in seeds}
        for t, tseeds in enumerate(tgt_seedsets):
            if not tseeds:
                continue
            if any(r in src_ranks for r, _, _ in tseeds):
                conflicts.append(s * T + t)
                continue
            bt, bl = INF, INF
            for r, pt, pl in tseeds:
                f = field.get(r)
                if f is not None and f[0] != INF:
                    at = f[0] - pt if f[0] > pt else 0
                    if at < bt:
                        bt = at
                        bl = f[1] - pl if f[1] > pl else 0
            if threshold != INF and bt != INF and bt > threshold:
                bt, bl = INF, INF
            out_t[s, t], out_l[s, t] = bt, bl
    return out_t, out_l, np.array(sorted(conflicts), dtype=np.uint64)



class CchTopo:
    """The reference's rank-space CCH topology (formats/cch_topo.rs:250-290):
    UP edges u -> v (v > u) and DOWN edges u -> v (v < u) as two CSRs with
    targets ascending per node, shortcut flags and middles (u32::MAX on an
    original arc)."""

    def __init__(self, n, up_off, up_tgt, down_off, down_tgt, up_short=None, down_short=None,
                 up_mid=None, down_mid=None):
        self.n = int(n)
        self.up_off, self.up_tgt = _a(up_off, np.uint64), _a(up_tgt, np.uint32)
        self.down_off, self.down_tgt = _a(down_off, np.uint64), _a(down_tgt, np.uint32)
        nu, nd = len(self.up_tgt), len(self.down_tgt)
        self.up_short = _a(np.zeros(nu, np.uint8) if up_short is None else up_short, np.uint8)
        self.down_short = _a(np.zeros(nd, np.uint8) if down_short is None else down_short, np.uint8)
        self.up_mid = _a(np.full(nu, INF, np.uint32) if up_mid is None else up_mid, np.uint32)
        self.down_mid = _a(np.full(nd, INF, np.uint32) if down_mid is None else down_mid, np.uint32)

    def _csr(self):
        return (self.n, self.up_off.ctypes.data, self.up_tgt.ctypes.data,
                self.down_off.ctypes.data, self.down_tgt.ctypes.data)

    @classmethod
    def from_upper(cls, topo):
        """Directed form of a chordal topology given in upper-neighbour form
        (edge e of rank j joins j and tgt[e] > j): every pair becomes an UP
        edge j -> tgt[e] and a DOWN edge tgt[e] -> j. Returns the topology and
        the per-edge weights (orig_up, orig_down) mapped onto it."""
        off, tgt = _a(topo["off"], np.uint64), _a(topo["tgt"], np.uint32)
        n = len(off) - 1
        low = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off).astype(np.int64))
        order = np.argsort(tgt, kind="stable")  # (target, source): sources already ascend
        down_off = np.zeros(n + 1, np.uint64)
        down_off[1:] = np.cumsum(np.bincount(tgt, minlength=n))
        t = cls(n, off, tgt, down_off, low[order])
        return t, order

    def relax(self, up_w, down_w, up_mid=None, down_mid=None, threads=1):
        """triangle_relax_parallel (customization.rs:1083-1200) from the given
        seeds; returns (up_w, down_w, up_mid, down_mid, passes). threads > 1
        (or 0 = all cores) runs the apex-parallel atomic form."""
        uw, dw = _a(up_w, np.uint32).copy(), _a(down_w, np.uint32).copy()
        um = (self.up_mid if up_mid is None else _a(up_mid, np.uint32)).copy()
        dm = (self.down_mid if down_mid is None else _a(down_mid, np.uint32)).copy()
        if threads == 1:
            passes = load().orc_cch_relax(*self._csr(), uw.ctypes.data, dw.ctypes.data,
                                          um.ctypes.data, dm.ctypes.data)
        else:
            used = ctypes.c_int(0)
            passes = load().orc_cch_relax_par(*self._csr(), uw.ctypes.data, dw.ctypes.data,
                                              um.ctypes.data, dm.ctypes.data, int(threads),
                                              ctypes.byref(used))
            self.threads_used = used.value
        if passes == 0:
            raise RuntimeError("triangle relaxation did not converge in 100 passes")
        return uw, dw, um, dm, passes

    def relax_lex(self, up_t, down_t, up_l, down_l, up_mid=None, down_mid=None):
        """triangle_relax_lex_parallel (customization.rs:1253-1436); returns
        (up_t, down_t, up_mid, down_mid, passes)."""
        ut, dt = _a(up_t, np.uint32).copy(), _a(down_t, np.uint32).copy()
        ul, dl = _a(up_l, np.uint32), _a(down_l, np.uint32)
        um = (self.up_mid if up_mid is None else _a(up_mid, np.uint32)).copy()
        dm = (self.down_mid if down_mid is None else _a(down_mid, np.uint32)).copy()
        passes = load().orc_cch_relax_lex(*self._csr(), self.up_short.ctypes.data,
                                          self.down_short.ctypes.data, ut.ctypes.data,
                                          dt.ctypes.data, ul.ctypes.data, dl.ctypes.data,
                                          um.ctypes.data, dm.ctypes.data)
        if passes == 0:
            raise RuntimeError("lexicographic relaxation did not converge in 100 passes")
        return ut, dt, um, dm, passes

    def bottom_up(self, orig_up, orig_down, up_mid=None, down_mid=None):
        """bottom_up_customize / bottom_up_with_external_middles
        (customization.rs:953-1052); returns (up_w, down_w)."""
        um = self.up_mid if up_mid is None else _a(up_mid, np.uint32)
        dm = self.down_mid if down_mid is None else _a(down_mid, np.uint32)
        ou, od = _a(orig_up, np.uint32), _a(orig_down, np.uint32)
        uw = np.empty(len(self.up_tgt), np.uint32)
        dw = np.empty(len(self.down_tgt), np.uint32)
        rc = load().orc_cch_bottom_up(*self._csr(), self.up_short.ctypes.data,
                                      self.down_short.ctypes.data, um.ctypes.data, dm.ctypes.data,
                                      ou.ctypes.data, od.ctypes.data, uw.ctypes.data,
                                      dw.ctypes.data)
        if rc:
            raise IndexError("shortcut middle is not a rank")
        return uw, dw


# ---------------------------------------------------------------------------
# Isochrone geometry (server/geometry.rs:281-418, range/sparse_contour.rs)

MODES = {"car": 0, "bike": 1, "foot": 2}


def _ring(fn, cap=1 << 16):
    """Calls fn(out, cap) -> n until the (x, y) ring fits."""
    while True:
        out = np.empty(2 * cap, np.float64)
        n = fn(out.ctypes.data, cap)
        if n <= cap:
            return out[:2 * n].reshape(-1, 2)
        cap = int(n)


def contour_cells(cells, anchor=None):
    """extract_contour_sparse on unit cells [(col, row), ...]: the ring of
    cell-centre vertices, (x, y) rows."""
    c = np.ascontiguousarray(np.asarray(cells, np.int32).reshape(-1, 2))
    ax, ay = anchor if anchor is not None else (0.0, 0.0)
    return _ring(lambda o, k: load().orc_contour_cells(len(c), c.ctypes.data,
                                                       int(anchor is not None), ax, ay, o, k))


def _segments(segments):
    off = np.zeros(len(segments) + 1, np.uint64)
    off[1:] = np.cumsum([len(s) for s in segments])
    pts = np.ascontiguousarray(np.asarray([p for s in segments for p in s], np.int32).reshape(-1, 2))
    return off, pts


def sparse_contour(segments, cell_m, dilation, erosion, simplify_m, anchor=None):
    """generate_sparse_contour_anchored: segments of (lat_e7, lon_e7) points;
    the outer ring as (lon, lat) rows."""
    if not segments:
        return np.empty((0, 2))
    off, pts = _segments(segments)
    a_lat, a_lon = anchor if anchor is not None else (0, 0)
    return _ring(lambda o, k: load().orc_sparse_contour(
        len(segments), off.ctypes.data, pts.ctypes.data, cell_m, dilation, erosion, simplify_m,
        int(anchor is not None), int(a_lat), int(a_lon), o, k))


def contour_config(mode, threshold_s):
    """SparseContourConfig::for_mode_name_with_threshold:
    (cell_m, dilation_rounds, erosion_rounds, simplify_m)."""
    c, s = ctypes.c_double(), ctypes.c_double()
    d, e = ctypes.c_int(), ctypes.c_int()
    load().orc_contour_config(MODES.get(mode, 0), int(threshold_s), ctypes.byref(c), ctypes.byref(d),
                              ctypes.byref(e), ctypes.byref(s))
    return c.value, d.value, e.value, s.value


def mercator(lat, lon):
    lat, lon = _a(np.atleast_1d(lat), np.float64), _a(np.atleast_1d(lon), np.float64)
    x, y = np.empty(len(lat)), np.empty(len(lat))
    load().orc_mercator(len(lat), lat.ctypes.data, lon.ctypes.data, x.ctypes.data, y.ctypes.data)
    return x, y


def inverse_mercator(x, y):
    x, y = _a(np.atleast_1d(x), np.float64), _a(np.atleast_1d(y), np.float64)
    lon, lat = np.empty(len(x)), np.empty(len(x))
    load().orc_inverse_mercator(len(x), x.ctypes.data, y.ctypes.data, lon.ctypes.data,
                                lat.ctypes.data)
    return lon, lat


def isochrone_geometry(nodes, dists, max_t, node_w, poly_off, poly, mode="car", origin=None,
                       tier=None):
    """build_isochrone_geometry_sparse: settled (node, dist) pairs, per-node
    weights and (lat_e7, lon_e7) polylines; returns (ring (lon, lat) rows,
    closed cells (col, row) rows ascending by row then column, grid origin
    (min_x, min_y) in Mercator metres). `tier` (default max_t) selects the
    contour configuration."""
    nodes, dists = _a(nodes, np.uint32), _a(dists, np.uint32)
    node_w, poly_off = _a(node_w, np.uint32), _a(poly_off, np.uint64)
    poly = np.ascontiguousarray(np.asarray(poly, np.int32).reshape(-1, 2))
    o_lon, o_lat = origin if origin is not None else (0.0, 0.0)
    cap_c = 1 << 20
    while True:
        cells = np.empty(2 * cap_c, np.int32)
        nc = ctypes.c_uint64(0)
        grid = np.zeros(2)
        ring = _ring(lambda o, k: load().orc_isochrone_geometry(
            len(nodes), nodes.ctypes.data, dists.ctypes.data, int(max_t), len(node_w),
            node_w.ctypes.data, poly_off.ctypes.data, poly.ctypes.data, MODES.get(mode, 0),
            int(origin is not None), o_lon, o_lat, o, k, cells.ctypes.data, cap_c,
            ctypes.byref(nc), grid.ctypes.data, int(max_t if tier is None else tier)))
        if nc.value <= cap_c:
            return ring, cells[:2 * nc.value].reshape(-1, 2), grid
        cap_c = int(nc.value)


def sparse_closed(segments, cell_m, dilation, erosion, anchor=None):
    """Stamped and closed cells of generate_sparse_contour_anchored's
    segments: ((col, row) rows ascending by row then column, grid origin)."""
    off, pts = _segments(segments)
    a_lat, a_lon = anchor if anchor is not None else (0, 0)
    cap = 1 << 20
    while True:
        cells = np.empty(2 * cap, np.int32)
        grid = np.zeros(2)
        n = load().orc_sparse_closed(len(segments), off.ctypes.data, pts.ctypes.data, cell_m,
                                     dilation, erosion, int(anchor is not None), int(a_lat),
                                     int(a_lon), cells.ctypes.data, cap, grid.ctypes.data)
        if n <= cap:
            return cells[:2 * n].reshape(-1, 2), grid
        cap = int(n)


def mask_csr(mask):
    """A radius mask (list, indexed by original source, of sorted lists of
    original destination indices) as (offsets u64, flat u32)."""
    off = np.zeros(len(mask) + 1, np.uint64)
    off[1:] = np.cumsum([len(m) for m in mask]) if len(mask) else []
    flat = np.asarray([v for m in mask for v in m], np.uint32)
    return off, flat


def tile_emit(matrix, n_src, n_dst, src_orig, dst_orig, threshold=INF, mask=None, lat=None,
              sparse=False):
    """build_matrix_batch / build_matrix_tile_batch (flight.rs:432-589):
    (source_idx, target_idx, duration_ms, distance_m) columns of a row-major
    n_src x n_dst block. `mask` as in mask_csr (or an (offsets, flat) pair)."""
    m = _a(np.asarray(matrix).reshape(-1), np.uint32)
    so, do = _a(src_orig, np.uint32), _a(dst_orig, np.uint32)
    la = None if lat is None else _a(np.asarray(lat).reshape(-1), np.uint32)
    if mask is not None and not (isinstance(mask, tuple) and len(mask) == 2
                                 and isinstance(mask[0], np.ndarray)):
        mask = mask_csr(mask)
    cap = max(1, n_src * n_dst)
    cols = [np.empty(cap, np.uint32) for _ in range(4)]
    moff, mflat = (None, None) if mask is None else (_a(mask[0], np.uint64),
                                                     _a(mask[1], np.uint32))
    n_mask = 0 if mask is None else len(moff) - 1
    keep = np.zeros(1, np.uint32) if mflat is None or len(mflat) == 0 else mflat
    k = load().orc_tile_emit(m.ctypes.data, None if la is None else la.ctypes.data, n_src, n_dst,
                             so.ctypes.data, do.ctypes.data, threshold,
                             None if moff is None else moff.ctypes.data,
                             None if moff is None else keep.ctypes.data, n_mask, int(sparse),
                             *[c.ctypes.data for c in cols])
    if k == 0xFFFFFFFFFFFFFFFF:
        raise IndexError("a source's original index has no radius list")
    return tuple(c[:k].copy() for c in cols)
