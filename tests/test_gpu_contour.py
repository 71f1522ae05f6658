"""GPU contour rasters (bf_contour_rasters) against the oracle's closed cell
sets (route/src/range/sparse_contour.rs:650-770), bit for bit, for batches of
isochrones with different cell sizes, morphology and anchors."""
import numpy as np
import pytest

import contourgen
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dil,ero", [(2, 2), (3, 3), (0, 0), (2, 1)])
def test_rasters_match_oracle(built, dil, ero):
    import bfphast
    rng = np.random.default_rng(100 + dil * 7 + ero)
    cells_m = [30.0, 60.0, 120.0, 30.0 * 6.67, 25.0, 40.0]
    isos, want = [], []
    for k in range(12):
        segs, anchor = contourgen.isochrone(rng, int(rng.integers(1, 400)))
        cell = cells_m[k % len(cells_m)]
        isos.append({"segments": contourgen.mercator_segments(segs), "cell_m": cell,
                     "anchor": contourgen.mercator_point(anchor) if anchor else None})
        want.append(orc.sparse_closed(segs, cell, dil, ero, anchor))
    got = bfphast.contour_rasters(isos, dil, ero)
    for (gc, go), (wc, wo) in zip(got, want):
        assert go == tuple(wo)
        assert np.array_equal(gc, wc)
    # a call after releasing the kept buffers allocates them again
    bfphast.load().bf_contour_release(0)
    again = bfphast.contour_rasters(isos[:3], dil, ero)
    for (gc, _), (wc, _) in zip(again, want[:3]):
        assert np.array_equal(gc, wc)


def test_empty_and_single_point_isochrones(built):
    import bfphast
    rng = np.random.default_rng(5)
    segs, _ = contourgen.isochrone(rng, 30)
    one = [[segs[0][0]]]
    isos = [{"segments": [], "cell_m": 30.0, "anchor": (4.8e5, 6.58e6)},
            {"segments": contourgen.mercator_segments(one), "cell_m": 30.0},
            {"segments": contourgen.mercator_segments(segs), "cell_m": 60.0}]
    got = bfphast.contour_rasters(isos, 2, 2)
    assert len(got[0][0]) == 0
    for (gc, _), s, cell in zip(got[1:], (one, segs), (30.0, 60.0)):
        wc, _ = orc.sparse_closed(s, cell, 2, 2)
        assert np.array_equal(gc, wc)


def test_polygons_match_oracle(built):
    # the whole pipeline: GPU rasters, then tracing, anchored ring,
    # back-projection and simplification, against the oracle's rings
    import bfphast
    rng = np.random.default_rng(77)
    segs_all, isos, cfgs = [], [], []
    for k in range(10):
        segs, anchor = contourgen.isochrone(rng, int(rng.integers(20, 600)), spread=0.01)
        mode = ("car", "bike", "foot")[k % 3]
        cell, dil, ero, simp = orc.contour_config(mode, (300, 1200, 3000, 7200)[k % 4])
        segs_all.append((segs, anchor))
        isos.append({"segments": contourgen.mercator_segments(segs), "cell_m": cell,
                     "anchor": contourgen.mercator_point(anchor) if anchor else None})
        cfgs.append((cell, dil, ero, simp))
    for dil, ero in {(c[1], c[2]) for c in cfgs}:
        idx = [k for k, c in enumerate(cfgs) if (c[1], c[2]) == (dil, ero)]
        pts, seg_pt, iso_seg = [], [0], [0]
        for k in idx:
            for a in isos[k]["segments"]:
                pts.append(a)
                seg_pt.append(seg_pt[-1] + len(a))
            iso_seg.append(len(seg_pt) - 1)
        has = np.array([isos[k]["anchor"] is not None for k in idx], np.uint8)
        anc = np.array([isos[k]["anchor"] or (0.0, 0.0) for k in idx])
        ras, words = bfphast.contour_rasters_flat(np.concatenate(pts), seg_pt, iso_seg,
                                                  [cfgs[k][0] for k in idx], dil, ero, has, anc)
        rings = bfphast.contour_polygons(ras, words, [cfgs[k][0] for k in idx],
                                         [cfgs[k][3] for k in idx], has, anc)
        for k, ring in zip(idx, rings):
            segs, anchor = segs_all[k]
            want = orc.sparse_contour(segs, cfgs[k][0], dil, ero, cfgs[k][3], anchor)
            assert np.array_equal(ring, want)


def test_isochrone_polygons_end_to_end(built, country_small):
    # bf_isochrone_polygons from origins to rings against the oracle's
    # handler restatement on the oracle's settled sets
    import bfphast
    e, cch = country_small
    rows, cols = 200, 250
    ii = np.arange(e["n_intersections"], dtype=np.int64)
    lat = (500_000_000 + (ii // cols) * 9000).astype(np.int32)
    lon = (30_000_000 + (ii % cols) * 14000).astype(np.int32)
    st = cch["rank_to_state"]
    tail, head = e["state_tail"][st], e["state_head"][st]
    poly = np.stack([np.stack([lat[tail], lon[tail]], 1), np.stack([lat[head], lon[head]], 1)],
                    1).reshape(-1, 2)
    off = np.arange(0, 2 * cch["n"] + 1, 2, dtype=np.uint64)
    w = e["node_weight"][st]
    geo = bfphast.Geometry(off, poly, w)
    g = bfphast.Graph.from_cch(cch)
    c = orc.Cch.from_dict(cch)
    origins = np.array([5, 1234, 40000, 77777 % cch["n"]], np.uint32)
    thr = np.array([3000, 18000, 6000, 36000], np.uint32)
    tiers = thr // 10
    for mode, name in ((bfphast.MODE_CAR, "car"), (bfphast.MODE_FOOT, "foot")):
        rings, ph = bfphast.isochrone_polygons(g, geo, origins, thr, tiers, mode)
        for i, o in enumerate(origins):
            rk, ds = c.bounded_seeded([(int(o), 0)], int(thr[i]))
            # the oracle's tier comes from the threshold it is given
            want = _oracle_ring(rk, ds, int(thr[i]), int(tiers[i]), w, off, poly, name)
            assert len(rings[i]) >= 3 and np.array_equal(rings[i], want)


def _oracle_ring(rk, ds, thr, tier, w, off, poly, mode):
    # build_isochrone_geometry_sparse with the contour tier of `tier`
    cell, dil, ero, simp = orc.contour_config(mode, tier)
    segs, anchor, best = [], None, 0xFFFFFFFF
    for r, d in zip(rk, ds):
        wr = int(w[r])
        if d > thr or wr == 0 or wr == 0xFFFFFFFF:
            continue
        a, b = poly[off[r]], poly[off[r] + 1]
        if d < best:
            best, anchor = d, (int(a[0]), int(a[1]))
        if d + wr <= thr:
            segs.append([(int(a[0]), int(a[1])), (int(b[0]), int(b[1]))])
            continue
        frac = np.float32(thr - d) / np.float32(wr)
        if frac <= 0:
            continue
        if frac >= 1:
            segs.append([(int(a[0]), int(a[1])), (int(b[0]), int(b[1]))])
            continue
        cl = int(a[0]) + int(np.trunc(np.float32(int(b[0]) - int(a[0])) * frac))
        cn = int(a[1]) + int(np.trunc(np.float32(int(b[1]) - int(a[1])) * frac))
        segs.append([(int(a[0]), int(a[1])), (cl, cn)])
    return orc.sparse_contour(segs, cell, dil, ero, simp, anchor)
