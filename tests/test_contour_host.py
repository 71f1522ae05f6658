"""bf_contour_polygons (boundary tracing, anchored ring, back-projection,
Douglas-Peucker, on the GPU) on rasters built from the oracle's closed cells,
against the oracle's whole contour pipeline
(route/src/range/sparse_contour.rs:770-1183), vertex for vertex; the
projection and tier helpers run on the host."""
import numpy as np
import pytest

import contourgen
from oracle import oracle as orc


def _raster(cells, grid, off):
    import bfphast
    c0, r0 = int(cells[:, 0].min()) - 1, int(cells[:, 1].min()) - 1
    c1, r1 = int(cells[:, 0].max()) + 1, int(cells[:, 1].max()) + 1
    wpr, h = (c1 - c0 + 1 + 63) // 64, r1 - r0 + 1
    words = np.zeros(wpr * h, np.uint64)
    lc, lr = cells[:, 0] - c0, cells[:, 1] - r0
    np.bitwise_or.at(words, lr * wpr + lc // 64, np.left_shift(np.uint64(1), (lc % 64).astype(np.uint64)))
    r = bfphast.Raster(col0=c0, row0=r0, width_words=wpr, height=h, word_offset=off,
                       origin_x=grid[0], origin_y=grid[1])
    return r, words


@pytest.mark.gpu
def test_host_polygons_match_oracle(built):
    import bfphast
    rng = np.random.default_rng(9)
    rasters, words, cfg, anchors, want = [], [], [], [], []
    off = 0
    for k in range(8):
        segs, anchor = contourgen.isochrone(rng, int(rng.integers(5, 300)), spread=0.01)
        cell, dil, ero, simp = orc.contour_config(("car", "bike", "foot")[k % 3], 600 + 900 * k)
        cells, grid = orc.sparse_closed(segs, cell, dil, ero, anchor)
        r, w = _raster(cells, grid, off)
        off += len(w)
        rasters.append(r)
        words.append(w)
        cfg.append((cell, simp))
        anchors.append(contourgen.mercator_point(anchor) if anchor else None)
        want.append(orc.sparse_contour(segs, cell, dil, ero, simp, anchor))
    has = np.array([a is not None for a in anchors], np.uint8)
    anc = np.array([a or (0.0, 0.0) for a in anchors])
    rings = bfphast.contour_polygons(rasters, np.concatenate(words), [c[0] for c in cfg],
                                     [c[1] for c in cfg], has, anc)
    for got, w in zip(rings, want):
        assert len(w) >= 3 and np.array_equal(got, w)


def test_projection_and_tiers_match_oracle(built):
    # the library's to_mercator and SparseContourConfig restatements agree
    # with the oracle's bit for bit (same host libm)
    import bfphast
    rng = np.random.default_rng(4)
    pts = np.stack([rng.integers(480_000_000, 520_000_000, 5000),
                    rng.integers(20_000_000, 60_000_000, 5000)], 1).astype(np.int32)
    xy = bfphast.mercator(pts)
    x, y = orc.mercator(pts[:, 0] / 1e7, pts[:, 1] / 1e7)
    assert np.array_equal(xy[:, 0], x) and np.array_equal(xy[:, 1], y)
    for mode, name in ((0, "car"), (1, "bike"), (2, "foot")):
        for t in (0, 300, 600, 601, 1800, 1801, 3600, 3601, 7200):
            assert bfphast.contour_config(mode, t) == orc.contour_config(name, t)


@pytest.mark.gpu
def test_host_polygons_concurrent_calls(built):
    # bf_contour_polygons from several host threads at once (the tracer's
    # device workspace is shared and its calls are serialised): every call
    # returns the single-threaded rings
    import threading
    import bfphast
    rng = np.random.default_rng(21)
    rasters, words, cells_m, simp_m = [], [], [], []
    off = 0
    for k in range(6):
        segs, _ = contourgen.isochrone(rng, int(rng.integers(20, 200)), spread=0.01)
        cell, dil, ero, simp = orc.contour_config("car", 600 + 600 * k)
        cells, grid = orc.sparse_closed(segs, cell, dil, ero)
        r, w = _raster(cells, grid, off)
        off += len(w)
        rasters.append(r)
        words.append(w)
        cells_m.append(cell)
        simp_m.append(simp)
    flat = np.concatenate(words)
    want = bfphast.contour_polygons(rasters, flat, cells_m, simp_m)
    got, errors = {}, []

    def run(i):
        try:
            for _ in range(3):
                got[i] = bfphast.contour_polygons(rasters[::-1], flat, cells_m[::-1], simp_m[::-1])
        except Exception as e:  # pragma: no cover - reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(6)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    for rings in got.values():
        for a, b in zip(rings, want[::-1]):
            assert np.array_equal(a, b)
