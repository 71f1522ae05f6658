"""Isochrone geometry oracle (route/src/server/geometry.rs:281-418,
route/src/range/sparse_contour.rs), pinned by the reference's own contour
tests. CPU only."""
import numpy as np
import pytest

from oracle import oracle as orc


def _half(ring):
    return [tuple(int(round(v * 2)) for v in p) for p in ring]


def test_cell_centre_rings(built, kats):
    # sparse_contour.rs:1453-1528: rings through perimeter-cell centres, no
    # consecutive duplicates, not pre-closed
    k = kats["sparse_contour"]
    for case in ("block3", "l_shape"):
        ring = orc.contour_cells(k[case]["cells"])
        q = _half(ring)
        assert sorted(q) == sorted(tuple(v) for v in k[case]["ring_half_cells"])
        assert len(q) == len(k[case]["ring_half_cells"])
        assert all(a != b for a, b in zip(q, q[1:])) and q[0] != q[-1]
    ring = orc.contour_cells(k["block3"]["cells"])  # :1483-1503, no half-cell overshoot
    assert ring[:, 0].min() == 0.5 and ring[:, 0].max() == 2.5
    assert ring[:, 1].min() == 0.5 and ring[:, 1].max() == 2.5


def test_negative_cells_across_tiles(built):
    # a 3x3 block around the origin spans four tiles and negative columns
    # (Euclidean tile division, sparse_contour.rs:1217-1241)
    ring = orc.contour_cells([(c, r) for r in range(-1, 2) for c in range(-1, 2)])
    assert sorted(_half(ring)) == sorted([(-1, -1), (1, -1), (3, -1), (3, 1), (3, 3), (1, 3),
                                          (-1, 3), (-1, 1)])


def _point_in_ring(p, ring):
    inside, n = False, len(ring)
    for i in range(n):
        (x1, y1), (x2, y2) = ring[i], ring[(i + 1) % n]
        if (y1 > p[1]) != (y2 > p[1]) and p[0] < (x2 - x1) * (p[1] - y1) / (y2 - y1) + x1:
            inside = not inside
    return inside


def test_anchored_component_selection(built, kats):
    # sparse_contour.rs:1421-1451
    k = kats["sparse_contour"]["anchored"]
    largest = orc.contour_cells(k["cells"])
    anchored = orc.contour_cells(k["cells"], anchor=k["origin"])
    assert len(largest) > len(anchored)
    near = min(np.hypot(*(anchored - np.array(k["origin"])).T))
    assert _point_in_ring(k["origin"], anchored) or near <= 1.0
    assert not _point_in_ring(k["origin"], largest)
    assert len(orc.contour_cells(k["cells"], anchor=k["inside_big"])) == len(largest)
    assert len(orc.contour_cells(k["cells"], anchor=k["outside"])) == len(largest)


def test_largest_component_and_determinism(built, kats):
    # sparse_contour.rs:1530-1576
    k = kats["sparse_contour"]["largest"]
    ring = orc.contour_cells(k["cells"])
    lo, hi = k["bbox"]
    assert len(ring) and (ring >= lo).all() and (ring <= hi).all()
    for _ in range(3):
        assert np.array_equal(orc.contour_cells(k["cells"]), ring)


def test_threshold_tiers(built, kats):
    # sparse_contour.rs:1243-1380
    k = kats["sparse_contour"]
    for mode, t, cm, sm in k["tiers"]:
        c, d, e, s = orc.contour_config(mode, t)
        b = k["base"][mode]
        assert abs(c - b[0] * cm) < 0.01 and abs(s - b[3] * sm) < 0.01
        assert (d, e) == (b[1], b[2])
    for mode in ("car", "bike", "foot", "truck", "bus"):
        prev = 0.0
        for t in (100, 600, 1200, 3600, 7200):
            c, d, e, s = orc.contour_config(mode, t)
            assert c > 0 and s >= prev
            prev = s


def test_mercator_round_trip(built):
    # sparse_contour.rs:1664-1671
    x, y = orc.mercator(50.8503, 4.3517)
    lon, lat = orc.inverse_mercator(x, y)
    assert abs(lat[0] - 50.8503) < 1e-9 and abs(lon[0] - 4.3517) < 1e-9


def test_ring_tracks_input_extent(built):
    # sparse_contour.rs:1592-1662: no morphology, 30 m cells at 50.8 N; the
    # ring's east-west extent is within 0.51 ground cells of the input
    lat, cell = 50.8, 30.0
    ground = cell * np.cos(np.radians(lat))
    m_per_deg = 6378137.0 * np.pi / 180.0 * np.cos(np.radians(lat))
    lon0 = 4.0
    lon1 = lon0 + 10.1 * ground / m_per_deg
    dlat = 1.5 * ground / 111320.0
    alat = lat - 0.25 * ground / 111320.0

    def seg(a, b, c, d):
        return [(int(a * 1e7), int(b * 1e7)), (int(c * 1e7), int(d * 1e7))]

    ring = orc.sparse_contour([seg(alat, lon0, alat, lon0), seg(lat, lon0, lat, lon1),
                               seg(lat + dlat, lon0, lat + dlat, lon1)], cell, 0, 0, 0.0)
    assert len(ring) >= 4
    half = 0.51 * ground / m_per_deg
    assert lon1 - half <= ring[:, 0].max() <= lon1 + half
    assert lon0 - half <= ring[:, 0].min() <= lon0 + half


def test_isochrone_geometry_pipeline(built):
    # build_isochrone_geometry_sparse on a small lattice of 2-point road
    # polylines: frontier roads are cut, the origin's component is returned
    rng = np.random.default_rng(3)
    rows, cols, step = 30, 30, 0.002
    lat0, lon0 = 50.80, 4.30
    pts, w, dist = [], [], []
    for r in range(rows):
        for c in range(cols - 1):
            a = (int((lat0 + r * step) * 1e7), int((lon0 + c * step) * 1e7))
            b = (int((lat0 + r * step) * 1e7), int((lon0 + (c + 1) * step) * 1e7))
            pts.append([a, b])
            w.append(int(rng.integers(50, 200)))
            dist.append(int(abs(r - rows // 2) * 150 + abs(c - cols // 2) * 150))
    off = np.zeros(len(pts) + 1, np.uint64)
    off[1:] = np.cumsum([len(p) for p in pts])
    poly = np.array([q for p in pts for q in p], np.int32)
    nodes = np.arange(len(pts), dtype=np.uint32)
    dist = np.array(dist, np.uint32)
    ring, cells, grid = orc.isochrone_geometry(nodes, dist, 1500, w, off, poly, "car")
    assert len(ring) >= 4 and len(cells) > 0
    o = np.array([lon0 + (cols // 2) * step, lat0 + (rows // 2) * step])
    assert ring[:, 0].min() < o[0] < ring[:, 0].max() and ring[:, 1].min() < o[1] < ring[:, 1].max()
    again = orc.isochrone_geometry(nodes, dist, 1500, w, off, poly, "car")
    assert np.array_equal(again[0], ring) and np.array_equal(again[1], cells)
    # a larger threshold reaches at least as many cells (coarser tier aside)
    _, cells2, _ = orc.isochrone_geometry(nodes, dist, 1400, w, off, poly, "car")
    assert len(cells2) <= len(cells)
