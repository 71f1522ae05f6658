"""Seeded reachable-segment sets for the contour tests: random walks of
(lat_e7, lon_e7) points around 50.8 N, 4.3 E (road-like steps of a few to a
few hundred metres), with an optional anchor."""
import numpy as np

from oracle import oracle as orc


def isochrone(rng, n_seg, spread=0.02):
    lat0, lon0 = 50.8 + rng.uniform(-0.1, 0.1), 4.3 + rng.uniform(-0.1, 0.1)
    segs = []
    for _ in range(n_seg):
        k = int(rng.integers(1, 6))
        lat = lat0 + rng.uniform(-spread, spread)
        lon = lon0 + rng.uniform(-spread, spread)
        pts = []
        for _ in range(k):
            pts.append((int(lat * 1e7), int(lon * 1e7)))
            lat += rng.normal(0, 0.0008)
            lon += rng.normal(0, 0.0012)
        segs.append(pts)
    anchor = None
    if rng.random() < 0.6:
        anchor = (int((lat0 + rng.uniform(-spread, spread)) * 1e7),
                  int((lon0 + rng.uniform(-spread, spread)) * 1e7))
    return segs, anchor


def mercator_segments(segs):
    """The segments' points projected exactly as the oracle projects them."""
    out = []
    for s in segs:
        a = np.asarray(s, np.float64)
        x, y = orc.mercator(a[:, 0] / 1e7, a[:, 1] / 1e7)
        out.append(np.stack([x, y], axis=1))
    return out


def mercator_point(p):
    x, y = orc.mercator(p[0] / 1e7, p[1] / 1e7)
    return (float(x[0]), float(y[0]))
