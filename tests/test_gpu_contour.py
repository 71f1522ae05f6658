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
