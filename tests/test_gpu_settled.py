"""Bulk settled sets (bf_isochrone_settled) against the oracle's bounded
seeded query (run_phast_bounded_fast_seeded, isochrone_handler.rs:338-491)
and the single-origin entry point, bit for bit, on 16-bit and 32-bit
waves."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("thr_set", [(300, 900, 3000, 9000), (70000, 120000)])
def test_settled_match_oracle(built, grid100, thr_set):
    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    c = orc.Cch.from_dict(cch)
    rng = np.random.default_rng(len(thr_set))
    n = 70
    origins = rng.integers(0, cch["n"], n).astype(np.uint32)
    thr = rng.choice(np.array(thr_set, np.uint32), n)
    got = g.isochrone_settled(origins, thr)
    bits, counts = g.isochrone_bitsets(origins, thr)
    for i in range(n):
        wr, wd = c.bounded_seeded([(int(origins[i]), 0)], int(thr[i]))
        assert np.array_equal(got[i][0], wr) and np.array_equal(got[i][1], wd)
        assert len(got[i][0]) == counts[i]
    for i in (0, n - 1):
        sr, sd = g.phast_bounded_seeded([(int(origins[i]), 0)], int(thr[i]))
        assert np.array_equal(got[i][0], sr) and np.array_equal(got[i][1], sd)


def test_settled_country_small(built, country_small):
    import bfphast
    _, cch = country_small
    g = bfphast.Graph.from_cch(cch)
    c = orc.Cch.from_dict(cch)
    origins = np.array([0, 17, 4000, cch["n"] - 1, 4000], np.uint32)
    thr = np.array([18000, 6000, 36000, 3000, 0], np.uint32)
    got = g.isochrone_settled(origins, thr)
    for i in range(len(origins)):
        wr, wd = c.bounded_seeded([(int(origins[i]), 0)], int(thr[i]))
        assert np.array_equal(got[i][0], wr) and np.array_equal(got[i][1], wd)
