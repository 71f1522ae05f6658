"""Persistent sweeps (one cooperative launch walking every level, grid
barriers between levels) against the per-level launches and the oracle
(tolerance 0: u32 min-plus), and the grid barrier's deadline.

The deadline is tested without faulting anything: the test hook
BF_TEST_WITHHOLD_ARRIVAL makes the persistent sweep run on two blocks of
which block 1 leaves before its first barrier arrival; block 0's wait runs
out after about a millisecond, it sets the error flag and returns, and the
call reports BF_ERR_TIMEOUT. The next call without the hook must be exact."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


@pytest.mark.parametrize("which", ["grid100", "country_small"])
def test_plain_persistent_matches_levels(built, grid100, country_small, which):
    import bfphast
    _, cch = grid100 if which == "grid100" else country_small
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    g.set_engine(bfphast.ENGINE_PLAIN)
    rng = np.random.default_rng(4)
    src = rng.choice(n, 70, replace=False).astype(np.uint32)  # three K = 32 batches
    tgt = rng.choice(n, 500, replace=False).astype(np.uint32)
    want, _ = c.matrix(src, tgt)
    for persist in (1, 0):
        g.set_tune(persistent_sweep=persist)
        got, st = g.matrix(src, tgt, stats=True)
        assert np.array_equal(got, want), persist
        if persist:  # one sweep launch per batch (+ upward and extraction)
            assert st["kernel_launches"] == 3 * 3 + 1  # + target positions
        for thr in (0, 2000):
            m = g.matrix(src, tgt, threshold=thr)
            assert np.array_equal(m, np.where(want <= thr, want, INF)), (persist, thr)


@pytest.mark.parametrize("lanes", [8, 64, 128, 256, 1024])
def test_isochrone_persistent_matches_oracle(built, country_small, lanes):
    import bfphast
    import workload
    _, cch = country_small
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    origins, thr = workload.isochrone_workload(cch["n"], min(lanes, 96) + 5, seed=lanes)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr)
    for persist in (3, 1):  # bit 1: isochrone waves in one persistent launch
        g.set_tune(isochrone_lanes=lanes if lanes >= 32 else 32, persistent_sweep=persist)
        bits, counts = g.isochrone_bitsets(origins, thr)
        assert np.array_equal(bits, want_bits), persist
        assert np.array_equal(counts, want_counts), persist


def test_barrier_deadline_reports_timeout(built, grid100):
    import bfphast
    _, cch = grid100
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    src = np.array([3, 1000, 30000], dtype=np.uint32)
    tgt = np.arange(0, n, 7, dtype=np.uint32)
    # 200 origins in one 256-lane wave: item slots of one warp, so the
    # grid100 levels above 32 items are grid segments with barriers
    origins = np.arange(0, n, n // 200, dtype=np.uint32)[:200]
    thr = np.full(200, 3000, dtype=np.uint32)
    g.set_tune(isochrone_lanes=256, persistent_sweep=3)
    g.set_engine(bfphast.ENGINE_PLAIN)
    os.environ["BF_TEST_WITHHOLD_ARRIVAL"] = "1"
    try:
        with pytest.raises(bfphast.BfError) as e:
            g.matrix(src, tgt)
        assert e.value.status == bfphast.BF_ERR_TIMEOUT
        with pytest.raises(bfphast.BfError) as e:
            g.isochrone_bitsets(origins, thr)
        assert e.value.status == bfphast.BF_ERR_TIMEOUT
    finally:
        del os.environ["BF_TEST_WITHHOLD_ARRIVAL"]
    want, _ = c.matrix(src, tgt)
    assert np.array_equal(g.matrix(src, tgt), want)
    bits, _ = g.isochrone_bitsets(origins, thr)
    wb, _ = c.isochrone_bitsets(origins, thr)
    assert np.array_equal(bits, wb)


def test_isochrone_autotune_and_tune_cache(built, country_small, tmp_path):
    """bf_autotune_isochrones keeps the fastest wave form; the tune cache
    restores it on the same graph and refuses another graph's."""
    import torch

    import bfphast
    import workload
    _, cch = country_small
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    origins, thr = workload.isochrone_workload(cch["n"], 600, seed=17)
    d_o = torch.from_numpy(origins.view(np.int32)).cuda()
    d_t = torch.from_numpy(thr.view(np.int32)).cuda()
    best = g.autotune_isochrones(d_o.data_ptr(), d_t.data_ptr(), len(origins), reps=1)
    assert best["tried"] >= 2 and best["isochrone_lanes"] in (256, 512, 1024, 2048)
    bits, counts = g.isochrone_bitsets(origins[:50], thr[:50])
    wb, wc = c.isochrone_bitsets(origins[:50], thr[:50])
    assert np.array_equal(bits, wb) and np.array_equal(counts, wc)
    path = tmp_path / "tune.json"
    g.tune_save(path)
    h = bfphast.Graph.from_cch(cch)
    h.tune_load(path)
    got = h.get_tune()
    for k in ("isochrone_lanes", "persistent_sweep", "threads_per_block", "edges_per_item"):
        assert got[k] == best[k], k
    _, other = (None, _chain_like())
    o = bfphast.Graph.from_cch(other)
    with pytest.raises(bfphast.BfError) as e:
        o.tune_load(path)
    assert e.value.status == bfphast.BF_ERR_INVALID


def _chain_like():
    n = 64
    up_off = np.minimum(np.arange(n + 1), n - 1).astype(np.uint64)
    down_off = np.concatenate([[0], np.arange(n)]).astype(np.uint64)
    return dict(n=n, up_off=up_off, up_tgt=np.arange(1, n, dtype=np.uint32),
                up_w=np.ones(n - 1, np.uint32), down_off=down_off,
                down_tgt=np.arange(0, n - 1, dtype=np.uint32), down_w=np.ones(n - 1, np.uint32))


def test_schedule_peeling_deadline_reports_timeout(built, grid100):
    """The device schedule builder's peeling rounds run in one cooperative
    launch; with the hook, block 1 leaves before its first barrier arrival,
    block 0's wait runs out, and the matrix call reports BF_ERR_TIMEOUT. Rows
    are only ever removed when nothing reads them, so the schedule left is a
    correct superset: the next calls, with and without the hook's targets,
    are exact."""
    import bfphast
    _, cch = grid100
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    g.set_tune(device_schedule=1)
    src = np.array([3, 1000, 30000, 17], dtype=np.uint32)
    tgt = np.arange(5, n, 97, dtype=np.uint32)
    os.environ["BF_TEST_WITHHOLD_ARRIVAL"] = "1"
    try:
        with pytest.raises(bfphast.BfError) as e:
            g.matrix(src, tgt)
        assert e.value.status == bfphast.BF_ERR_TIMEOUT
    finally:
        del os.environ["BF_TEST_WITHHOLD_ARRIVAL"]
    want, _ = c.matrix(src, tgt)
    assert np.array_equal(g.matrix(src, tgt), want)
    tgt2 = np.arange(11, n, 89, dtype=np.uint32)
    want2, _ = c.matrix(src, tgt2)
    assert np.array_equal(g.matrix(src, tgt2), want2)
