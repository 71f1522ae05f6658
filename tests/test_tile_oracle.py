"""The tile-emission oracle against the reference's matrix_sparse_tests
(route/src/server/flight.rs:4976-5380), transcribed in
tests/golden/reference_kats.json."""
import json
import pathlib

import numpy as np
import pytest

from oracle import oracle as orc

MAX = orc.INF
KATS = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_kats.json").read_text())
T = KATS["tile_emit"]


def emit(k, sparse, threshold=MAX, mask=True, lat=False):
    return orc.tile_emit(k["m"], len(k["src"]), len(k["dst"]), k["src"], k["dst"], threshold,
                         k.get("mask") if mask else None, k.get("lat") if lat else None, sparse)


def rows(cols):
    return sorted(zip(*[c.tolist() for c in cols]))


def test_small_dense_full_grid():  # I1
    s, t, du, di = emit(T["small"], False)
    assert len(s) == T["small"]["dense_rows"]
    assert int((du == MAX).sum()) == T["small"]["dense_sentinels"]


def test_small_sparse_equals_dense_minus_sentinels():  # I2, I3, I4
    k = T["small"]
    s, t, du, di = emit(k, True)
    assert [list(r[:3]) for r in rows((s, t, du))] == k["sparse"]
    dense = emit(k, False)
    assert len(s) == int((dense[2] != MAX).sum())
    assert (du != MAX).all() and (di == MAX).all()


def test_small_distance_with_lat():  # I5
    k = T["small"]
    s, t, du, di = emit(k, True, lat=True)
    assert [list(r) for r in rows((s, t, di))] == k["sparse_lat"]


def test_small_no_mask_drops_only_unreachable():  # I6
    s, t, du, di = emit(T["small"], True, mask=False)
    assert [list(r) for r in rows((s, t))] == T["small"]["no_mask_sparse_pairs"]


def test_all_reachable_sparse_equals_dense():  # I7-I8
    k = T["all_reachable"]
    dense, sparse = emit(k, False), emit(k, True)
    assert all(np.array_equal(a, b) for a, b in zip(dense, sparse)) and len(dense[0]) == k["rows"]
    s, _, _, _ = emit(T["all_sentinel"], True)
    assert len(s) == 0


def test_original_indices_preserved():  # I9
    k = T["noncontig"]
    s, t, du, _ = emit(k, True)
    assert [list(r) for r in rows((s, t, du))] == k["sparse"]


def test_tile_dense_and_sparse():  # T1, T2
    k = T["tile"]
    s, t, du, di = emit(k, False, k["threshold"])
    assert len(s) == k["dense_rows"] and int((du == MAX).sum()) == k["dense_sentinels"]
    assert (di == MAX).all()
    s, t, du, di = emit(k, True, k["threshold"])
    assert [list(r) for r in rows((s, t, du))] == k["sparse"]


def test_tile_threshold_gates_cells():  # T3
    k = T["tile"]
    s, t, _, _ = emit(k, True, MAX, mask=False)
    assert [list(r) for r in rows((s, t))] == k["unbounded_pairs"]
    s, t, _, _ = emit(k, True, 500, mask=False)
    assert not any(a == 3 and b == 4 for a, b in zip(s, t))


def test_tile_radius_prunes_reachable_and_empty_tiles():  # T4, T5, T6
    k = T["radius"]
    assert [list(r) for r in rows(emit(k, True)[:3])] == k["sparse"]
    assert len(emit(T["all_sentinel"], True)[0]) == 0
    assert len(emit(T["pruned_empty"], True)[0]) == 0
    s, t, du, di = emit(T["all_sentinel"], False)
    assert len(s) == 4 and (du == MAX).all() and (di == MAX).all()


def test_tile_lat_distance():  # tile_emits_lat_as_distance_when_present, tile_distance_max_without_lat
    k = T["tile_lat"]
    s, t, du, di = emit(k, False, lat=True)
    assert [list(r) for r in zip(t.tolist(), du.tolist(), di.tolist())] == k["rows"]
    assert (emit(k, False)[3] == MAX).all()


def test_saturation_and_missing_mask_row():
    s, t, du, di = orc.tile_emit([4294967, 4294968, MAX - 1], 1, 3, [0], [0, 1, 2], sparse=True)
    assert du.tolist() == [4294967000, MAX, MAX]  # u32::saturating_mul(1000)
    with pytest.raises(IndexError):
        orc.tile_emit([1], 1, 1, [3], [0], mask=[[0]])


def _numpy_emit(m, n_src, n_dst, src, dst, threshold, mask, lat, sparse):
    """An independent vectorised statement of the same rules."""
    m = np.asarray(m, np.uint64).reshape(n_src, n_dst)
    src, dst = np.asarray(src, np.uint64), np.asarray(dst, np.uint64)
    d = m.copy()
    if mask is not None:
        keep = np.array([[int(t) in set(mask[int(s)]) for t in dst] for s in src], bool).reshape(
            n_src, n_dst)
        d[~keep] = MAX
    d[(d > threshold) & (d != MAX)] = MAX
    s_col = np.repeat(src, n_dst).reshape(n_src, n_dst)
    t_col = np.tile(dst, n_src).reshape(n_src, n_dst)
    dur = np.where(d == MAX, MAX, np.minimum(d * 1000, MAX))
    dist = np.full((n_src, n_dst), MAX, np.uint64)
    if lat is not None:
        dist = np.where(d == MAX, MAX, np.asarray(lat, np.uint64).reshape(n_src, n_dst))
    sel = (d != MAX) if sparse else np.ones_like(d, bool)
    return tuple(a[sel].astype(np.uint32) for a in (s_col, t_col, dur, dist))


@pytest.mark.parametrize("seed", range(6))
def test_oracle_against_numpy_restatement(seed):
    rng = np.random.default_rng(seed)
    n_src, n_dst = int(rng.integers(0, 9)), int(rng.integers(0, 13))
    m = rng.integers(0, 9_000_000, n_src * n_dst).astype(np.uint32)
    m[rng.random(n_src * n_dst) < 0.25] = MAX
    src = rng.choice(20, n_src, replace=False).astype(np.uint32)
    dst = rng.choice(30, n_dst, replace=False).astype(np.uint32)
    mask = [sorted(rng.choice(30, int(rng.integers(0, 30)), replace=False).tolist())
            for _ in range(20)] if seed % 2 else None
    lat = rng.integers(0, 1 << 32, n_src * n_dst, dtype=np.uint64).astype(np.uint32) \
        if seed % 3 else None
    for sparse in (False, True):
        for thr in (MAX, 5_000_000):
            got = orc.tile_emit(m, n_src, n_dst, src, dst, thr, mask, lat, sparse)
            want = _numpy_emit(m, n_src, n_dst, src, dst, thr, mask, lat, sparse)
            assert all(np.array_equal(a, b) for a, b in zip(got, want))
