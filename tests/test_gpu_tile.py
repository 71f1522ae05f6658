"""Matrix tile emission on the GPU (bf_tile_emit, bf_tile_emit_device)
against the oracle's restatement of build_matrix_batch /
build_matrix_tile_batch (route/src/server/flight.rs:432-589): the
reference's fixtures, seeded random blocks (dense and sparse, radius masks,
time bounds, lat columns, saturating durations, ragged and empty shapes) and
the device-pointer variant; every column compared exactly."""
import json
import pathlib

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

MAX = orc.INF
KATS = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_kats.json").read_text())


@pytest.fixture(scope="module")
def bf():
    import bfphast
    bfphast.load()
    return bfphast


def same(a, b):
    return len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("name", ["small", "all_reachable", "noncontig", "tile", "radius",
                                  "all_sentinel", "pruned_empty", "tile_lat"])
@pytest.mark.parametrize("sparse", [False, True])
def test_reference_fixtures(bf, name, sparse):
    k = KATS["tile_emit"][name]
    args = (k["m"], len(k["src"]), len(k["dst"]), k["src"], k["dst"], k.get("threshold", MAX),
            k.get("mask"), k.get("lat"), sparse)
    assert same(bf.tile_emit(*args), orc.tile_emit(*args))


def random_case(rng, n_src, n_dst, with_mask, with_lat, p_max=0.2):
    m = rng.integers(0, 200_000, (n_src, n_dst), dtype=np.uint64).astype(np.uint32)
    m[rng.random((n_src, n_dst)) < p_max] = MAX
    m[rng.random((n_src, n_dst)) < 0.01] = 4_294_968  # saturates at 1000x
    src = rng.choice(3 * n_src + 5, n_src, replace=False).astype(np.uint32)
    dst = rng.choice(3 * n_dst + 5, n_dst, replace=False).astype(np.uint32)
    mask = None
    if with_mask:
        mask = [np.sort(rng.choice(3 * n_dst + 5, rng.integers(0, 3 * n_dst + 5), replace=False))
                .astype(np.uint32).tolist() for _ in range(3 * n_src + 5)]
    lat = rng.integers(0, 1 << 32, (n_src, n_dst), dtype=np.uint64).astype(np.uint32) \
        if with_lat else None
    return m, src, dst, mask, lat


@pytest.mark.parametrize("shape", [(0, 5), (5, 0), (1, 1), (1, 2049), (7, 333), (64, 97),
                                   (300, 1000), (16, 4096)])
@pytest.mark.parametrize("with_mask", [False, True])
def test_random_blocks(bf, shape, with_mask):
    rng = np.random.default_rng(sum(shape) * 7 + with_mask)
    n_src, n_dst = shape
    m, src, dst, mask, lat = random_case(rng, n_src, n_dst, with_mask, True)
    for sparse in (False, True):
        for thr in (MAX, 100_000):
            for la in (None, lat):
                args = (m, n_src, n_dst, src, dst, thr, mask, la, sparse)
                assert same(bf.tile_emit(*args), orc.tile_emit(*args)), (sparse, thr, la is None)


@pytest.mark.parametrize("n_dst", [4567, 4568])  # four-cell path when rows are a multiple of 4
def test_device_variant_matches_host(bf, n_dst):
    import torch
    rng = np.random.default_rng(5)
    n_src = 123
    m, src, dst, mask, lat = random_case(rng, n_src, n_dst, True, True)
    moff, mflat = orc.mask_csr(mask)
    dev = torch.device("cuda:0")
    t = lambda a, dt=torch.int32: torch.from_numpy(np.ascontiguousarray(a).view(
        np.int32 if dt == torch.int32 else np.int64)).to(dev)
    dm, dl, ds, dd = t(m.reshape(-1)), t(lat.reshape(-1)), t(src), t(dst)
    dmo, dmk = t(moff, torch.int64), t(mflat)
    cols = [torch.empty(n_src * n_dst, dtype=torch.int32, device=dev) for _ in range(4)]
    for sparse in (False, True):
        rows = bf.tile_emit_device(dm.data_ptr(), n_src, n_dst, ds.data_ptr(), dd.data_ptr(),
                                   [c.data_ptr() for c in cols], 150_000, dmo.data_ptr(),
                                   dmk.data_ptr(), len(mask), len(mflat), dl.data_ptr(), sparse)
        got = tuple(c[:rows].cpu().numpy().view(np.uint32) for c in cols)
        want = orc.tile_emit(m, n_src, n_dst, src, dst, 150_000, mask, lat, sparse)
        assert same(got, want)


def test_large_dense_and_sparse(bf):
    rng = np.random.default_rng(9)
    n_src, n_dst = 2500, 3001  # 7.5 M cells, several thousand blocks
    m, src, dst, _, _ = random_case(rng, n_src, n_dst, False, False, p_max=0.5)
    for sparse in (False, True):
        got = bf.tile_emit(m, n_src, n_dst, src, dst, 120_000, None, None, sparse)
        want = orc.tile_emit(m, n_src, n_dst, src, dst, 120_000, None, None, sparse)
        assert same(got, want)


def test_missing_radius_list_is_an_error(bf):
    with pytest.raises(bf.BfError, match="radius list"):
        bf.tile_emit([1, 2], 1, 2, [3], [0, 1], mask=[[0]])
    # the library stays usable afterwards
    assert same(bf.tile_emit([1, 2], 1, 2, [0], [0, 1], mask=[[1]], sparse=True),
                orc.tile_emit([1, 2], 1, 2, [0], [0, 1], mask=[[1]], sparse=True))


@pytest.mark.parametrize("n_dst,list_max,span", [(2048, 600, 0), (5000, 4096, 0),
                                                  (3000, 5000, 0), (3000, 2000, 400_000)])
def test_sparse_radius_lists_staged(bf, n_dst, list_max, span):
    """Sparse emission of wide rows (2048 cells or more: a block per row
    segment) with radius lists short enough (at most 4096 entries) to be
    searched in shared memory, including lists of exactly the staging limit
    and, for list_max 5000, rows whose list is too long, whose blocks search
    global memory; with span 400 000, destination ids beyond the shared
    bitmap's 2^17 ids, which are searched in the staged list."""
    rng = np.random.default_rng(n_dst + list_max)
    n_src = 37
    m, src, dst, _, lat = random_case(rng, n_src, n_dst, False, True)
    if span:
        dst = rng.choice(span, n_dst, replace=False).astype(np.uint32)
    else:
        span = 3 * n_dst + 5
    mask = []
    for r in range(3 * n_src + 5):
        k = list_max if r % 3 == 0 else int(rng.integers(0, list_max + 1))
        mask.append(np.sort(rng.choice(span, min(k, span), replace=False)).astype(np.uint32)
                    .tolist())
    for thr in (MAX, 100_000):
        args = (m, n_src, n_dst, src, dst, thr, mask, lat, True)
        assert same(bf.tile_emit(*args), orc.tile_emit(*args)), thr


def test_wide_rows_missing_radius_list_is_an_error(bf):
    """A wide row (a block per row segment) whose source has no radius list
    is an error whether or not the sparse form runs; the next call works."""
    rng = np.random.default_rng(21)
    n_src, n_dst = 3, 20000  # two segments per row
    m, src, dst, _, _ = random_case(rng, n_src, n_dst, False, False)
    src = np.array([0, 1, 5], dtype=np.uint32)  # original index 5 has no list
    mask = [[1, 2, 3], list(range(0, 60000, 7)), [4]]
    for sparse in (False, True):
        with pytest.raises(bf.BfError, match="radius list"):
            bf.tile_emit(m, n_src, n_dst, src, dst, MAX, mask, None, sparse)
    src = np.array([0, 1, 2], dtype=np.uint32)
    args = (m, n_src, n_dst, src, dst, 150_000, mask, None, True)
    assert same(bf.tile_emit(*args), orc.tile_emit(*args))
