"""bf_query_batch_noalloc — the entry point for callers that cannot allocate
memory (a process whose device memory is all reserved by its own pool, or a
hot path that cannot afford cudaMalloc's implicit synchronisation).

It must give exactly the oracle's distances (tolerance 0: u32 min-plus) on
consecutive calls that share its static scratch array — including a call
right after one that filled the array with a much deeper ancestor path — and
the same distances as bf_query_batch; it must reject requests beyond the
scratch limit and out-of-range sources without spoiling the next call, and
run on a caller's own stream. Collected last so that a run stopping at the
first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _noalloc(g, d_src, k, threshold, d_out, stream):
    import bfphast
    return bfphast.load().bf_query_batch_noalloc(g.handle, ctypes.c_void_p(d_src), k, threshold,
                                                  ctypes.c_void_p(d_out),
                                                  ctypes.c_void_p(stream))


def _run(g, n, src, thr, stream=None):
    """One call through the C ABI; returns (status, k x n distances or None)."""
    import torch

    import bfphast
    k = len(src)
    st = torch.cuda.current_stream() if stream is None else stream
    with torch.cuda.stream(st):
        d_src = torch.from_numpy(np.asarray(src, dtype=np.uint32).view(np.int32)).cuda()
        out = torch.full((max(k, 1) * n,), -7, dtype=torch.int32, device="cuda")  # stale data
    st.synchronize()
    rc = _noalloc(g, d_src.data_ptr(), k, thr, out.data_ptr(), st.cuda_stream)
    if rc != bfphast.BF_OK:
        return rc, None
    return rc, out[:k * n].view(k, n).cpu().numpy().view(np.uint32)


def _chain(n):
    """Ranks 0..n-1 in a line: elimination-tree depth n - 1."""
    up_off = np.minimum(np.arange(n + 1), n - 1).astype(np.uint64)
    down_off = np.concatenate([[0], np.arange(n)]).astype(np.uint64)
    return dict(n=n, up_off=up_off, up_tgt=np.arange(1, n, dtype=np.uint32),
                up_w=(1 + np.arange(n - 1) % 7).astype(np.uint32), down_off=down_off,
                down_tgt=np.arange(0, n - 1, dtype=np.uint32),
                down_w=(2 + np.arange(n - 1) % 5).astype(np.uint32))


def _oracle(c, src, thr):
    # the oracle's query_batch takes at most K = 8 sources, like the reference's
    src = np.asarray(src, dtype=np.uint32)
    want = np.concatenate([c.query_batch(src[i:i + 8]) for i in range(0, len(src), 8)])
    return want if thr == INF else np.where(want <= thr, want, INF)


def test_noalloc_matches_oracle_twice(built, grid100, country_small):
    import bfphast
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    # a k = 0 call is the documented warm-up: no work, status OK
    assert _run(g, n, [], INF)[0] == bfphast.BF_OK
    calls = [([0, 17, 5000, 12345, 35723, 9, 9, 30000] + list(range(100, 124)), INF),
             ([777, 20000, 3], 2500)]
    for src, thr in calls:
        rc, got = _run(g, n, src, thr)
        assert rc == bfphast.BF_OK, bfphast.load().bf_last_error()
        assert np.array_equal(got, _oracle(c, src, thr))
        assert np.array_equal(got, g.query_batch(np.asarray(src, dtype=np.uint32),
                                                 threshold=thr))
    # the country graph: a full 32-source call, twice in a row
    _, cchc = country_small
    cc = orc.Cch.from_dict(cchc)
    gc = bfphast.Graph.from_cch(cchc)
    nc = cchc["n"]
    rng = np.random.default_rng(9)
    for thr in (INF, 4000):
        src = rng.choice(nc, 32, replace=False).astype(np.uint32)
        rc, got = _run(gc, nc, src, thr)
        assert rc == bfphast.BF_OK, bfphast.load().bf_last_error()
        assert np.array_equal(got, _oracle(cc, src, thr))


def test_noalloc_clean_after_deeper_path(built, grid100):
    """A chain 20 000 deep fills far more of the shared array than the grid's
    paths; the grid call that follows must not see any of it."""
    import bfphast
    N = 20000
    ch = _chain(N)
    gch = bfphast.Graph.from_cch(ch)
    cch_or = orc.Cch.from_dict(ch)
    src = [0, 1, 9999, N - 1]
    rc, got = _run(gch, N, src, INF)
    assert rc == bfphast.BF_OK, bfphast.load().bf_last_error()
    assert np.array_equal(got, _oracle(cch_or, src, INF))
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    src = list(range(5, 35723, 1151))[:32]
    rc, got = _run(g, cch["n"], src, INF)
    assert rc == bfphast.BF_OK, bfphast.load().bf_last_error()
    assert np.array_equal(got, _oracle(c, src, INF))


def test_noalloc_rejects_beyond_limits(built, grid100):
    import torch

    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    d = torch.zeros(64, dtype=torch.int32, device="cuda")
    rc = _noalloc(g, d.data_ptr(), 33, bfphast.INF, d.data_ptr(), 0)
    assert rc == bfphast.BF_ERR_INVALID
    assert b"exceeds" in bfphast.load().bf_last_error()
    # 27 sources on a 20 000-deep chain need 27 * 8 * 20 000 bytes > 4 MiB
    N = 20000
    gch = bfphast.Graph.from_cch(_chain(N))
    rc = _noalloc(gch, d.data_ptr(), 27, bfphast.INF, d.data_ptr(), 0)
    assert rc == bfphast.BF_ERR_INVALID
    assert b"scratch" in bfphast.load().bf_last_error()


def test_noalloc_bad_source_then_valid(built, grid100):
    """A source id beyond the graph is caught on the device; the next call works."""
    import bfphast
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    rc, _ = _run(g, n, [3, n + 5], INF)
    assert rc == bfphast.BF_ERR_INVALID
    src = [3, 4, 35000]
    rc, got = _run(g, n, src, INF)
    assert rc == bfphast.BF_OK, bfphast.load().bf_last_error()
    assert np.array_equal(got, _oracle(c, src, INF))


def test_noalloc_on_caller_stream(built, grid100):
    import torch

    import bfphast
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    st = torch.cuda.Stream()
    src = [11, 22, 33000, 17]
    for thr in (INF, 900):
        rc, got = _run(g, cch["n"], src, thr, stream=st)
        assert rc == bfphast.BF_OK, bfphast.load().bf_last_error()
        assert np.array_equal(got, _oracle(c, src, thr))
