"""bf_query_batch_noalloc — the entry point for callers that cannot allocate
memory (a process whose device memory is all reserved by its own pool, or a
hot path that cannot afford cudaMalloc's implicit synchronisation).

It must give exactly the distances of bf_query_batch (tolerance 0: u32
min-plus) on consecutive calls that share its static scratch array, and reject
requests beyond the scratch limit. Collected last so that a run stopping at
the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(g, d_src, k, threshold, d_out, stream):
    import bfphast
    return bfphast.load().bf_query_batch_noalloc(g.handle, ctypes.c_void_p(d_src), k, threshold,
                                                  ctypes.c_void_p(d_out),
                                                  ctypes.c_void_p(stream))


def test_noalloc_matches_query_batch_twice(built, grid100):
    import torch

    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    stream = torch.cuda.current_stream().cuda_stream
    calls = [(np.array([0, 17, 5000, 12345, 35723, 9, 9, 30000] + list(range(100, 124)),
                       dtype=np.uint32), bfphast.INF),
             (np.array([777, 20000, 3], dtype=np.uint32), 2500)]
    out = torch.empty(32 * n, dtype=torch.int32, device="cuda")
    for src, thr in calls:
        k = len(src)
        d_src = torch.from_numpy(src.view(np.int32)).cuda()
        out.fill_(-7)  # stale contents must not leak into the result
        rc = _noalloc(g, d_src.data_ptr(), k, thr, out.data_ptr(), stream)
        assert rc == bfphast.BF_OK, bfphast.load().bf_last_error()
        got = out[:k * n].view(k, n).cpu().numpy().view(np.uint32)
        want = g.query_batch(src, threshold=thr)
        assert np.array_equal(got, want)


def test_noalloc_rejects_beyond_limits(built, grid100):
    import torch

    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    d = torch.zeros(64, dtype=torch.int32, device="cuda")
    rc = _noalloc(g, d.data_ptr(), 33, bfphast.INF, d.data_ptr(), 0)
    assert rc == bfphast.BF_ERR_INVALID
    assert b"exceeds" in bfphast.load().bf_last_error()
