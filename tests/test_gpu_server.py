"""Serving loop: continuous batching of mixed matrix / isochrone requests.

Every result must be identical alone (bf_matrix / bf_isochrone_bitsets) and
in the mix (tolerance 0: exact u32 min-plus). Failures are injected on the
host only (malformed requests, cancellation, a full queue)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _drain(srv, expected, timeout_s=60):
    done = {}
    t0 = time.time()
    while len(done) < expected and time.time() - t0 < timeout_s:
        for c in srv.poll(wait_ms=200):
            done[c["ticket"]] = c
    return done


def test_mixed_requests_equal_alone(built, grid100):
    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    rng = np.random.default_rng(5)
    srv = bfphast.Server(g, hbm_budget=4 << 30, max_inflight=8)
    reqs = []
    for i in range(30):
        if i % 3 == 2:
            o = int(rng.integers(0, n))
            thr = int(rng.choice([300, 1200, 3600, INF]))
            t, out = srv.submit_isochrone(o, thr, tag=i)
            reqs.append(("iso", t, out, o, thr))
        else:
            S, T = int(rng.integers(1, 200)), int(rng.integers(1, 200))
            src, tgt = rng.integers(0, n, S), rng.integers(0, n, T)
            thr = int(rng.choice([INF, 2000, 500]))
            t, out = srv.submit_matrix(src, tgt, thr, tag=i)
            reqs.append(("mat", t, out, (src, tgt), thr))
    done = _drain(srv, len(reqs))
    assert len(done) == len(reqs)
    for kind, t, out, args, thr in reqs:
        c = done[t]
        assert c["status"] == bfphast.BF_OK
        assert c["submit_s"] <= c["admit_s"] <= c["done_s"]
        if kind == "mat":
            alone = g.matrix(args[0], args[1], threshold=thr)
            assert np.array_equal(out, alone)
        else:
            bits, _ = g.isochrone_bitsets([args], [thr])
            assert np.array_equal(out, bits[0])
    srv.close()


def test_invalid_and_cancel(built, grid100):
    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    srv = bfphast.Server(g, hbm_budget=4 << 30)
    with pytest.raises(bfphast.BfError) as e:
        srv.submit_matrix([0, n], [1])
    assert e.value.status == bfphast.BF_ERR_INVALID
    tickets = [srv.submit_matrix(np.arange(64), np.arange(100, 400))[0] for _ in range(40)]
    rc = srv.cancel(tickets[-1])
    done = _drain(srv, len(tickets))
    assert len(done) == len(tickets)
    if rc == bfphast.BF_OK:
        assert done[tickets[-1]]["status"] == bfphast.BF_ERR_CANCELLED
    assert all(done[t]["status"] == bfphast.BF_OK for t in tickets[:-1])
    assert srv.cancel(10 ** 9) == bfphast.BF_ERR_INVALID
    srv.close()


def test_full_queue_is_busy(built, grid100):
    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    srv = bfphast.Server(g, hbm_budget=4 << 30, max_queue=2)
    accepted, busy = [], 0
    for _ in range(200):
        try:
            accepted.append(srv.submit_matrix(np.arange(300), np.arange(300))[0])
        except bfphast.BfError as e:
            assert e.status == bfphast.BF_ERR_BUSY
            busy += 1
    done = _drain(srv, len(accepted))
    assert len(done) == len(accepted)
    assert all(c["status"] == bfphast.BF_OK for c in done.values())
    assert busy + len(accepted) == 200
    srv.close()


def test_timeout_then_served(built, country_small):
    """A device wait bounded by 1 ms runs out on a large matrix: the request
    completes with BF_ERR_TIMEOUT after its slot drained; the graph then
    serves the same request exactly (a fresh server with the default bound)."""
    import bfphast
    _, cch = country_small
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    rng = np.random.default_rng(12)
    # 4000 x 20000 cells: a sweep of most of the graph for 4000 lanes and a
    # 320 MB read-back, far more than 1 ms of device work
    src, tgt = rng.integers(0, n, 4000), rng.integers(0, n, 20000)
    srv = bfphast.Server(g, hbm_budget=4 << 30, timeout_ms=1, slots=1)
    t, out = srv.submit_matrix(src, tgt)
    done = _drain(srv, 1)
    srv.close()
    assert done[t]["status"] == bfphast.BF_ERR_TIMEOUT
    srv = bfphast.Server(g, hbm_budget=4 << 30, slots=1)
    t, out = srv.submit_matrix(src, tgt)
    done = _drain(srv, 1)
    srv.close()
    assert done[t]["status"] == bfphast.BF_OK
    assert np.array_equal(out, g.matrix(src, tgt))


def test_admission_by_budget(built, grid100):
    """A request whose device I/O alone exceeds the server's I/O budget is
    refused at submission; requests that fit one at a time but not together
    are queued and all served exactly."""
    import bfphast
    _, cch = grid100
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    budget = 64 << 20  # 32 MiB for request I/O
    srv = bfphast.Server(g, hbm_budget=budget, slots=2)
    big = np.arange(3000, dtype=np.uint32)
    with pytest.raises(bfphast.BfError) as e:
        srv.submit_matrix(big, big)  # 36 MB of output alone
    assert e.value.status == bfphast.BF_ERR_BUSY
    rng = np.random.default_rng(2)
    reqs = []
    for i in range(6):  # ~20 MB of output each: at most one in flight at a time
        src, tgt = rng.integers(0, n, 2200), rng.integers(0, n, 2200)
        t, out = srv.submit_matrix(src, tgt, tag=i)
        reqs.append((t, out, src, tgt))
    done = _drain(srv, len(reqs), timeout_s=120)
    srv.close()
    assert len(done) == len(reqs)
    for t, out, src, tgt in reqs:
        assert done[t]["status"] == bfphast.BF_OK
        assert np.array_equal(out, g.matrix(src, tgt))
    # admissions never overlapped: each began after the previous one finished
    spans = sorted((done[t]["admit_s"], done[t]["done_s"]) for t, *_ in reqs)
    assert all(a2 >= d1 - 1e-3 for (_, d1), (a2, _) in zip(spans, spans[1:]))


def test_mixed_equal_alone_country_waves(built, country_small):
    """The country graph with a budget small enough that matrix batches run
    in several waves of lanes: every result equals the same request alone."""
    import bfphast
    _, cch = country_small
    g = bfphast.Graph.from_cch(cch)
    n = cch["n"]
    rng = np.random.default_rng(31)
    srv = bfphast.Server(g, hbm_budget=256 << 20, max_inflight=8, slots=2)
    reqs = []
    for i in range(16):
        if i % 4 == 3:
            o = int(rng.integers(0, n))
            thr = int(rng.choice([3000, 12000, 36000]))
            t, out = srv.submit_isochrone(o, thr, tag=i)
            reqs.append(("iso", t, out, o, thr))
        else:
            S, T = int(rng.integers(200, 1500)), int(rng.integers(100, 800))
            src, tgt = rng.integers(0, n, S), rng.integers(0, n, T)
            thr = int(rng.choice([INF, 9000]))
            t, out = srv.submit_matrix(src, tgt, thr, tag=i)
            reqs.append(("mat", t, out, (src, tgt), thr))
    done = _drain(srv, len(reqs), timeout_s=120)
    srv.close()
    assert len(done) == len(reqs)
    for kind, t, out, args, thr in reqs:
        assert done[t]["status"] == bfphast.BF_OK
        if kind == "mat":
            assert np.array_equal(out, g.matrix(args[0], args[1], threshold=thr))
        else:
            bits, _ = g.isochrone_bitsets([args], [thr])
            assert np.array_equal(out, bits[0])
