"""Router cost model (phast_wins / update_cost_ewma, route/src/matrix/
bucket_ch.rs:6655-6712) through the C ABI. Host logic only: no GPU needed."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def lib(built):
    import bfphast
    return bfphast.load()


def _r():
    import bfphast
    return bfphast.Router(0, 0)


def test_structural_fallback(lib):
    # before both costs are measured: scan = n_nodes, sweep = clamp(n/400, 500, 20000)
    r = _r()
    n = 1_000_000                                                 # sweep = 2500
    assert lib.bf_router_phast_wins(ctypes.byref(r), 1, 1000, n, 0) == 1   # 1e6 < 1001*2500
    assert lib.bf_router_phast_wins(ctypes.byref(r), 3, 1000, n, 0) == 0   # 3e6 >= 1003*2500
    # n = 100: sweep clamps up to 500, 1 * 100 < 2 * 500
    assert lib.bf_router_phast_wins(ctypes.byref(r), 1, 1, 100, 0) == 1
    assert lib.bf_router_phast_wins(None, 1, 1, 100, 0) == 1
    # n = 1e9: sweep clamps down to 20000, 1e9 >= 2 * 20000
    assert lib.bf_router_phast_wins(ctypes.byref(r), 1, 1, 10**9, 0) == 0


def test_tall_shapes_and_override(lib):
    import bfphast
    r = _r()
    assert lib.bf_router_phast_wins(ctypes.byref(r), 10, 9, 100, bfphast.ROUTE_AUTO) == 0
    assert lib.bf_router_phast_wins(ctypes.byref(r), 10, 9, 100, bfphast.ROUTE_PHAST) == 0
    assert lib.bf_router_phast_wins(ctypes.byref(r), 9, 10, 10**9, bfphast.ROUTE_PHAST) == 1
    assert lib.bf_router_phast_wins(ctypes.byref(r), 1, 10**6, 10, bfphast.ROUTE_BUCKET) == 0


def test_ewma_updates(lib):
    import bfphast
    r = _r()
    lib.bf_router_observe(ctypes.byref(r), bfphast.COST_SWEEP, 1000)
    assert r.sweep_ns == 1000                       # first sample taken as is
    lib.bf_router_observe(ctypes.byref(r), bfphast.COST_SWEEP, 0)
    assert r.sweep_ns == 750                        # prev - prev/4 + sample/4
    lib.bf_router_observe(ctypes.byref(r), bfphast.COST_SWEEP, 2001)
    assert r.sweep_ns == 750 - 187 + 500
    lib.bf_router_observe(ctypes.byref(r), bfphast.COST_SCAN, 0)
    assert r.scan_ns == 1                           # never below 1
    lib.bf_router_observe(ctypes.byref(r), 7, 123)  # unknown cell: ignored
    assert (r.sweep_ns, r.scan_ns) == (1063, 1)


def test_measured_costs_decide(lib):
    import bfphast
    r = _r()
    lib.bf_router_observe(ctypes.byref(r), bfphast.COST_SCAN, 1000)
    # only one cost measured: still the structural bound
    assert lib.bf_router_phast_wins(ctypes.byref(r), 10, 100, 10**9, 0) == 0
    lib.bf_router_observe(ctypes.byref(r), bfphast.COST_SWEEP, 100)
    assert lib.bf_router_phast_wins(ctypes.byref(r), 10, 100, 10**9, 0) == 1   # 10000 < 11000
    assert lib.bf_router_phast_wins(ctypes.byref(r), 11, 100, 10**9, 0) == 1   # 11000 < 11100
    assert lib.bf_router_phast_wins(ctypes.byref(r), 12, 100, 10**9, 0) == 0   # 12000 >= 11200
    st = bfphast.Stats()
    st.n_sources, st.total_ms = 1000, 2.0           # one GPU call for 1000 fields: 2 us each
    r2 = _r()
    lib.bf_router_observe_stats(ctypes.byref(r2), ctypes.byref(st))
    assert r2.scan_ns == 2000
