"""Bulk isochrone reachable sets on the GPU vs the CPU oracle (bit-exact).

Oracle: run_phast_bounded_fast_seeded (isochrone_handler.rs:338-491); bit r of
origin i's row is set iff rank r is settled with dist <= T_i."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _graph(cch):
    import bfphast
    return bfphast.Graph.from_cch(cch)


def test_grid100_bitsets_match_oracle(built, grid100):
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    n = cch["n"]
    origins = np.array([0, 1, 77, 5000, 12345, 20000, n - 1, 77, 31000, 4242], dtype=np.uint32)
    thr = np.array([0, 300, 1200, 3000, 6000, 18000, 36000, INF, 900, 1], dtype=np.uint32)
    bits, counts = g.isochrone_bitsets(origins, thr)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr, threads=4)
    assert np.array_equal(bits, want_bits)
    assert np.array_equal(counts, want_counts)
    assert counts[0] == 1  # threshold 0: only the origin itself


def test_country_small_bitsets_match_oracle(built, country_small):
    import workload
    _, cch = country_small
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    origins, thr = workload.isochrone_workload(cch["n"], 45, seed=3)
    bits, counts = g.isochrone_bitsets(origins, thr)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr)
    assert np.array_equal(bits, want_bits)
    assert np.array_equal(counts, want_counts)


def test_bitsets_device_variant_and_popcount(built, grid100):
    import torch
    _, cch = grid100
    g = _graph(cch)
    n = cch["n"]
    origins = np.arange(0, n, 997, dtype=np.uint32)
    thr = np.full(len(origins), 2500, dtype=np.uint32)
    bits, counts = g.isochrone_bitsets(origins, thr)
    w64 = (n + 63) // 64
    d_o = torch.from_numpy(origins.view(np.int32)).cuda()
    d_t = torch.from_numpy(thr.view(np.int32)).cuda()
    d_b = torch.zeros(len(origins) * w64, dtype=torch.int64, device="cuda")
    d_c = torch.zeros(len(origins), dtype=torch.int64, device="cuda")
    g.isochrone_bitsets_device(d_o.data_ptr(), d_t.data_ptr(), len(origins), d_b.data_ptr(),
                               d_c.data_ptr())
    assert np.array_equal(d_b.cpu().numpy().view(np.uint64).reshape(len(origins), w64), bits)
    assert np.array_equal(d_c.cpu().numpy().view(np.uint64), counts)
    pop = np.array([int(np.unpackbits(r.view(np.uint8)).sum()) for r in bits])
    assert np.array_equal(pop, counts)


def test_bitsets_empty_and_invalid(built, grid100):
    import bfphast
    _, cch = grid100
    g = _graph(cch)
    bits, counts = g.isochrone_bitsets(np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    assert bits.shape[0] == 0 and counts.shape == (0,)
    with pytest.raises(bfphast.BfError):
        g.isochrone_bitsets([cch["n"]], [100])


@pytest.mark.parametrize("iso_lanes", [32, 64, 0])
def test_wave_widths_match_oracle(built, country_small, iso_lanes):
    import workload
    _, cch = country_small
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    g.set_tune(isochrone_lanes=iso_lanes)
    origins, thr = workload.isochrone_workload(cch["n"], 150, seed=17)
    bits, counts = g.isochrone_bitsets(origins, thr)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr)
    assert np.array_equal(bits, want_bits)
    assert np.array_equal(counts, want_counts)


@pytest.mark.parametrize("half", [1, 0])
def test_16bit_and_32bit_lanes_match_oracle(built, country_small, half):
    # thresholds below 0xFFFF take the clamped 16-bit lanes unless disabled
    import workload
    _, cch = country_small
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    g.set_tune(isochrone_lanes=64, isochrone_16bit=half)
    origins, thr = workload.isochrone_workload(cch["n"], 130, seed=23)
    bits, counts = g.isochrone_bitsets(origins, thr)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr)
    assert np.array_equal(bits, want_bits)
    assert np.array_equal(counts, want_counts)


def test_16bit_boundary_thresholds(built, grid100):
    # 0xFFFE is the largest threshold the 16-bit lanes hold; 0xFFFF and above
    # run on 32-bit lanes. Both must agree with the oracle.
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    origins = np.array([3, 400, 9000, 22222, 35000, 7], dtype=np.uint32)
    for t in (0xFFFE, 0xFFFF, 0x10000):
        thr = np.full(len(origins), t, dtype=np.uint32)
        thr[0] = 50
        bits, counts = g.isochrone_bitsets(origins, thr)
        want_bits, want_counts = c.isochrone_bitsets(origins, thr)
        assert np.array_equal(bits, want_bits) and np.array_equal(counts, want_counts)


@pytest.mark.parametrize("lanes", [64, 256, 1024])
def test_staged_levels_match_oracle(built, country_small, lanes):
    """Runs of small levels whose items and edge records are bulk-copied into
    shared memory give the oracle's bitsets, like the global-memory form."""
    import workload
    _, cch = country_small
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    origins, thr = workload.isochrone_workload(cch["n"], min(lanes, 96) + 3, seed=lanes + 1)
    want_bits, want_counts = c.isochrone_bitsets(origins, thr)
    for staged in (1, 0):
        g.set_tune(isochrone_lanes=lanes, staged_levels=staged)
        bits, counts = g.isochrone_bitsets(origins, thr)
        assert np.array_equal(bits, want_bits), staged
        assert np.array_equal(counts, want_counts), staged
