"""The host CCH pipeline: the contracted graph answers exactly like plain
Dijkstra on the edge-based graph (the validate-cch / validate-phast pattern of
route/src/validate/cch_correctness.rs:70 and route/src/range/mod.rs:728-818),
and it is deterministic across runs and machines (golden fingerprint)."""
import pathlib

import numpy as np
import pytest

from oracle import oracle as orc

INF = 0xFFFFFFFF


def _check_against_dijkstra(ebg, cch, n_src, seed):
    c = orc.Cch.from_dict(cch)
    rng = np.random.default_rng(seed)
    r2s, s2r = cch["rank_to_state"], cch["state_to_rank"]
    for s_state in rng.integers(0, ebg["n"], n_src):
        want = orc.dijkstra_ebg(ebg, int(s_state))
        got_by_rank = c.phast_query(int(s2r[s_state]))
        got = got_by_rank[s2r]  # back to state order
        assert np.array_equal(got, want), "CCH PHAST differs from Dijkstra"


def test_grid100_cch_equals_dijkstra(grid100):
    ebg, cch = grid100
    _check_against_dijkstra(ebg, cch, 12, 3)


def test_country_small_cch_equals_dijkstra(country_small):
    ebg, cch = country_small
    _check_against_dijkstra(ebg, cch, 6, 4)


def test_permutation_and_edge_directions(grid100):
    _, cch = grid100
    n = cch["n"]
    assert sorted(cch["rank_to_state"].tolist()) == list(range(n))
    assert np.array_equal(cch["state_to_rank"][cch["rank_to_state"]], np.arange(n))
    src_up = np.repeat(np.arange(n), np.diff(cch["up_off"].astype(np.int64)))
    src_dn = np.repeat(np.arange(n), np.diff(cch["down_off"].astype(np.int64)))
    assert (cch["up_tgt"] > src_up).all() and (cch["down_tgt"] < src_dn).all()
    assert (cch["up_w"] != INF).all() and (cch["down_w"] != INF).all()


def test_deterministic_and_golden_fingerprint(grid100):
    import cchbuild
    import sys
    sys.path.insert(0, str(pathlib.Path(__file__).parent / "golden"))
    from make_golden import fingerprint
    _, cch = grid100
    _, again = cchbuild.build_synthetic(cchbuild.KIND_GRID, 100, 100, seed=42, threads=3)
    assert fingerprint(cch) == fingerprint(again)
    g = np.load(pathlib.Path(__file__).parent / "golden" / "grid100_matrix.npz")
    assert int(g["n"]) == cch["n"]
    assert str(g["sha256"]) == fingerprint(cch)


def test_config_shape_grid100(grid100):
    ebg, cch = grid100
    assert ebg["n_intersections"] == 10000
    # 19800 lattice roads, 5% removed
    assert 18500 < ebg["n_roads"] < 19100
    assert cch["n"] == ebg["n"]


def test_hand_built_arcs():
    import cchbuild
    # a 4-state ring with a chord: arcs with weights
    src = [0, 1, 2, 3, 0]
    dst = [1, 2, 3, 0, 2]
    w = [5, 5, 5, 5, 12]
    ebg, cch = cchbuild.build_from_arcs(4, src, dst, w, [0, 1, 2, 3], [0, 0, 0, 0])
    c = orc.Cch.from_dict(cch)
    s2r = cch["state_to_rank"]
    for s in range(4):
        want = orc.dijkstra_ebg(ebg, s)
        assert np.array_equal(c.phast_query(int(s2r[s]))[s2r], want)


def test_invalid_params_rejected(built):
    import cchbuild
    with pytest.raises(RuntimeError):
        cchbuild.build_synthetic(7, 10, 10)
    with pytest.raises(RuntimeError):
        cchbuild.build_synthetic(cchbuild.KIND_GRID, 1, 10)
