"""Writes the golden fixtures under tests/golden/.

reference_kats.json
    Known-answer vectors transcribed from the reference's own unit tests
    (paths relative to the butterfly-osm repository):
      * route/src/range/phast.rs:1180-1250   5-node CCH (build_test_cch) and
        its forward / reverse results (test_reverse_phast_simple :1255-1390,
        test_reverse_phast_bounded :1420-1445)
      * route/src/range/phast.rs:1447-1560   asymmetric 3-node CCH
        (test_reverse_phast_asymmetric)
      * route/src/matrix/bucket_ch.rs:4855-4905  4-node CCH with INF entries
        (make_cch) — 3 finite UP and 3 finite DOWN edges survive the flats
      * route/src/matrix/bucket_ch.rs:5619-5700  broom graph, closed-form
        matrix d(s,t) = wu[s] + wd[t] (0 on the diagonal) with the bounded
        thresholds the tests sweep (:5721-5760)
      * route/src/server/isochrone_handler.rs:1806-1869  two-channel
        lexicographic tie (phast_2ch_lex_tests): two equal-time paths to node
        3, the shorter length must win whichever path pops first
      * route/src/customization.rs:2269-2487  CCH customization on a
        4-node directed topology (topo_4node): a shortcut 2 -> 3 expanded
        through external middle 0 or 1 (lengths 13 and 105), the packed
        (weight, middle) order, and the three (time, length) lexicographic
        middle elections
      * route/src/server/flight.rs:4976-5380  matrix RecordBatch emission
        (matrix_sparse_tests): the small-path and tile fixtures, radius
        masks, the time bound, sparse dropping, non-contiguous original
        indices, all-sentinel blocks and the lat (distance) column
      * route/src/range/sparse_contour.rs:1187-1672  isochrone contour:
        cell-centre rings of a 3x3 block and an L-shape, anchored component
        selection, the largest component without an anchor, and the
        threshold tiers of SparseContourConfig

grid100_matrix.npz
    The 100 x 100 matrix of the 100 x 100 synthetic grid computed by the CPU
    oracle (a restatement of compute_matrix_flat_soa) with the seeded
    sources/targets of workload.sources_targets, plus a fingerprint of the
    contracted graph so drift of the build pipeline between machines is
    caught. Regenerate with:  python tests/golden/make_golden.py
"""
import hashlib
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "butterfly-osm_gb300"))
sys.path.insert(0, str(ROOT))

INF = 0xFFFFFFFF


def kats():
    broom = {}
    for n_leaf in (5, 12):
        wu = [(i + 1) * 10 for i in range(n_leaf)]
        wd = [i + 1 for i in range(n_leaf)]
        n = n_leaf + 1
        up_off = [min(i, n_leaf) for i in range(n + 1)]
        down_off = [0] * (n_leaf + 1) + [n_leaf]
        expect = [[0 if s == t else wu[s] + wd[t] for t in range(n_leaf)] for s in range(n_leaf)]
        broom[str(n_leaf)] = dict(
            cch=dict(n=n, up_off=up_off, up_tgt=[n_leaf] * n_leaf, up_w=wu, down_off=down_off,
                     down_tgt=list(range(n_leaf)), down_w=wd),
            expect=expect,
            thresholds=[0, 15, 25, 55, 1000] if n_leaf == 5 else [0, 30, 75, 130, 100000])
    four = dict(n=4, up_off=[0, 1, 2, 3, 3], up_tgt=[3, 3, 3], up_short=[0, 0, 1],
                up_mid=[INF, INF, 0], down_off=[0, 0, 0, 2, 2], down_tgt=[0, 1],
                down_short=[0, 0], down_mid=[INF, INF])
    customize = {
        "source": "route/src/customization.rs:2269-2487",
        "topo": four,
        # shortcut_len_along_time_follows_the_time_optimal_middle (:2302-2350):
        # original lengths 0->3 = 10, 1->3 = 100, 2->0 = 3, 2->1 = 5
        "bottom_up": [dict(orig_up=[10, 100, 0], orig_down=[3, 5], up_mid=[INF, INF, m],
                           down_mid=[INF, INF], up=[10, 100, want], down=[3, 5])
                      for m, want in ((0, 13), (1, 105))],
        # pack_wm_is_a_bijection_and_orders_by_weight_then_middle (:2352-2371)
        "pack_order": [[[10, INF], [11, 0]], [[10, 3], [10, 4]]],
        # lex_election_* (:2420-2487): seeds (time, length) per edge, the
        # shortcut's converged time and elected middle
        "lex": [
            dict(up_t=[7, 5, 10], down_t=[3, 5], up_l=[10, 100, 105], down_l=[3, 5],
                 time=10, middle=0),
            dict(up_t=[5, 5, 10], down_t=[5, 5], up_l=[100, 10, 999], down_l=[5, 3],
                 time=10, middle=1),
            dict(up_t=[7, 5, 999], down_t=[3, 5], up_l=[6, 6, 999], down_l=[4, 4],
                 time=10, middle=0),
        ],
    }
    block3 = [[c, r] for r in range(3) for c in range(3)]
    strip = [[0, 0], [1, 0], [0, 1], [1, 1]] + [[c, r] for c in range(10, 40) for r in range(10, 13)]
    contour = {
        "source": "route/src/range/sparse_contour.rs:1187-1672",
        # test_center_emission_square_block (:1453-1481): half-cell units
        "block3": {"cells": block3, "ring_half_cells": [[1, 1], [3, 1], [5, 1], [5, 3], [5, 5],
                                                        [3, 5], [1, 5], [1, 3]]},
        # test_center_emission_l_shape_dedup (:1505-1528)
        "l_shape": {"cells": [[0, 0], [1, 0], [0, 1]], "ring_half_cells": [[1, 1], [3, 1], [1, 3]]},
        # anchored_extraction_prefers_origin_component (:1421-1451)
        "anchored": {"cells": strip, "origin": [1.0, 1.0], "inside_big": [20.0, 11.5],
                     "outside": [100.0, 100.0]},
        # test_largest_component_wins (:1555-1576)
        "largest": {"cells": [[c, r] for r in range(5) for c in range(5)]
                    + [[300, 300], [301, 300], [300, 301], [301, 301]], "bbox": [0.0, 5.0]},
        # test_adaptive_* (:1243-1380): (mode, threshold_s) -> cell and
        # simplification multipliers of the mode's base config
        "tiers": [["car", 300, 1.0, 1.0], ["car", 600, 1.0, 1.0], ["car", 601, 2.0, 2.0],
                  ["car", 1800, 2.0, 2.0], ["car", 3600, 4.0, 4.0], ["car", 7200, 6.67, 8.0]],
        "base": {"car": [30.0, 2, 2, 30.0], "bike": [40.0, 3, 3, 40.0], "foot": [25.0, 3, 3, 25.0],
                 "truck": [30.0, 2, 2, 30.0]},
    }
    MAX = INF
    tile_emit = {
        "source": "route/src/server/flight.rs:4976-5380",
        # small_fixture (:5002-5015): rows are (source, target, duration_ms[, distance_m])
        "small": dict(m=[100, MAX, 300, MAX, 200, 250], src=[0, 1], dst=[0, 1, 2],
                      mask=[[0, 2], [1]], lat=[1100, MAX, 3300, MAX, 2200, 2500],
                      dense_rows=6, dense_sentinels=3,
                      sparse=[[0, 0, 100000], [0, 2, 300000], [1, 1, 200000]],
                      sparse_lat=[[0, 0, 1100], [0, 2, 3300], [1, 1, 2200]],
                      no_mask_sparse_pairs=[[0, 0], [0, 2], [1, 1], [1, 2]]),
        # small_no_sentinels_sparse_equals_dense (:5123-5133)
        "all_reachable": dict(m=[10, 20, 30, 40, 50, 60], src=[0, 1], dst=[0, 1, 2], rows=6),
        # small_original_indices_preserved (:5138-5150)
        "noncontig": dict(m=[70, MAX, MAX, 90], src=[2, 5], dst=[1, 4],
                          sparse=[[2, 1, 70000], [5, 4, 90000]]),
        # tile_fixture (:5168-5180), threshold 500
        "tile": dict(m=[50, MAX, 300, MAX, 120, 999], src=[0, 3], dst=[1, 2, 4],
                     mask=[[1, 2, 4], [], [], [2, 4]], threshold=500, dense_rows=6,
                     dense_sentinels=3,
                     sparse=[[0, 1, 50000], [0, 4, 300000], [3, 2, 120000]],
                     unbounded_pairs=[[0, 1], [0, 4], [3, 2], [3, 4]]),
        # tile_radius_mask_prunes_reachable (:5240-5262)
        "radius": dict(m=[40, 80], src=[0], dst=[1, 2], mask=[[2]], sparse=[[0, 2, 80000]]),
        # tile_sparse_all_sentinels_is_none (:5264-5285)
        "all_sentinel": dict(m=[MAX] * 4, src=[0, 1], dst=[0, 1]),
        "pruned_empty": dict(m=[10, 20], src=[0], dst=[0, 1], mask=[[]]),
        # tile_emits_lat_as_distance_when_present (:5340-5355)
        "tile_lat": dict(m=[50, 100], lat=[700, 1400], src=[0], dst=[0, 1],
                         rows=[[0, 50000, 700], [1, 100000, 1400]]),
    }
    return {
        "tile_emit": tile_emit,
        "sparse_contour": contour,
        "cch_customize": customize,
        "five_node": {
            "source": "route/src/range/phast.rs:1180-1250",
            "cch": dict(n=5, up_off=[0, 1, 2, 4, 4, 4], up_tgt=[2, 2, 3, 4], up_w=[10, 3, 7, 5],
                        down_off=[0, 0, 0, 2, 3, 4], down_tgt=[0, 1, 2, 2],
                        down_w=[10, 3, 7, 5]),
            "fwd": {"0": [0, 13, 10, 17, 15]},
            "rev": {"0": [0, 13, 10, 17, 15]},
            "rev_bounded_count": {"target": 0, "threshold": 12, "count": 2},
        },
        "asym_three_node": {
            "source": "route/src/range/phast.rs:1447-1560",
            "cch": dict(n=3, up_off=[0, 1, 2, 2], up_tgt=[2, 2], up_w=[10, 5],
                        down_off=[0, 0, 0, 2], down_tgt=[0, 1], down_w=[20, 3]),
            "fwd": {"0": [0, 13, 10], "1": [25, 0, 5], "2": [20, 3, 0]},
            "rev": {"0": [0, 25, 20]},
        },
        "inf_four_node": {
            "source": "route/src/matrix/bucket_ch.rs:4855-4905",
            "cch": dict(n=4, up_off=[0, 1, 2, 4, 4], up_tgt=[2, 2, 3, 3], up_w=[10, 3, 7, INF],
                        down_off=[0, 0, 0, 2, 4], down_tgt=[0, 1, 2, 2],
                        down_w=[10, 3, 7, INF]),
            "finite_up": 3,
            "finite_down": 3,
        },
        "broom": {"source": "route/src/matrix/bucket_ch.rs:5619-5760", **broom},
        "two_channel_tie": {
            "source": "route/src/server/isochrone_handler.rs:1806-1869",
            "cases": [
                # shorter length arrives second (:1806-1845)
                dict(cch=dict(n=4, up_off=[0, 2, 3, 4, 4], up_tgt=[1, 2, 3, 3], up_w=[3, 5, 7, 5],
                              down_off=[0, 0, 0, 0, 0], down_tgt=[], down_w=[]),
                     up_len=[100, 1, 100, 1], down_len=[], seeds=[[0, 0, 0]], threshold=1000,
                     node=3, time=10, len=2),
                # shorter length arrives first (:1847-1868)
                dict(cch=dict(n=4, up_off=[0, 2, 3, 4, 4], up_tgt=[1, 2, 3, 3], up_w=[5, 3, 5, 7],
                              down_off=[0, 0, 0, 0, 0], down_tgt=[], down_w=[]),
                     up_len=[100, 1, 100, 1], down_len=[], seeds=[[0, 0, 0]], threshold=1000,
                     node=3, time=10, len=2),
            ],
        },
    }


def fingerprint(cch):
    h = hashlib.sha256()
    for k in ("up_off", "up_tgt", "up_w", "down_off", "down_tgt", "down_w"):
        h.update(np.ascontiguousarray(cch[k]).tobytes())
    return h.hexdigest()


def main():
    (HERE / "reference_kats.json").write_text(json.dumps(kats(), indent=1) + "\n")
    import cchbuild
    import workload
    from oracle import oracle as orc
    _, cch = cchbuild.build_synthetic(cchbuild.KIND_GRID, 100, 100, seed=42)
    src, tgt = workload.sources_targets(cch["n"], 100, 100, seed=42)
    m, _ = orc.Cch.from_dict(cch).matrix(src, tgt, threads=0)
    np.savez_compressed(HERE / "grid100_matrix.npz", sources=src, targets=tgt, matrix=m,
                        n=np.uint32(cch["n"]), n_up=np.uint64(len(cch["up_tgt"])),
                        n_down=np.uint64(len(cch["down_tgt"])),
                        sha256=np.array(fingerprint(cch)))
    print("wrote", HERE / "reference_kats.json", HERE / "grid100_matrix.npz")


if __name__ == "__main__":
    main()
