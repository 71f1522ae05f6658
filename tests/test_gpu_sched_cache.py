"""Cached target-restricted schedules are reused only for exactly the same
targets.

The batched engine keeps the last target-restricted sweep schedule (rows,
work items, the target-row table and a captured CUDA graph) and reuses it
when a call asks for the same targets. Distinct target lists of one length,
alternated on one graph, must each give the oracle's cells (tolerance 0:
u32 min-plus) through both matrix engines, the seeded matrix and the serving
loop. The same checks run again in a fresh process in which every target
list hashes alike (BF_TEST_SCHED_KEY_COLLIDE), so only the exact comparison
of the targets can tell the schedules apart."""
import os
import pathlib
import subprocess
import sys
import time

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF
ROOT = pathlib.Path(__file__).resolve().parent.parent


def _target_sets(n, T, k, seed):
    rng = np.random.default_rng(seed)
    return [rng.choice(n, T, replace=False).astype(np.uint32) for _ in range(k)]


def check_alternating(cch):
    """Every check of this file on one graph; raises AssertionError on a mismatch."""
    import bfphast
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    rng = np.random.default_rng(3)
    src = rng.choice(n, 40, replace=False).astype(np.uint32)
    tsets = _target_sets(n, 64, 3, seed=4)
    # a permutation of the first set: same members, different order
    tsets.append(tsets[0][::-1].copy())
    full = np.stack([c.phast_query(s) for s in src])
    for eng in (bfphast.ENGINE_BATCHED, bfphast.ENGINE_PLAIN):
        g.set_engine(eng)
        for rep in range(2):
            for tgt in tsets:
                got = g.matrix(src, tgt)
                assert np.array_equal(got, full[:, tgt]), (eng, rep)
                thr = 1500
                got = g.matrix(src, tgt, threshold=thr)
                want = full[:, tgt]
                assert np.array_equal(got, np.where(want <= thr, want, INF)), (eng, rep, thr)
    g.set_engine(bfphast.ENGINE_BATCHED)
    # seeded matrices: one seed per source and target, target ranks alternating
    src_seeds = [[(int(s), 0)] for s in src[:12]]
    for rep in range(2):
        for tgt in tsets:
            tgt_seeds = [[(int(t), 0)] for t in tgt]
            got = g.matrix_seeded(src_seeds, tgt_seeds, INF)
            want, _ = orc.table_phast_lopsided(c, src_seeds, tgt_seeds, INF)
            assert np.array_equal(got, want), rep
    # serving loop: requests of equal shape with alternating targets, one at a time
    srv = bfphast.Server(g, hbm_budget=2 << 30, max_inflight=1)
    try:
        for rep in range(2):
            for tgt in tsets:
                t, out = srv.submit_matrix(src, tgt, INF)
                done = {}
                t0 = time.time()
                while t not in done and time.time() - t0 < 60:
                    for comp in srv.poll(wait_ms=200):
                        done[comp["ticket"]] = comp
                assert t in done and done[t]["status"] == bfphast.BF_OK
                assert np.array_equal(out, full[:, tgt]), rep
    finally:
        srv.close()
    g.close()


def test_alternating_targets_exact(built, grid100, country_small):
    check_alternating(grid100[1])
    check_alternating(country_small[1])


def test_alternating_targets_with_colliding_hash(built, grid100):
    """A fresh process where all target lists share one hash key."""
    env = dict(os.environ, BF_TEST_SCHED_KEY_COLLIDE="1")
    code = (
        "import sys; sys.path[:0] = [%r, %r, %r]\n"
        "import cchbuild, test_gpu_sched_cache as t\n"
        "_, cch = cchbuild.build_synthetic(cchbuild.KIND_GRID, 100, 100, seed=42)\n"
        "t.check_alternating(cch)\n"
        "print('ok')\n" % (str(ROOT / "butterfly-osm_gb300"), str(ROOT), str(ROOT / "tests")))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
