"""Target-restricted schedules built on the device against the host-built
ones and the oracle.

The device builder (elimination-tree ancestors of the targets, peeled to the
rows that reach a target along DOWN edges) must select exactly the rows and
edges the host builder selects, so the swept row and edge counts agree, and
every matrix cell must equal the oracle's (tolerance 0: u32 min-plus)."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF


def _cases(n, rng):
    return [
        ("random", rng.choice(n, 300, replace=False)),
        ("duplicates", np.concatenate([rng.choice(n, 50), rng.choice(n, 50)])),
        ("single", np.array([int(rng.integers(0, n))])),
        ("top ranks", np.arange(n - 40, n)),
        ("bottom ranks", np.arange(0, 40)),
    ]


@pytest.mark.parametrize("which", ["grid100", "country_small"])
def test_device_schedule_matches_host(built, grid100, country_small, which):
    import bfphast
    _, cch = grid100 if which == "grid100" else country_small
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    rng = np.random.default_rng(21)
    src = rng.choice(n, 24, replace=False).astype(np.uint32)
    full = np.stack([c.phast_query(s) for s in src])
    dev = bfphast.Graph.from_cch(cch)
    host = bfphast.Graph.from_cch(cch)
    host.set_tune(device_schedule=0)
    for name, tgt in _cases(n, rng):
        tgt = np.asarray(tgt, dtype=np.uint32)
        md, sd = dev.matrix(src, tgt, stats=True)
        mh, sh = host.matrix(src, tgt, stats=True)
        assert np.array_equal(md, full[:, tgt]), name
        assert np.array_equal(mh, full[:, tgt]), name
        assert sd["swept_nodes"] == sh["swept_nodes"], name
        assert sd["swept_edges"] == sh["swept_edges"], name
        for thr in (0, 1800):
            got = dev.matrix(src, tgt, threshold=thr)
            want = full[:, tgt]
            assert np.array_equal(got, np.where(want <= thr, want, INF)), (name, thr)


def test_device_schedule_all_targets(built, grid100):
    """Every node a target: nothing is peeled, the whole graph is swept."""
    import bfphast
    _, cch = grid100
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    src = np.array([0, 123, 35000, 17], dtype=np.uint32)
    tgt = np.arange(n, dtype=np.uint32)
    m, st = g.matrix(src, tgt, stats=True)
    assert st["swept_nodes"] == n
    assert np.array_equal(m, c.query_batch(src))


def test_device_then_host_schedule_on_one_graph(built, country_small):
    """Switching builders on one graph keeps the rank -> row map consistent."""
    import bfphast
    _, cch = country_small
    n = cch["n"]
    c = orc.Cch.from_dict(cch)
    g = bfphast.Graph.from_cch(cch)
    rng = np.random.default_rng(8)
    src = rng.choice(n, 16, replace=False).astype(np.uint32)
    full = np.stack([c.phast_query(s) for s in src])
    for k in range(6):
        g.set_tune(device_schedule=k % 2)
        tgt = rng.choice(n, 200, replace=False).astype(np.uint32)
        assert np.array_equal(g.matrix(src, tgt), full[:, tgt]), k


def test_schedule_levels_table(built, country_small):
    """bf_schedule_levels reports the last restricted schedule per level: its
    totals are the swept rows and edges, alike for both builders."""
    import bfphast
    _, cch = country_small
    n = cch["n"]
    rng = np.random.default_rng(5)
    src = rng.choice(n, 8, replace=False).astype(np.uint32)
    tgt = rng.choice(n, 400, replace=False).astype(np.uint32)
    tables = []
    for dev in (1, 0):
        g = bfphast.Graph.from_cch(cch)
        g.set_tune(device_schedule=dev)
        _, st = g.matrix(src, tgt, stats=True)
        items, edges, rows = g.schedule_levels()
        assert int(rows.sum()) == st["swept_nodes"] and int(edges.sum()) == st["swept_edges"]
        tables.append((items, edges, rows))
    for a, b in zip(tables[0], tables[1]):
        assert np.array_equal(a, b)
