"""GPU engine vs the CPU oracle, through the C ABI. Bit-exact (tolerance 0:
all arithmetic is u32 saturating min-plus)."""
import pathlib

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
INF = 0xFFFFFFFF
GOLDEN = pathlib.Path(__file__).parent / "golden"


def _graph(d, **kw):
    import bfphast
    return bfphast.Graph(d["n"], d["up_off"], d["up_tgt"], d["up_w"], d["down_off"],
                         d["down_tgt"], d["down_w"], **kw)


ENGINES = ["plain", "batched"]


def _engine(g, name):
    import bfphast
    g.set_engine(bfphast.ENGINE_PLAIN if name == "plain" else bfphast.ENGINE_BATCHED)


@pytest.mark.parametrize("engine", ENGINES)
def test_kat_five_node_and_asym(built, kats, engine):
    for key in ("five_node", "asym_three_node"):
        k = kats[key]
        g = _graph(k["cch"])
        _engine(g, engine)
        for s, want in k["fwd"].items():
            assert g.phast_query(int(s)).tolist() == want
        n = k["cch"]["n"]
        m = g.matrix(np.arange(n), np.arange(n))
        c = orc.Cch(**{"n": n, **{x: k["cch"][x] for x in ("up_off", "up_tgt", "up_w",
                                                          "down_off", "down_tgt", "down_w")}})
        want, _ = c.matrix(np.arange(n), np.arange(n))
        assert np.array_equal(m, want)


@pytest.mark.parametrize("engine", ENGINES)
def test_kat_inf_four_node(built, kats, engine):
    g = _graph(kats["inf_four_node"]["cch"])
    _engine(g, engine)
    info = g.info()
    assert info["n_up"] == 3 and info["n_down"] == 3
    assert g.phast_query(0).tolist() == [0, 13, 10, 17]
    assert g.phast_query(3).tolist() == [17, 10, 7, 0]


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("n_leaf", ["5", "12"])
def test_kat_broom_bounded(built, kats, engine, n_leaf):
    b = kats["broom"][n_leaf]
    g = _graph(b["cch"])
    _engine(g, engine)
    n = int(n_leaf)
    expect = np.array(b["expect"], dtype=np.uint32)
    assert np.array_equal(g.matrix(np.arange(n), np.arange(n)), expect)
    for thr in b["thresholds"]:
        m = g.matrix(np.arange(n), np.arange(n), threshold=thr)
        assert np.array_equal(m, np.where(expect <= thr, expect, INF))


@pytest.mark.parametrize("engine", ENGINES)
def test_grid100_matrix_golden(built, grid100, engine):
    _, cch = grid100
    gold = np.load(GOLDEN / "grid100_matrix.npz")
    g = _graph(cch)
    _engine(g, engine)
    m = g.matrix(gold["sources"], gold["targets"])
    assert m.dtype == np.uint32 and np.array_equal(m, gold["matrix"])


@pytest.mark.parametrize("engine", ENGINES)
def test_grid100_query_batch_vs_oracle(built, grid100, engine):
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    _engine(g, engine)
    src = np.array([0, 1, 77, 5000, 12345, 20000, 35723, 35000], dtype=np.uint32)
    assert np.array_equal(g.query_batch(src), c.query_batch(src))
    # 40 sources: more than one K = 32 batch
    src40 = np.arange(0, cch["n"], cch["n"] // 40, dtype=np.uint32)[:40]
    got = g.query_batch(src40)
    for lane in range(0, 40, 7):
        assert np.array_equal(got[lane], c.phast_query(src40[lane]))


@pytest.mark.parametrize("engine", ENGINES)
def test_grid100_bounded(built, grid100, engine):
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    _engine(g, engine)
    src = np.arange(3, cch["n"], 997, dtype=np.uint32)[:36]
    full = np.stack([c.phast_query(s) for s in src])
    tgt = np.arange(0, cch["n"], 3, dtype=np.uint32)
    for thr in (0, 400, 2500, 9000):
        m = g.matrix(src, tgt, threshold=thr)
        want = full[:, tgt]
        assert np.array_equal(m, np.where(want <= thr, want, INF))


def test_country_small_matrix(built, country_small):
    import workload
    _, cch = country_small
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    src, tgt = workload.sources_targets(cch["n"], 70, 300, seed=5)
    want, _ = c.matrix(src, tgt)
    for eng in ENGINES:
        _engine(g, eng)
        assert np.array_equal(g.matrix(src, tgt), want)


def test_invalid_ids_rejected(built, grid100):
    import bfphast
    _, cch = grid100
    g = _graph(cch)
    with pytest.raises(bfphast.BfError) as e:
        g.matrix([0, cch["n"]], [1])
    assert e.value.status == bfphast.BF_ERR_INVALID
    # the graph stays usable after a rejected call
    assert g.phast_query(0)[0] == 0


def test_empty_inputs(built, grid100):
    _, cch = grid100
    g = _graph(cch)
    assert g.matrix(np.zeros(0, np.uint32), [1, 2]).shape == (0, 2)
    assert g.matrix([1, 2], np.zeros(0, np.uint32)).shape == (2, 0)


def test_duplicate_sources_and_targets(built, grid100):
    _, cch = grid100
    c = orc.Cch.from_dict(cch)
    g = _graph(cch)
    src = np.array([9, 9, 9, 100, 9], dtype=np.uint32)
    tgt = np.array([9, 100, 100, 9], dtype=np.uint32)
    want, _ = c.matrix(src, tgt)
    assert np.array_equal(g.matrix(src, tgt), want)


@pytest.mark.parametrize("tune", [dict(threads_per_block=32, edges_per_item=1, graph_capture=0,
                                       lanes_per_wave=32),
                                  dict(threads_per_block=256, edges_per_item=64,
                                       graph_capture=1, lanes_per_wave=0),
                                  dict(threads_per_block=64, edges_per_item=3, graph_capture=1,
                                       lanes_per_wave=64, overlap_upward=0),
                                  dict(threads_per_block=128, edges_per_item=16, graph_capture=1,
                                       lanes_per_wave=0, small_level_rows=4096,
                                       small_level_edges=2)])
def test_tunables_keep_results_exact(built, grid100, tune):
    _, cch = grid100
    gold = np.load(GOLDEN / "grid100_matrix.npz")
    g = _graph(cch)
    g.set_tune(**tune)
    assert g.get_tune()["edges_per_item"] == tune["edges_per_item"]
    for _ in range(3):  # first call builds the schedule, later ones replay it
        assert np.array_equal(g.matrix(gold["sources"], gold["targets"]), gold["matrix"])


def test_autotune_picks_a_valid_choice(built, grid100):
    import torch
    import workload
    _, cch = grid100
    g = _graph(cch)
    src, tgt = workload.sources_targets(cch["n"], 300, 500, seed=77)
    d_s = torch.from_numpy(src.view(np.int32)).cuda()
    d_t = torch.from_numpy(tgt.view(np.int32)).cuda()
    best = g.autotune(d_s.data_ptr(), len(src), d_t.data_ptr(), len(tgt), reps=1)
    assert best["tried"] >= 11 and best["step_ms"] > 0
    assert best["threads_per_block"] in (64, 128, 256)
    gold = np.load(GOLDEN / "grid100_matrix.npz")
    assert np.array_equal(g.matrix(gold["sources"], gold["targets"]), gold["matrix"])


@pytest.mark.parametrize("mapped", [1, 0])
def test_page_locked_output(built, grid100, mapped):
    # a page-locked output buffer is written by the extraction kernel directly
    import torch
    _, cch = grid100
    gold = np.load(GOLDEN / "grid100_matrix.npz")
    g = _graph(cch)
    g.set_tune(mapped_output=mapped)
    S, T = len(gold["sources"]), len(gold["targets"])
    out = torch.full((S * T,), -1, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    out = out.reshape(S, T)
    for _ in range(2):
        m = g.matrix(gold["sources"], gold["targets"], out=out)
        assert m is out or np.shares_memory(m, out)
        assert np.array_equal(out, gold["matrix"])


def _with_parallel_up_edges(d, seed):
    """The CSR with a copy of every fifth finite UP edge listed again (weights
    above, equal to and below the original), in shuffled order within each
    source's list."""
    rng = np.random.default_rng(seed)
    n = d["n"]
    off, tgt, w = d["up_off"], d["up_tgt"], d["up_w"]
    new_off, new_t, new_w = [0], [], []
    for u in range(n):
        t = list(tgt[off[u]:off[u + 1]])
        ww = list(w[off[u]:off[u + 1]])
        for k in range(len(t)):
            if ww[k] != INF and rng.random() < 0.2:
                t.append(t[k])
                ww.append(int(max(0, min(INF - 1, int(ww[k]) + int(rng.integers(-3, 4))))))
        order = rng.permutation(len(t))
        new_t += [t[i] for i in order]
        new_w += [ww[i] for i in order]
        new_off.append(len(new_t))
    out = dict(d)
    out["up_off"] = np.asarray(new_off, np.uint64)
    out["up_tgt"] = np.asarray(new_t, np.uint32)
    out["up_w"] = np.asarray(new_w, np.uint32)
    return out


@pytest.mark.parametrize("engine", ENGINES)
def test_parallel_up_edges(built, grid100, engine):
    # a CSR that lists some UP edges twice: every relaxation takes the smaller
    # weight, as the oracle relaxing each listed edge does
    _, base = grid100
    d = _with_parallel_up_edges(base, 11)
    g = _graph(d)
    _engine(g, engine)
    c = orc.Cch(**{x: d[x] for x in ("n", "up_off", "up_tgt", "up_w", "down_off", "down_tgt",
                                      "down_w")})
    rng = np.random.default_rng(3)
    src = rng.choice(d["n"], 40, replace=False)
    tgt = rng.choice(d["n"], 300, replace=False)
    want, _ = c.matrix(src, tgt)
    assert np.array_equal(g.matrix(src, tgt), want)
    assert g.info()["n_up"] == int((base["up_w"] != INF).sum())
