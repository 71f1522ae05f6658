"""The ncu summaries the benchmark reads (`profiles/*.json`) add up.

`bench.py` scales full-size DRAM traffic from these small captures
(traffic = DRAM bytes per algorithmic byte x the run's algorithmic bytes),
so their per-launch byte counts, sums and ratios are checked here against
the algorithmic-byte formulas they state."""
import json
import pathlib

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _load(name):
    return json.loads((ROOT / "profiles" / name).read_text())


def test_sweep_capture_adds_up():
    p = _load("sweep_items_country2000.json")
    lanes = 2000
    alg = dram = 0
    for ln in p["launches"]:
        want = 16 * ln["items"] + 8 * ln["edges"] + 4 * lanes * (ln["edges"] + ln["rows"])
        assert ln["alg_bytes"] == want
        alg += ln["alg_bytes"]
        dram += ln["dram_read"] + ln["dram_write"]
    assert p["alg_bytes_sum"] == alg
    assert p["dram_bytes_sum"] == dram
    assert abs(p["traffic_per_alg_byte"] - dram / alg) < 5e-4
    assert 0.5 < p["traffic_per_alg_byte"] < 2.0


def test_customize_capture_adds_up():
    p = _load("customize_country1000.json")
    dram = sum(k["dram_read"] + k["dram_write"] for k in p["kernels_per_run"].values())
    assert p["dram_bytes_per_run"] == dram
    assert abs(p["traffic_per_alg_byte"] - dram / p["algorithmic_bytes"]) < 5e-4
    shares = sum(k["share"] for k in p["kernels_per_run"].values())
    assert abs(shares - 1.0) < 0.01


def test_capture_commands_stay_small():
    # a capture with more than the launch time collects from one kernel
    # pattern and a few launches, and every ncu command leaves the clocks alone
    p = _load("sweep_items_country2000.json")
    assert "--clock-control none" in p["command"] and "-c 3" in p["command"]
    assert "-k regex:k_sweep_items" in p["command"]
    for md in (ROOT / "profiles").glob("*.md"):
        text = md.read_text()
        if "ncu " in text:
            assert "--clock-control none" in text, md.name
