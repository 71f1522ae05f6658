"""Benchmark: 10k x 10k duration matrix on the country-scale synthetic CCH.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step): the 10 000 x 10 000 u32 duration matrix, sources and
targets uniform over the ranks of the 2000 x 2500 lattice road graph with a
3-level hierarchy (11.94 M edge states after edge-based expansion), contracted
by the host CCH pipeline. The batched GPU engine computes it; the plain GPU
sweep (one K = 32 batch per launch sequence) is timed on a slice of the same
workload for the speed-up, and the CPU restatement of the reference's K = 8
SoA batched PHAST (compute_matrix_flat_soa) is timed on a bounded sample.

value   cells/s with sources, targets and the output resident in HBM
        (bf_matrix_device, CUDA events on the launching stream)
e2e     cells/s through bf_matrix with pinned host buffers: the H2D copy of
        sources/targets and the D2H copy of the whole matrix are inside the
        timed region
Every step overwrites an 11 GB distance slab, far larger than L2 (126 MB).

N > 1 (torchrun): every rank runs the same workload on its own GPU with its own
seed (weak scaling, no collective on the data path); value = all ranks'
cells / max-over-ranks time.
"""
import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "butterfly-osm_gb300"))
sys.path.insert(0, str(ROOT))

S_CELLS = 10000
T_CELLS = 10000
METRIC = "10k x 10k matrix cells/s (bit-exact vs CPU PHAST)"
UNIT = "cells/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sources", type=int, default=S_CELLS)
    ap.add_argument("--targets", type=int, default=T_CELLS)
    ap.add_argument("--rows", type=int, default=2000)
    ap.add_argument("--cols", type=int, default=2500)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default tunables (short profiling runs)")
    ap.add_argument("--serve-s", type=float, default=60.0,
                    help="seconds of Poisson arrivals per serving rate (0 = skip)")
    ap.add_argument("--serve-rates", default="50,100,250,500",
                    help="arrival rates (requests per second), comma-separated")
    ap.add_argument("--fresh-steps", type=int, default=10,
                    help="timed steps with a new target set each (0 = skip)")
    ap.add_argument("--plain-sources", type=int, default=1000,
                    help="plain-engine matrix side (sources = targets, K = 32)")
    ap.add_argument("--level-table", default="",
                    help="write the matrix schedule's per-level items / edges / rows (JSON) "
                         "to this path, to attribute profiled sweep launches to levels")
    ap.add_argument("--isochrones", type=int, default=100000,
                    help="bulk isochrone origins (0 = skip)")
    ap.add_argument("--no-tiles", action="store_true",
                    help="skip the matrix tile emission leg")
    ap.add_argument("--no-customize", action="store_true",
                    help="skip the CCH customization leg")
    ap.add_argument("--contours", type=int, default=64,
                    help="isochrone contour rasters in one batch (0 = skip)")
    ap.add_argument("--tiles-synthetic", action="store_true",
                    help="only the tile emission leg, on a seeded 10k x 10k matrix whose "
                         "in-bound fraction (2.1 %% within 30 minutes) is the country matrix's; "
                         "no graph (a small device footprint for kernel captures)")
    return ap.parse_args()


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            # nvidia-smi's start-up holds driver locks that stall CUDA calls:
            # let it deliver its first sample before the timed region opens
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def build_workload(args, seed):
    import cchbuild
    import workload
    e, cch = cchbuild.build_synthetic(cchbuild.KIND_COUNTRY, args.rows, args.cols, seed=42,
                                      with_topo=not getattr(args, "no_customize", True))
    if getattr(args, "contours", 0):
        cch["geo"] = {k: e[k] for k in ("n_intersections", "state_tail", "state_head",
                                        "node_weight")}
    n = cch["n"]
    src, tgt = workload.sources_targets(n, args.sources, args.targets, seed=seed)
    return cch, src, tgt


def cpu_sample(cch, src, tgt, budget_s, rows=None):
    """Time the CPU restatement of compute_matrix_flat_soa (K = 8) on a row
    sample on all host threads. Returns (dict, sample_rows, sample_matrix)."""
    import numpy as np
    from oracle import oracle as orc
    c = orc.Cch.from_dict(cch)
    threads = os.cpu_count() or 1
    if rows is None:
        # calibrate on 2 K=8 batches per host thread, then size the sample to
        # about budget_s seconds of CPU work (at least a 1% row sample)
        cal = max(8, min(len(src), 16 * threads))
        t0 = time.perf_counter()
        c.matrix(src[np.linspace(0, len(src) - 1, cal).astype(np.int64)], tgt, threads=threads)
        per_row = (time.perf_counter() - t0) / cal
        rows = int(budget_s / max(per_row, 1e-9))
        rows = max(8, min(len(src), max(rows, len(src) // 100)))
    pick = np.linspace(0, len(src) - 1, rows).astype(np.int64)
    t0 = time.perf_counter()
    m, used = c.matrix(src[pick], tgt, threads=threads)
    dt = time.perf_counter() - t0
    cells = rows * len(tgt)
    return ({"value": cells / dt, "unit": UNIT, "cores": int(used), "kind": "port",
             "sample": "%d of %d rows (seeded even spacing) x %d targets, %.1f s"
                       % (rows, len(src), len(tgt), dt)}, pick, m)


def run_ours(args, rank, world, dist):
    import numpy as np
    import torch
    import bfphast
    import replicas
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    cch, src, tgt = build_workload(args, seed=42 + rank)
    S, T = len(src), len(tgt)
    g = bfphast.Graph.from_cch(cch, device=dev)
    stream = torch.cuda.current_stream()
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_tgt = torch.from_numpy(tgt.view(np.int32)).cuda()
    d_out = torch.empty(S * T, dtype=torch.int32, device="cuda")

    def step():
        return g.matrix_device(d_src.data_ptr(), S, d_tgt.data_ptr(), T, d_out.data_ptr(),
                               stream=stream.cuda_stream)

    # per-graph autotune on a different sample of the same shape
    import workload
    ts, tt = workload.sources_targets(cch["n"], S, T, seed=1042 + rank)
    d_ts = torch.from_numpy(ts.view(np.int32)).cuda()
    d_tt = torch.from_numpy(tt.view(np.int32)).cuda()
    if args.no_autotune:
        tune = dict(g.get_tune(), autotuned=False)
    else:
        tune = g.autotune(d_ts.data_ptr(), S, d_tt.data_ptr(), T, reps=2)
    del d_ts, d_tt

    for _ in range(args.warmup):
        step()
    sync = (lambda: dist.barrier()) if dist else (lambda: None)
    sync()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            stats.append(step())
        e1.record(stream)
        torch.cuda.synchronize()
    sync()
    ms = e0.elapsed_time(e1) / args.steps
    ms_all = replicas.max_over_ranks(ms, dist, device="cuda")
    value = replicas.whole_job_rate(S * T, world, ms_all / 1e3)
    out_dev = d_out.view(S, T).cpu().numpy().view(np.uint32)

    # e2e: host (pinned) buffers through bf_matrix, copies inside the region
    h_src = torch.from_numpy(src.view(np.int32)).pin_memory().numpy().view(np.uint32)
    h_tgt = torch.from_numpy(tgt.view(np.int32)).pin_memory().numpy().view(np.uint32)
    h_out = torch.empty(S * T, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    h_out = h_out.reshape(S, T)
    for _ in range(max(1, args.warmup)):
        g.matrix(h_src, h_tgt, out=h_out)
    sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        g.matrix(h_src, h_tgt, out=h_out)
    e2e_s = replicas.max_over_ranks((time.perf_counter() - t0) / args.steps, dist, device="cuda")
    e2e_ok = bool(np.array_equal(h_out, out_dev))

    # roofline of the dominant kernel (the restricted downward sweep)
    st = stats[-1]
    K, M, N = st["lanes"], st["swept_edges"], st["swept_nodes"]
    alg_bytes = 8 * M + 4 * (N + 1) + 4 * K * M + 4 * K * N
    sweep_s = st["downward_ms"] / 1e3
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / sweep_s / 1e9
    # DRAM traffic: bytes per algorithmic byte from a three-launch capture of
    # large levels at 2000 lanes, scaled by this sweep's algorithmic bytes
    traffic = ratio = None
    prof = ROOT / "profiles" / "sweep_items_country2000.json"
    if prof.exists():
        ratio = json.loads(prof.read_text()).get("traffic_per_alg_byte")
        if ratio:
            traffic = int(round(ratio * alg_bytes))
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "traffic_source": ("scaled: %s DRAM bytes per algorithmic byte, 3 launches at "
                               "2000 lanes" % ratio) if traffic else None,
            "peak_kind": peak_kind, "kernel": "k_sweep_items",
            "alg_bytes_per_sweep": alg_bytes, "sweep_ms": round(st["downward_ms"], 3),
            "swept_nodes": N, "swept_edges": M, "lanes": K}

    if args.level_table:
        items, edges, rows = g.schedule_levels()
        keep = items > 0  # launches go to levels with work items, in order
        pathlib.Path(args.level_table).write_text(json.dumps({
            "lanes": int(st["lanes"]), "items": items[keep].tolist(),
            "edges": edges[keep].tolist(), "rows": rows[keep].tolist()}))
    # plain GPU sweep on its own workload (1000 x 1000, K = 32 batches): the
    # >= 10x denominator, CUDA events on the launching stream
    plain = run_plain(g, src, tgt, out_dev, args.plain_sources, stream)
    fresh = None
    if args.fresh_steps > 0:
        fresh = run_fresh(g, cch, src, S, T, args.fresh_steps, max(3, args.warmup), stream,
                          rank, dist)

    res = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_all, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
           "data": "synthetic (seeded country-scale lattice road graph, CCH built in-run)",
           "config": {"workload": "country 2000x2500 lattice, 10k x 10k matrix, batched engine",
                      "n_nodes": cch["n"], "m_down": int(len(cch["down_tgt"])),
                      "m_up": int(len(cch["up_tgt"])), "sources": S, "targets": T,
                      "parallelism": "dp%d" % world if world > 1 else "single",
                      "l2": "slab of %.1f GB rewritten every step (> L2)"
                            % (st["lanes"] * max(N, 1) * 4 / 1e9),
                      "tune": tune},
           "e2e": {"value": round(replicas.whole_job_rate(S * T, world, e2e_s), 1), "unit": UNIT,
                   "h2d_bytes_per_step": (S + T) * 4, "d2h_bytes_per_step": S * T * 4,
                   "ms_per_step": round(e2e_s * 1e3, 3), "matches_device_run": e2e_ok},
           "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
           "roofline": roof,
           "plain_gpu": dict(plain, speedup_batched_over_plain=round(
               value / world / plain["value"], 2)),
           "phases_ms": {"upward": round(st["upward_ms"], 3),
                         "downward": round(st["downward_ms"], 3),
                         "extract": round(st["extract_ms"], 3)},
           "clocks": clk.summary()}
    if fresh:
        res["fresh_targets"] = fresh
    if args.isochrones > 0:
        res["isochrones"] = run_isochrones(g, cch, args.isochrones, seed=42 + rank)
    if args.serve_s > 0 and rank == 0:
        rates = [float(x) for x in args.serve_rates.split(",") if x.strip()]
        runs = [run_serving(g, cch["n"], args.serve_s, r) for r in rates]
        res["serving"] = {"by_rate": runs,
                          "mix": runs[0]["mix"] if runs else None,
                          "workload": "Poisson arrivals for %.0f s at each rate on the "
                                      "country graph" % args.serve_s}
    if args.contours > 0 and rank == 0:
        res["contours"] = run_contours(g, cch, args.contours, args.cols)
    if not args.no_customize and rank == 0:
        res["customize"] = run_customize(cch, args.steps, args.warmup, not args.no_cpu)
    if not args.no_tiles and rank == 0:
        res["tiles"] = run_tiles(out_dev, args.steps, args.warmup, not args.no_cpu)
    return res, cch, src, tgt, out_dev


def run_plain(g, src, tgt, out_dev, side, stream):
    """The plain engine (one K = 32 batch at a time) on a side x side matrix
    of the same graph: CUDA events around one call after a warm-up call,
    checked against the batched engine's cells."""
    import numpy as np
    import torch
    import bfphast
    side = min(side, len(src), len(tgt))
    d_s = torch.from_numpy(src[:side].view(np.int32)).cuda()
    d_t = torch.from_numpy(tgt[:side].view(np.int32)).cuda()
    d_o = torch.empty(side * side, dtype=torch.int32, device="cuda")
    g.set_engine(bfphast.ENGINE_PLAIN)
    try:
        g.matrix_device(d_s.data_ptr(), side, d_t.data_ptr(), side, d_o.data_ptr(),
                        stream=stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = g.matrix_device(d_s.data_ptr(), side, d_t.data_ptr(), side, d_o.data_ptr(),
                             stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
    finally:
        g.set_engine(bfphast.ENGINE_BATCHED)
    ms = e0.elapsed_time(e1)
    got = d_o.view(side, side).cpu().numpy().view(np.uint32)
    return {"value": round(side * side / ms * 1e3, 1), "unit": UNIT, "ms": round(ms, 3),
            "workload": "%d x %d matrix, K = 32 lanes per batch, %d batches"
                        % (side, side, (side + 31) // 32),
            "gpu_launches": int(st["kernel_launches"]),
            "bit_exact_vs_batched": bool(np.array_equal(got, out_dev[:side, :side]))}


def run_fresh(g, cch, src, S, T, steps, warmup, stream, rank, dist):
    """10k x 10k matrices with a NEW seeded target set every step (the
    caller shape of a matrix server: each request brings its own targets), so
    every step builds its target-restricted schedule: device-resident ids
    (`value`) and through bf_matrix with page-locked host buffers (`e2e`).
    The last step's matrix is checked on a row sample against the oracle."""
    import numpy as np
    import torch
    import replicas
    import workload
    from oracle import oracle as orc
    n = cch["n"]
    sets = [workload.uniform_ids(n, T, 7001 + 97 * i + rank) for i in range(warmup + steps)]
    d_sets = [torch.from_numpy(t.view(np.int32)).cuda() for t in sets]
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_out = torch.empty(S * T, dtype=torch.int32, device="cuda")

    def step(i):
        return g.matrix_device(d_src.data_ptr(), S, d_sets[i].data_ptr(), T, d_out.data_ptr(),
                               stream=stream.cuda_stream)

    for i in range(warmup):
        step(i)
    sync = (lambda: dist.barrier()) if dist else (lambda: None)
    sync()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    e0.record(stream)
    for i in range(warmup, warmup + steps):
        stats.append(step(i))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = replicas.max_over_ranks(e0.elapsed_time(e1) / steps, dist, device="cuda")
    last = d_out.view(S, T).cpu().numpy().view(np.uint32)
    pick = np.linspace(0, S - 1, 16).astype(np.int64)
    want, _ = orc.Cch.from_dict(cch).matrix(src[pick], sets[-1], threads=os.cpu_count() or 1)
    exact = bool(np.array_equal(last[pick], want))
    # end to end with page-locked host buffers, a new target set per step
    pin = lambda a: torch.from_numpy(a.view(np.int32)).pin_memory().numpy().view(np.uint32)
    h_src = pin(src)
    h_sets = [pin(t) for t in sets]
    h_out = torch.empty(S * T, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    h_out = h_out.reshape(S, T)
    g.matrix(h_src, h_sets[0], out=h_out)
    sync()
    t0 = time.perf_counter()
    for i in range(warmup, warmup + steps):
        g.matrix(h_src, h_sets[i], out=h_out)
    e2e_s = replicas.max_over_ranks((time.perf_counter() - t0) / steps, dist, device="cuda")
    sched = [s_["schedule_ms"] for s_ in stats]
    return {"value": round(replicas.whole_job_rate(S * T, 1, ms / 1e3), 1), "unit": UNIT,
            "ms_per_step": round(ms, 3), "steps": steps,
            "schedule_ms_mean": round(float(np.mean(sched)), 3),
            "schedule_ms_max": round(float(np.max(sched)), 3),
            "upward_ms": round(float(np.mean([s_["upward_ms"] for s_ in stats])), 3),
            "downward_ms": round(float(np.mean([s_["downward_ms"] for s_ in stats])), 3),
            "swept_nodes_mean": round(float(np.mean([s_["swept_nodes"] for s_ in stats])), 1),
            "gpu_launches": int(sum(s_["kernel_launches"] for s_ in stats)),
            "e2e": {"value": round(replicas.whole_job_rate(S * T, 1, e2e_s), 1), "unit": UNIT,
                    "h2d_bytes_per_step": (S + T) * 4, "d2h_bytes_per_step": S * T * 4,
                    "ms_per_step": round(e2e_s * 1e3, 3)},
            "bit_exact_sample": {"rows": len(pick), "targets": T, "equal": exact},
            "workload": "10k x 10k, a new seeded 10k-target set every step"}


def run_serving(g, n, seconds, rate, seed=7):
    """Serving mix on the same graph: Poisson arrivals at `rate` req/s for
    `seconds`; 70% matrices with S and T log-uniform in [10, 5000], 30%
    isochrones with a threshold uniform in [300, 3600] s. Latency is
    completion minus submission (server clock)."""
    import numpy as np
    import bfphast
    rng = np.random.default_rng(seed)
    count = int(rng.poisson(rate * seconds))
    arrivals = np.sort(rng.uniform(0, seconds, count))
    specs = []
    for _ in range(count):
        if rng.random() < 0.7:
            S = int(np.exp(rng.uniform(np.log(10), np.log(5000))))
            T = int(np.exp(rng.uniform(np.log(10), np.log(5000))))
            specs.append(("m", rng.integers(0, n, S).astype(np.uint32),
                          rng.integers(0, n, T).astype(np.uint32)))
        else:
            specs.append(("i", int(rng.integers(0, n)), int(rng.integers(3000, 36001))))
    srv = bfphast.Server(g, hbm_budget=60 << 30, max_inflight=64)
    kinds, done = {}, {}
    rejected = 0
    t0 = time.perf_counter()
    for i, (at, sp) in enumerate(zip(arrivals, specs)):
        wait = t0 + at - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        try:
            if sp[0] == "m":
                t, _ = srv.submit_matrix(sp[1], sp[2], tag=i)
                kinds[t] = ("m", len(sp[1]) * len(sp[2]))
            else:
                t, _ = srv.submit_isochrone(sp[1], sp[2], tag=i)
                kinds[t] = ("i", 0)
        except bfphast.BfError as e:
            if e.status != bfphast.BF_ERR_BUSY:
                raise
            rejected += 1
        for c in srv.poll(wait_ms=0):
            done[c["ticket"]] = c
    while len(done) < len(kinds) and time.perf_counter() - t0 < seconds + 120:
        for c in srv.poll(wait_ms=100):
            done[c["ticket"]] = c
    elapsed = time.perf_counter() - t0
    srv.close()
    lat = {k: [] for k in ("m", "i")}
    cells = ok = 0
    for t, c in done.items():
        if c["status"] == 0:
            ok += 1
            kd, cl = kinds[t]
            lat[kd].append((c["done_s"] - c["submit_s"]) * 1e3)
            cells += cl
    alll = lat["m"] + lat["i"]
    pct = lambda v, q: round(float(np.percentile(v, q)), 2) if v else None
    return {"requests": count, "completed_ok": ok, "rejected_busy": rejected,
            "failed": len(done) - ok, "unfinished": len(kinds) - len(done),
            "seconds": seconds, "rate_req_s": rate, "elapsed_s": round(elapsed, 2),
            "p50_ms": pct(alll, 50), "p99_ms": pct(alll, 99),
            "matrix_p50_ms": pct(lat["m"], 50), "matrix_p99_ms": pct(lat["m"], 99),
            "isochrone_p50_ms": pct(lat["i"], 50), "isochrone_p99_ms": pct(lat["i"], 99),
            "cells_per_s": round(cells / elapsed, 1),
            "isochrones_per_s": round(len(lat["i"]) / elapsed, 1),
            "mix": "70% matrices S,T log-uniform[10,5000]; 30% isochrones T U[300,3600] s"}


def run_isochrones(g, cch, count, seed=42):
    """Bulk isochrones: `count` origins uniform over ranks,
    thresholds uniform over {300, 600, 1200, 1800, 3600} s; bitsets written
    to HBM in chunks of 20 000 origins; a sample is checked bit for bit
    against the CPU oracle, which is also timed on the host cores."""
    import numpy as np
    import torch
    import workload
    from oracle import oracle as orc
    n = cch["n"]
    w64 = (n + 63) // 64
    o, t = workload.isochrone_workload(n, count, seed=seed)
    chunk = min(count, 20000)
    d_b = torch.empty(chunk * w64, dtype=torch.int64, device="cuda")
    d_c = torch.empty(chunk, dtype=torch.int64, device="cuda")
    d_o = torch.from_numpy(o.view(np.int32)).cuda()
    d_t = torch.from_numpy(t.view(np.int32)).cuda()
    stream = torch.cuda.current_stream()
    # wave width and form tuned on another sample of the same shape
    to, tt = workload.isochrone_workload(n, min(count, 4096), seed=seed + 1000)
    d_to = torch.from_numpy(to.view(np.int32)).cuda()
    d_tt = torch.from_numpy(tt.view(np.int32)).cuda()
    tune = g.autotune_isochrones(d_to.data_ptr(), d_tt.data_ptr(), len(to), reps=1)
    del d_to, d_tt
    g.isochrone_bitsets_device(d_o.data_ptr(), d_t.data_ptr(), min(count, 1024),
                               d_b.data_ptr(), d_c.data_ptr())  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    counts = np.zeros(count, dtype=np.uint64)
    last = None
    sweep_bytes, sweep_ms, waves, lanes = 0, 0.0, 0, 0
    e0.record(stream)
    for c0 in range(0, count, chunk):
        m = min(chunk, count - c0)
        st = g.isochrone_bitsets_device(d_o.data_ptr() + 4 * c0, d_t.data_ptr() + 4 * c0, m,
                                        d_b.data_ptr(), d_c.data_ptr(),
                                        stream=stream.cuda_stream)
        launches += st["kernel_launches"]
        sweep_bytes += st["sweep_bytes"]
        sweep_ms += st["downward_ms"]
        waves += st["waves"]
        lanes = max(lanes, st["lanes"])
        counts[c0:c0 + m] = d_c[:m].cpu().numpy().view(np.uint64)
        last = (c0, m)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    # end to end through the host-buffer call, before the CPU sample's host
    # allocations
    e2e = run_isochrones_e2e(g, o, t, w64, min(count, 2048))
    # bit-exact sample from the last chunk + CPU oracle rate on the host cores
    c = orc.Cch.from_dict(cch)
    c0, m = last
    pick = np.linspace(c0, c0 + m - 1, min(m, 1024)).astype(np.int64)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    wb, wc = c.isochrone_bitsets(o[pick], t[pick], threads=threads)
    cpu_s = time.perf_counter() - t0
    got = d_b.view(chunk, w64)[torch.from_numpy(pick - c0)].cpu().numpy().view(np.uint64)
    exact = bool(np.array_equal(got, wb)) and bool(np.array_equal(counts[pick], wc))
    del wb
    # the CPU rate on about 10 s of work: further 1024-origin pieces of the
    # chunk (other origins than the checked ones), results dropped
    cpu_n = len(pick)
    rest = np.setdiff1d(np.arange(c0, c0 + m), pick)
    for k0 in range(0, len(rest), 1024):
        if cpu_s >= 10.0:
            break
        part = rest[k0:k0 + 1024]
        t0 = time.perf_counter()
        c.isochrone_bitsets(o[part], t[part], threads=threads)
        cpu_s += time.perf_counter() - t0
        cpu_n += len(part)
    peak, peak_kind = measured_peak()
    achieved = sweep_bytes / (sweep_ms / 1e3) / 1e9 if sweep_ms else 0.0
    return {"origins": count, "value": round(count / sec, 1), "unit": "isochrones/s",
            "seconds": round(sec, 3), "gpu_launches": int(launches),
            "mean_reachable_nodes": round(float(counts.mean()), 1),
            "thresholds_s": list(workload.ISO_THRESHOLDS_S),
            "waves": int(waves), "lanes_per_wave": int(lanes),
            "tune": {"isochrone_lanes": tune["isochrone_lanes"],
                     "persistent_waves": bool(tune["persistent_sweep"] & 2),
                     "candidates": tune["tried"], "sample_ms": round(tune["step_ms"], 2)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                         "peak_kind": peak_kind, "kernel": "k_sweep_gated16 (all waves)",
                         "alg_bytes": int(sweep_bytes), "sweep_ms": round(sweep_ms, 3),
                         "bytes_rule": "per wave: 16 B per work item + 8 B per edge record "
                                       "scanned, 2 B x lanes per active source row gathered "
                                       "and per row written"},
            "e2e": e2e,
            "bit_exact_sample": {"origins": len(pick), "equal": exact},
            "cpu_baseline": {"value": round(cpu_n / cpu_s, 2), "unit": "isochrones/s",
                             "cores": threads, "kind": "port",
                             "sample": "%d origins of the last chunk, %.1f s" % (cpu_n, cpu_s)}}


def run_isochrones_e2e(g, o, t, w64, m):
    """bf_isochrone_bitsets with page-locked host buffers on the first m
    origins of the workload: origins and thresholds in, every bitset row
    (ceil(n / 64) words per origin) and count out, inside the timed call."""
    import numpy as np
    import torch
    pin = lambda k, dt: torch.empty(k, dtype=dt, pin_memory=True).numpy()
    h_o, h_t = pin(m, torch.int32).view(np.uint32), pin(m, torch.int32).view(np.uint32)
    h_o[:], h_t[:] = o[:m], t[:m]
    bits = pin(m * w64, torch.int64).view(np.uint64).reshape(m, w64)
    counts = pin(m, torch.int64).view(np.uint64)
    g.isochrone_bitsets(h_o, h_t, out=(bits, counts))
    t0 = time.perf_counter()
    g.isochrone_bitsets(h_o, h_t, out=(bits, counts))
    sec = time.perf_counter() - t0
    return {"value": round(m / sec, 1), "unit": "isochrones/s", "origins": m,
            "ms": round(sec * 1e3, 2), "h2d_bytes_per_step": 8 * m,
            "d2h_bytes_per_step": 8 * m * (w64 + 1)}


def run_contours(g, cch, count, cols, threshold_s=1800, seed=11):
    """Isochrone polygons for `count` origins through bf_isochrone_polygons:
    settled sets in bulk, each reachable road whole or cut at the threshold
    (the reference's f32 cut), contour rasters, ring tracing and
    simplification on the GPU. Road geometry: synthetic lattice
    coordinates (about 100 m spacing), each road a straight tail -> head
    polyline, the fixture's node weights. Distances are deciseconds (the
    graph's unit); the contour tier comes from the threshold in seconds. The
    whole call runs once as warm-up, then is timed. A sample of origins is
    checked ring for ring against the oracle's pipeline from the origin
    (bounded query, then build_isochrone_geometry_sparse), which is timed on
    one host thread over about 5 s of the batch's origins as the CPU
    baseline."""
    import numpy as np
    import bfphast
    from oracle import oracle as orc
    geo = cch.pop("geo")
    r2s = cch["rank_to_state"]
    ii = np.arange(geo["n_intersections"], dtype=np.int64)
    lat = (500_000_000 + (ii // cols) * 9000).astype(np.int32)
    lon = (30_000_000 + (ii % cols) * 14000).astype(np.int32)
    tail, head = geo["state_tail"][r2s], geo["state_head"][r2s]
    poly = np.stack([np.stack([lat[tail], lon[tail]], 1), np.stack([lat[head], lon[head]], 1)],
                    1).reshape(-1, 2)
    off = np.arange(0, 2 * len(r2s) + 1, 2, dtype=np.uint64)
    w = np.ascontiguousarray(geo["node_weight"][r2s], np.uint32)
    t0 = time.perf_counter()
    gm = bfphast.Geometry(off, poly, w)
    geo_ms = (time.perf_counter() - t0) * 1e3
    origins = np.random.default_rng(seed).integers(0, cch["n"], count).astype(np.uint32)
    thr = np.full(count, 10 * threshold_s, np.uint32)
    tiers = np.full(count, threshold_s, np.uint32)
    bfphast.isochrone_polygons(g, gm, origins, thr, tiers)  # warm-up
    t0 = time.perf_counter()
    rings, ph = bfphast.isochrone_polygons(g, gm, origins, thr, tiers)
    sec = time.perf_counter() - t0
    _, wst = g.isochrone_settled(origins, thr, stats=True)  # the settled-set wave's device split
    wave = {k: round(wst[k], 2) for k in ("upward_ms", "downward_ms", "extract_ms", "total_ms")}
    wave["launches"] = wst["kernel_launches"]
    c = orc.Cch.from_dict(cch)
    # three origins checked ring for ring; the CPU rate over about 5 s of the
    # batch's origins (one host thread, as the reference builds one request)
    pick = [0, count // 2, count - 1][:count]
    order = pick + [k for k in range(count) if k not in pick]
    exact, cpu_s, cpu_n = True, 0.0, 0
    for k in order:
        if k not in pick and cpu_s >= 5.0:
            break
        t0 = time.perf_counter()
        rk, ds = c.bounded_seeded([(int(origins[k]), 0)], int(thr[k]))
        want, _, _ = orc.isochrone_geometry(rk, ds, int(thr[k]), w, off, poly,
                                            "car", tier=threshold_s)
        cpu_s += time.perf_counter() - t0
        cpu_n += 1
        if k in pick:
            exact = exact and bool(np.array_equal(rings[k], want))
    cell, dil, ero, simp = bfphast.contour_config(bfphast.MODE_CAR, threshold_s)
    return {"isochrones": count, "threshold_s": threshold_s, "cell_m": cell,
            "morphology": [dil, ero], "value": round(count / sec, 1), "unit": "polygons/s",
            "ms": round(sec * 1e3, 2),
            "phases_ms": {"settled_sets": round(ph[0], 2), "segments": round(ph[1], 2),
                          "rasters": round(ph[2], 2), "polygons": round(ph[3], 2)},
            "settled_wave": wave,
            "mean_ring_vertices": round(float(np.mean([len(r) for r in rings])), 1),
            "geometry_create_ms": round(geo_ms, 1),
            "bit_exact_sample": {"isochrones": len(pick), "equal": exact},
            "cpu_baseline": {"value": round(cpu_n / cpu_s, 3), "unit": "polygons/s",
                             "cores": 1, "kind": "port",
                             "sample": "%d origins of the batch from the origin (bounded query "
                                       "and geometry), %.1f s" % (cpu_n, cpu_s)},
            "data": "synthetic lattice coordinates, straight tail -> head road polylines"}


def run_tiles(mat, steps, warmup, with_cpu, seed=13):
    """Matrix tile emission (build_matrix_batch / build_matrix_tile_batch,
    flight.rs:432-589) of the 10k x 10k matrix just computed: the four UInt32
    RecordBatch columns. `dense`: every cell, no bound (20 algorithmic bytes
    per cell: the duration read, four u32 written), through
    bf_tile_emit_device on the device-resident matrix, CUDA events on the
    launching stream; `sparse`: a seeded radius mask keeping 20 % of each
    row's destinations and a 30-minute bound, sentinel cells dropped. `e2e`:
    bf_tile_emit with page-locked host arrays (matrix in, columns out). The
    CPU baseline is the oracle's single-threaded builder loop (the reference
    builds a tile on one thread) on a row sample; a row sample of both forms
    is compared column for column."""
    import numpy as np
    import torch
    import bfphast
    from oracle import oracle as orc
    S, T = mat.shape
    n = S * T
    dev = torch.device("cuda:0")
    d_m = torch.from_numpy(np.ascontiguousarray(mat).reshape(-1).view(np.int32)).to(dev)
    d_s = torch.arange(S, dtype=torch.int32, device=dev)
    d_t = torch.arange(T, dtype=torch.int32, device=dev)
    cols = [torch.empty(n, dtype=torch.int32, device=dev) for _ in range(4)]
    rng = np.random.default_rng(seed)
    counts, flat = np.zeros(S, np.int64), []
    for r0 in range(0, S, 1000):  # each destination kept with probability 0.2
        rr, cc = np.nonzero(rng.random((min(1000, S - r0), T)) < 0.2)
        counts[r0:r0 + 1000] = np.bincount(rr, minlength=min(1000, S - r0))
        flat.append(cc.astype(np.uint32))
    mask = np.concatenate(flat)
    moff = np.zeros(S + 1, np.uint64)
    moff[1:] = np.cumsum(counts)
    n_mask = len(mask)
    d_moff = torch.from_numpy(moff.view(np.int64)).to(dev)
    d_mask = torch.from_numpy(mask.view(np.int32)).to(dev)
    bound = 18000  # 30 minutes in the graph's deciseconds
    stream = torch.cuda.current_stream()

    def emit(sparse):
        return bfphast.tile_emit_device(
            d_m.data_ptr(), S, T, d_s.data_ptr(), d_t.data_ptr(), [c.data_ptr() for c in cols],
            bound if sparse else bfphast.INF, d_moff.data_ptr() if sparse else None,
            d_mask.data_ptr() if sparse else None, S if sparse else 0,
            n_mask if sparse else 0, None, sparse, 0, stream.cuda_stream)

    out = {}
    for sparse in (False, True):
        for _ in range(warmup):
            rows = emit(sparse)
        times = []
        for _ in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            rows = emit(sparse)
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        ms = float(np.median(times))
        got = [c[:min(rows, 200 * T)].cpu().numpy().view(np.uint32) for c in cols]
        sample = 200
        want = orc.tile_emit(mat[:sample], sample, T, np.arange(sample), np.arange(T),
                             bound if sparse else orc.INF,
                             (moff[:sample + 1], mask[:int(moff[sample])]) if sparse else None,
                             None, sparse)
        exact = all(np.array_equal(g[:len(w)], w) for g, w in zip(got, want))
        alg = (4 * n + 16 * rows) + ((4 * n_mask) if sparse else 0)
        peak, peak_src = measured_peak()
        out["sparse" if sparse else "dense"] = {
            "rows": int(rows), "ms": round(ms, 3), "cells_per_s": round(n / ms * 1e3, 1),
            # sparse: count, three scan kernels, ordered write
            "gpu_launches": 5 if sparse else 1,
            "roofline": {"bound": "hbm", "achieved": round(alg / ms / 1e6, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(alg / ms / 1e6 / peak, 3),
                         "algorithmic_bytes": int(alg), "peak_source": peak_src},
            "bit_exact_sample": {"rows": sample, "equal": bool(exact)}}
    # end to end: page-locked host matrix in, page-locked columns out
    pin = lambda k: torch.empty(k, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    h_m = pin(n)
    h_m[:] = mat.reshape(-1)
    h_cols = [pin(n) for _ in range(4)]
    sr, tr = np.arange(S, dtype=np.uint32), np.arange(T, dtype=np.uint32)
    for sparse in (False, True):
        kw = dict(threshold=bound if sparse else bfphast.INF,
                  mask=(moff, mask) if sparse else None, sparse=sparse, out=h_cols)
        bfphast.tile_emit(h_m, S, T, sr, tr, **kw)
        t0 = time.perf_counter()
        for _ in range(steps):
            r = bfphast.tile_emit(h_m, S, T, sr, tr, **kw)
        sec = (time.perf_counter() - t0) / steps
        rows = len(r[0])
        out["sparse" if sparse else "dense"]["e2e"] = {
            "value": round(n / sec, 1), "unit": "cells/s", "ms": round(sec * 1e3, 2),
            "h2d_bytes_per_step": int(4 * n + (8 * (S + 1) + 4 * n_mask if sparse else 0)),
            "d2h_bytes_per_step": int(16 * rows)}
    if with_cpu:
        rows_cpu = S  # the whole matrix (about 0.4 s on one host thread)
        t0 = time.perf_counter()
        orc.tile_emit(mat[:rows_cpu], rows_cpu, T, np.arange(rows_cpu), np.arange(T))
        sec = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(rows_cpu * T / sec, 1), "unit": "cells/s",
                               "cores": 1, "kind": "port",
                               "sample": "%d rows x %d targets, dense, %.2f s" % (rows_cpu, T, sec)}
    out["workload"] = "10k x 10k matrix of the country graph (device-resident), original indices = positions"
    return out


def run_customize(cch, steps, warmup, with_cpu):
    """CCH customization of the country topology through bf_cch_customize:
    original arc weights in, customized UP / DOWN weights and middles out
    (customize_cch_time_in_memory's weight stage), host arrays page-locked.
    Device time from the library's CUDA events on its stream; the state
    (1.4 GB of pair slots) exceeds L2. Checked bit for bit against the fixture builder's weights and the
    CPU oracle, which is timed as the reference runs it (apex-parallel
    passes of atomic fetch_min on the host cores)."""
    import numpy as np
    import bfphast
    from oracle import oracle as orc
    import torch
    u = cch.pop("topo")
    d, order = orc.CchTopo.from_upper(u)

    def pinned(n):  # page-locked host arrays, as the e2e contract asks
        return torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)

    nu, nd = len(d.up_tgt), len(d.down_tgt)
    ou, od = pinned(nu), pinned(nd)
    ou[:] = u["orig_up"]
    od[:] = u["orig_down"][order]
    got = (pinned(nu), pinned(nd), pinned(nu), pinned(nd))
    g = bfphast.Cch.from_oracle_topo(d, with_short=False)
    info = g.info()
    for _ in range(max(1, warmup)):
        g.customize(ou, od, out=got)
    dev, tot = [], []
    for _ in range(steps):
        g.customize(ou, od, out=got)
        inf = g.info()
        dev.append(inf["last_device_ms"])
        tot.append(inf["last_total_ms"])
    dev_ms, tot_ms = statistics.median(dev), statistics.median(tot)
    T, E, P = info["triangles"], info["up_edges"] + info["down_edges"], info["pairs"]
    exact = bool(np.array_equal(got[0], u["cust_up"])) and \
        bool(np.array_equal(got[1], u["cust_down"][order]))
    # per pair candidate (two directed triangles): 4 B target index + 16 B
    # target slot; per pair: 16 B slot written + 2 x 4 B edge ids + 2 x 8 B
    # inputs; per edge: 4 B slot id + 8 B slot word + 8 B outputs
    algo = 10 * T + 40 * P + 20 * E
    peak, peak_src = measured_peak()
    roof = {"bound": "hbm", "achieved": round(algo / (dev_ms / 1e3) / 1e9, 1), "peak": peak,
            "unit": "GB/s", "frac": round(algo / (dev_ms / 1e3) / 1e9 / peak, 3),
            "peak_source": peak_src, "algorithmic_bytes": algo,
            "traffic": scaled_traffic("customize_country1000.json", algo),
            "traffic_source": "scaled: DRAM bytes per algorithmic byte of a full customization "
                              "of the 1000x1250 CCH (one-pass capture)"}
    res = {"workload": "country 2000x2500 CCH: %d ranks, %d UP + %d DOWN edges, %d triangles"
                       % (info["n_nodes"], info["up_edges"], info["down_edges"], T),
           "metric": "customization time", "value": round(dev_ms, 3), "unit": "ms",
           "higher_is_better": False, "triangles_per_s": round(T / (dev_ms / 1e3), 1),
           "levels": info["levels"], "pairs": P, "plan_ms": round(info["plan_ms"], 1),
           "target_index": info["target_index"], "steps": steps,
           "e2e": {"value": round(tot_ms, 3), "unit": "ms", "h2d_bytes_per_step": 4 * E,
                   "d2h_bytes_per_step": 16 * E},
           "gpu_launches": info["levels"] + 4, "roofline": roof,
           "bit_exact_vs_builder": exact}
    if with_cpu:
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        w = d.relax(ou, od, threads=threads)
        cpu_s = time.perf_counter() - t0
        res["bit_exact_vs_oracle"] = all(bool(np.array_equal(a, b)) for a, b in zip(got, w[:4]))
        res["cpu_baseline"] = {"value": round(cpu_s * 1e3, 1), "unit": "ms", "cores": threads,
                               "kind": "port",
                               "sample": "the full topology, %d apex-parallel passes" % w[4]}
    g.close()
    return res


def scaled_traffic(name, alg_bytes):
    """DRAM traffic for `alg_bytes` algorithmic bytes: the committed ncu
    summary's DRAM bytes per algorithmic byte (a smaller case of the same
    kernels) times alg_bytes, or None."""
    prof = ROOT / "profiles" / name
    if not prof.exists():
        return None
    try:
        ratio = json.loads(prof.read_text()).get("traffic_per_alg_byte")
    except (ValueError, OSError):
        return None
    return int(round(ratio * alg_bytes)) if ratio else None


def run_reference(args):
    """The reference path on the host cores: the CPU restatement of
    BatchedPhastEngine::compute_matrix_flat_soa (K = 8, rayon-shaped threads),
    each step a bounded row sample of the same 10k x 10k workload (the Rust
    reference cannot be compiled here)."""
    cch, src, tgt = build_workload(args, seed=42)
    threads = os.cpu_count() or 1
    rows = 8 * threads  # one K = 8 batch per thread per step
    for _ in range(args.warmup):
        cpu_sample(cch, src, tgt, 0, rows=8)
    vals = []
    for _ in range(args.steps):
        d, _, _ = cpu_sample(cch, src, tgt, 0, rows=rows)
        vals.append(d["value"])
    value = statistics.median(vals)
    cb = dict(d)
    cb["value"] = value
    return {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(rows * len(tgt) / value * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded country-scale lattice road graph, CCH built in-run)",
            "config": {"workload": "country 2000x2500 lattice, 10k x 10k matrix, row sample",
                       "n_nodes": cch["n"], "sources": len(src), "targets": len(tgt)},
            "cpu_baseline": cb,
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        tdist.init_process_group("nccl")
        dist = tdist
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        if dist:
            dist.destroy_process_group()
        return
    import numpy as np
    if args.tiles_synthetic:
        # durations uniform above the 30-minute bound (18000 deciseconds)
        # except a seeded 2.1 % within it, as in the country 10k x 10k matrix
        rng = np.random.default_rng(1)
        mat = rng.integers(18001, 200000, (args.sources, args.targets), dtype=np.uint32)
        inb = rng.random(mat.shape) < 0.021
        mat[inb] = rng.integers(0, 18001, int(inb.sum()), dtype=np.uint32)
        if rank == 0:
            print(json.dumps({"tiles": run_tiles(mat, args.steps, args.warmup, False),
                              "data": "synthetic 10k x 10k matrix, 2.1 % of cells within "
                                      "the 30-minute bound"}), flush=True)
        if dist:
            dist.destroy_process_group()
        return
    res, cch, src, tgt, out = run_ours(args, rank, world, dist)
    if rank == 0:
        if not args.no_cpu:
            cb, pick, m = cpu_sample(cch, src, tgt, args.cpu_sample_s)
            res["cpu_baseline"] = cb
            res["bit_exact_sample"] = {"rows": len(pick), "targets": len(tgt),
                                       "equal": bool(np.array_equal(out[pick], m))}
        print(json.dumps(res), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
