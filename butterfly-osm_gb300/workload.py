"""Seeded workloads of the K-lane PHAST engine.

The configurations restate the reference's measured shapes on synthetic road
graphs (the reference's own data, a Belgium extract, is not available):

  grid100     100 x 100 jittered grid (cch KIND_GRID), 100 x 100 matrix
  country     2000 x 2500 lattice with road hierarchy (cch KIND_COUNTRY)
              - 1000 x 1000 matrix, plain sweep, K = 32
              - 10000 x 10000 matrix, batched engine
              - 100000 bulk isochrones, thresholds {300,600,1200,1800,3600} s
              - serving mix: Poisson arrivals, 70% matrices / 30% isochrones

Sources and targets are uniform over CCH ranks like bench/main.rs:1295-1306 of
the reference (which draws them with a seeded StdRng, seed 42). Sampling here
uses splitmix64 so the same seed gives the same ids on every platform.
Durations are deciseconds; a threshold of t seconds is 10 * t.
"""
import numpy as np

MASK = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed, count):
    """count consecutive splitmix64 outputs for a seed (uint64 array)."""
    with np.errstate(over="ignore"):
        i = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform_ids(n, count, seed):
    """count ids uniform over [0, n) (multiply-shift of the high 32 bits)."""
    hi = splitmix64(seed, count) >> np.uint64(32)
    return ((hi * np.uint64(n)) >> np.uint64(32)).astype(np.uint32)


def sources_targets(n, S, T, seed=42):
    return uniform_ids(n, S, seed), uniform_ids(n, T, seed + 1)


ISO_THRESHOLDS_S = (300, 600, 1200, 1800, 3600)


def isochrone_workload(n, count, seed=42):
    """Origins uniform over ranks, thresholds (deciseconds) uniform over the set."""
    origins = uniform_ids(n, count, seed + 2)
    pick = uniform_ids(len(ISO_THRESHOLDS_S), count, seed + 3)
    thr = np.array(ISO_THRESHOLDS_S, dtype=np.uint32)[pick] * np.uint32(10)
    return origins, thr


GRID100 = dict(kind=0, rows=100, cols=100)
COUNTRY = dict(kind=1, rows=2000, cols=2500)
