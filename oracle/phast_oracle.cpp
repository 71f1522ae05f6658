// phast_oracle.cpp — CPU oracle for the K-lane PHAST engine.
//
// TEST INFRASTRUCTURE ONLY. This file is a plain restatement of the
// reference's CPU PHAST code paths. It is used by tests/, by the smoke check
// and by bench.py's CPU-baseline leg as the checker and as the timed CPU
// baseline. It is never linked into or called by the product library.
//
// Every function cites the reference function it restates (paths relative to
// the butterfly-osm repository). Arithmetic is u32 with saturating add and
// u32::MAX (0xFFFFFFFF) as "unreachable", exactly as in the reference.

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <functional>
#include <queue>
#include <vector>

namespace {

using u32 = uint32_t;
using u64 = uint64_t;
constexpr u32 INF = 0xFFFFFFFFu;

inline u32 sat_add(u32 a, u32 b) {
  u64 s = (u64)a + b;
  return s >= INF ? INF : (u32)s;
}

struct Csr {
  const u64* off;
  const u32* tgt;
  const u32* w;
};

using MinHeap = std::priority_queue<std::pair<u32, u32>, std::vector<std::pair<u32, u32>>,
                                    std::greater<std::pair<u32, u32>>>;

// Upward Dijkstra from one origin writing into dist (stride elements apart);
// bounded by `threshold` when `bounded` is set (phast.rs:308-315 early stop).
void upward(const Csr& up, u32 origin, u32* dist, size_t stride, bool bounded, u32 threshold) {
  MinHeap pq;
  pq.push({0u, origin});
  while (!pq.empty()) {
    auto [d, u] = pq.top();
    pq.pop();
    if (bounded && d > threshold) break;
    if (d > dist[(size_t)u * stride]) continue;
    for (u64 i = up.off[u]; i < up.off[u + 1]; ++i) {
      u32 w = up.w[i];
      if (w == INF) continue;
      u32 v = up.tgt[i];
      u32 nd = sat_add(d, w);
      if (nd < dist[(size_t)v * stride]) {
        dist[(size_t)v * stride] = nd;
        pq.push({nd, v});
      }
    }
  }
}

}  // namespace

extern "C" {

// PhastEngine::query — route/src/range/phast.rs:155-263.
// Unbounded single-source PHAST over the rank-aligned CCH (INF weights are
// skipped in both phases, phast.rs:191-193 and :238-240).
void orc_phast_query(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                     const u64* dn_off, const u32* dn_tgt, const u32* dn_w, u32 origin,
                     u32* dist) {
  std::fill(dist, dist + n, INF);
  dist[origin] = 0;
  upward({up_off, up_tgt, up_w}, origin, dist, 1, false, INF);
  for (u32 r = n; r-- > 0;) {
    u32 du = dist[r];
    if (du == INF) continue;
    for (u64 i = dn_off[r]; i < dn_off[r + 1]; ++i) {
      u32 w = dn_w[i];
      if (w == INF) continue;
      u32 v = dn_tgt[i];
      u32 nd = sat_add(du, w);
      if (nd < dist[v]) dist[v] = nd;
    }
  }
}

// BatchedPhastEngine::query_batch — route/src/matrix/batched_phast.rs:131-260.
// k <= 8 sources; K separate upward heaps, one downward scan that skips a node
// when every lane is unreachable (:220-223). Output is AoS: dist[lane*n+node].
int orc_query_batch(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                    const u64* dn_off, const u32* dn_tgt, const u32* dn_w, const u32* src,
                    u32 k, u32* dist) {
  if (k > 8) return 1;  // batched_phast.rs:132 asserts sources.len() <= K_LANES
  std::fill(dist, dist + (size_t)k * n, INF);
  for (u32 l = 0; l < k; ++l) dist[(size_t)l * n + src[l]] = 0;
  Csr up{up_off, up_tgt, up_w};
  for (u32 l = 0; l < k; ++l) upward(up, src[l], dist + (size_t)l * n, 1, false, INF);
  for (u32 r = n; r-- > 0;) {
    if (dn_off[r] == dn_off[r + 1]) continue;
    bool any = false;
    for (u32 l = 0; l < k; ++l) any |= dist[(size_t)l * n + r] != INF;
    if (!any) continue;
    for (u64 i = dn_off[r]; i < dn_off[r + 1]; ++i) {
      u32 w = dn_w[i];
      if (w == INF) continue;
      u32 v = dn_tgt[i];
      for (u32 l = 0; l < k; ++l) {
        u32 du = dist[(size_t)l * n + r];
        if (du != INF) {
          u32 nd = sat_add(du, w);
          u32& dv = dist[(size_t)l * n + v];
          if (nd < dv) dv = nd;
        }
      }
    }
  }
  return 0;
}

// BatchedPhastEngine::query_batch_bounded — batched_phast.rs:271-445.
// Per-lane upward early stop at d > T, per-lane active blocks of 512 ranks,
// downward relaxes only new_dist <= T. Values > T are implementation
// artefacts in the reference too; only entries <= T are meaningful.
int orc_query_batch_bounded(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                            const u64* dn_off, const u32* dn_tgt, const u32* dn_w,
                            const u32* src, u32 k, u32 threshold, u32* dist) {
  if (k > 8) return 1;
  const u32 BS = 512;
  u32 nb = (n + BS - 1) / BS;
  std::vector<std::vector<uint8_t>> active(k, std::vector<uint8_t>(nb, 0));
  std::fill(dist, dist + (size_t)k * n, INF);
  for (u32 l = 0; l < k; ++l) {
    dist[(size_t)l * n + src[l]] = 0;
    active[l][src[l] / BS] = 1;
  }
  for (u32 l = 0; l < k; ++l) {
    u32* d = dist + (size_t)l * n;
    MinHeap pq;
    pq.push({0u, src[l]});
    while (!pq.empty()) {
      auto [du, u] = pq.top();
      pq.pop();
      if (du > threshold) break;
      if (du > d[u]) continue;
      for (u64 i = up_off[u]; i < up_off[u + 1]; ++i) {
        u32 w = up_w[i];
        if (w == INF) continue;
        u32 v = up_tgt[i], nd = sat_add(du, w);
        if (nd < d[v]) {
          d[v] = nd;
          pq.push({nd, v});
          if (nd <= threshold) active[l][v / BS] = 1;
        }
      }
    }
  }
  std::vector<uint8_t> lane_on(k, 0);
  for (u32 l = 0; l < k; ++l)
    for (u32 b = 0; b < nb; ++b) lane_on[l] |= active[l][b];
  for (u32 r = n; r-- > 0;) {
    if (dn_off[r] == dn_off[r + 1]) continue;
    u32 blk = r / BS;
    bool any = false;
    for (u32 l = 0; l < k; ++l) any |= lane_on[l] && active[l][blk];
    if (!any) continue;
    for (u64 i = dn_off[r]; i < dn_off[r + 1]; ++i) {
      u32 w = dn_w[i];
      if (w == INF) continue;
      u32 v = dn_tgt[i];
      for (u32 l = 0; l < k; ++l) {
        if (!lane_on[l] || !active[l][blk]) continue;
        u32 du = dist[(size_t)l * n + r];
        if (du == INF) continue;
        u32 nd = sat_add(du, w);
        u32& dv = dist[(size_t)l * n + v];
        if (nd <= threshold && nd < dv) {
          dv = nd;
          active[l][v / BS] = 1;
        }
      }
    }
  }
  return 0;
}

// BatchedPhastEngine::compute_matrix_flat_soa + query_batch_soa_raw —
// batched_phast.rs:756-917. K = 8 lanes in SoA layout dist[node*8 + lane];
// sources chunked by 8; the row-major S x T matrix is gathered from the SoA
// slab. n_threads > 1 runs independent K-batches on worker threads, the
// rayon shape of bucket_ch.rs:6814-6823. Returns the number of threads used.
int orc_matrix_soa(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                   const u64* dn_off, const u32* dn_tgt, const u32* dn_w, const u32* src,
                   u64 S, const u32* tgt, u64 T, u32* out, int n_threads) {
  const u32 K = 8;
  u64 nbatch = (S + K - 1) / K;
  if (n_threads <= 0) n_threads = omp_get_max_threads();
  int used = 1;
#pragma omp parallel num_threads(n_threads)
  {
#pragma omp single
    used = omp_get_num_threads();
    std::vector<u32> soa((size_t)n * K);
    Csr up{up_off, up_tgt, up_w};
#pragma omp for schedule(dynamic, 1)
    for (u64 b = 0; b < nbatch; ++b) {
      u64 s0 = b * K;
      u32 k = (u32)std::min<u64>(K, S - s0);
      std::fill(soa.begin(), soa.end(), INF);
      for (u32 l = 0; l < k; ++l) soa[(size_t)src[s0 + l] * K + l] = 0;
      for (u32 l = 0; l < k; ++l) upward(up, src[s0 + l], soa.data() + l, K, false, INF);
      for (u32 r = n; r-- > 0;) {
        if (dn_off[r] == dn_off[r + 1]) continue;
        const u32* ur = soa.data() + (size_t)r * K;
        bool any = false;
        for (u32 l = 0; l < k; ++l) any |= ur[l] != INF;
        if (!any) continue;
        u32 du[K];
        for (u32 l = 0; l < K; ++l) du[l] = l < k ? ur[l] : INF;
        for (u64 i = dn_off[r]; i < dn_off[r + 1]; ++i) {
          u32 w = dn_w[i];
          if (w == INF) continue;
          u32* vr = soa.data() + (size_t)dn_tgt[i] * K;
          for (u32 l = 0; l < k; ++l)
            if (du[l] != INF) {
              u32 nd = sat_add(du[l], w);
              if (nd < vr[l]) vr[l] = nd;
            }
        }
      }
      for (u32 l = 0; l < k; ++l)
        for (u64 t = 0; t < T; ++t) out[(s0 + l) * T + t] = soa[(size_t)tgt[t] * K + l];
    }
  }
  return used;
}

// run_phast_bounded_fast_seeded — route/src/server/isochrone_handler.rs:338-491
// with PhastState (:132-227). Multi-seed (rank, cost) init, bounded upward
// heap (break at d > T), block-gated downward scan (4096-rank blocks, skip
// d_u > T), and the ascending-rank collection of settled (rank, d <= T).
// Writes up to `cap` pairs; returns the number of settled pairs.
u64 orc_phast_bounded_seeded(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                             const u64* dn_off, const u32* dn_tgt, const u32* dn_w,
                             const u32* seed_rank, const u32* seed_cost, u32 n_seeds,
                             u32 threshold, u32* out_rank, u32* out_dist, u64 cap) {
  const u32 BS = 4096;
  u32 nb = (n + BS - 1) / BS;
  // a fresh generation per call: version == 1 marks "set this query"
  std::vector<u32> dist(n, INF);
  std::vector<uint8_t> version(n, 0), block(nb, 0);
  auto get = [&](u32 v) { return version[v] ? dist[v] : INF; };
  auto set = [&](u32 v, u32 d) {
    dist[v] = d;
    version[v] = 1;
    block[v / BS] = 1;
  };
  for (u32 i = 0; i < n_seeds; ++i)
    if (seed_cost[i] < get(seed_rank[i])) set(seed_rank[i], seed_cost[i]);
  MinHeap pq;
  for (u32 i = 0; i < n_seeds; ++i)
    if (get(seed_rank[i]) == seed_cost[i]) pq.push({seed_cost[i], seed_rank[i]});
  while (!pq.empty()) {
    auto [d, u] = pq.top();
    pq.pop();
    if (d > threshold) break;
    if (d > get(u)) continue;
    for (u64 i = up_off[u]; i < up_off[u + 1]; ++i) {
      u32 v = up_tgt[i], nd = sat_add(d, up_w[i]);
      if (nd < get(v)) {
        set(v, nd);
        pq.push({nd, v});
      }
    }
  }
  for (u32 b = nb; b-- > 0;) {
    if (!block[b]) continue;
    u32 lo = b * BS, hi = std::min(n, lo + BS);
    for (u32 r = hi; r-- > lo;) {
      u32 du = get(r);
      if (du == INF || du > threshold) continue;
      for (u64 i = dn_off[r]; i < dn_off[r + 1]; ++i) {
        u32 v = dn_tgt[i], nd = sat_add(du, dn_w[i]);
        if (nd < get(v)) set(v, nd);
      }
    }
  }
  u64 cnt = 0;
  for (u32 b = 0; b < nb; ++b) {
    if (!block[b]) continue;
    u32 lo = b * BS, hi = std::min(n, lo + BS);
    for (u32 r = lo; r < hi; ++r)
      if (version[r] && dist[r] <= threshold) {
        if (cnt < cap) {
          out_rank[cnt] = r;
          out_dist[cnt] = dist[r];
        }
        ++cnt;
      }
  }
  return cnt;
}

// run_phast_bounded_fast_seeded_2ch — route/src/server/isochrone_handler.rs:500-625.
// As orc_phast_bounded_seeded with a length-along-time channel carried in
// lockstep: seeds (rank, time, len) enter only when their time is below the
// rank's current time (:527-531); relaxations adopt a strictly smaller time,
// or an equal finite time with a strictly shorter length, and re-push in the
// upward phase (:543-571, lazy lexicographic tie-break); the downward scan
// applies the same rule without re-push (:592-612). up_l / dn_l are the
// length weights aligned with up_w / dn_w; edges with time INF are absent
// from the reference flats and skipped here. Writes up to `cap` triples in
// ascending rank; returns the number of settled nodes (time <= threshold).
u64 orc_phast_bounded_seeded_2ch(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                                 const u64* dn_off, const u32* dn_tgt, const u32* dn_w,
                                 const u32* up_l, const u32* dn_l, const u32* seed_rank,
                                 const u32* seed_cost, const u32* seed_len, u32 n_seeds,
                                 u32 threshold, u32* out_rank, u32* out_time, u32* out_len,
                                 u64 cap) {
  const u32 BS = 4096;
  u32 nb = (n + BS - 1) / BS;
  std::vector<u32> dist(n, INF), len(n, INF);
  std::vector<uint8_t> version(n, 0), block(nb, 0);
  auto get = [&](u32 v) { return version[v] ? dist[v] : INF; };
  auto get_len = [&](u32 v) { return version[v] ? len[v] : INF; };
  auto set = [&](u32 v, u32 d, u32 l) {
    dist[v] = d;
    len[v] = l;
    version[v] = 1;
    block[v / BS] = 1;
  };
  for (u32 i = 0; i < n_seeds; ++i)
    if (seed_cost[i] < get(seed_rank[i])) set(seed_rank[i], seed_cost[i], seed_len[i]);
  MinHeap pq;
  for (u32 i = 0; i < n_seeds; ++i)
    if (get(seed_rank[i]) == seed_cost[i]) pq.push({seed_cost[i], seed_rank[i]});
  while (!pq.empty()) {
    auto [d, u] = pq.top();
    pq.pop();
    if (d > threshold) break;
    if (d > get(u)) continue;
    const u32 lu = get_len(u);
    for (u64 i = up_off[u]; i < up_off[u + 1]; ++i) {
      if (up_w[i] == INF) continue;
      const u32 v = up_tgt[i], nt = sat_add(d, up_w[i]), ct = get(v);
      if (nt < ct) {
        set(v, nt, sat_add(lu, up_l[i]));
        pq.push({nt, v});
      } else if (nt == ct && ct != INF) {
        const u32 nl = sat_add(lu, up_l[i]);
        if (nl < get_len(v)) {
          set(v, nt, nl);
          pq.push({nt, v});
        }
      }
    }
  }
  for (u32 b = nb; b-- > 0;) {
    if (!block[b]) continue;
    u32 lo = b * BS, hi = std::min(n, lo + BS);
    for (u32 r = hi; r-- > lo;) {
      const u32 du = get(r);
      if (du == INF || du > threshold) continue;
      const u32 lu = get_len(r);
      for (u64 i = dn_off[r]; i < dn_off[r + 1]; ++i) {
        if (dn_w[i] == INF) continue;
        const u32 v = dn_tgt[i], nt = sat_add(du, dn_w[i]), ct = get(v);
        if (nt < ct) {
          set(v, nt, sat_add(lu, dn_l[i]));
        } else if (nt == ct && ct != INF) {
          const u32 nl = sat_add(lu, dn_l[i]);
          if (nl < get_len(v)) set(v, nt, nl);
        }
      }
    }
  }
  u64 cnt = 0;
  for (u32 b = 0; b < nb; ++b) {
    if (!block[b]) continue;
    u32 lo = b * BS, hi = std::min(n, lo + BS);
    for (u32 r = lo; r < hi; ++r)
      if (version[r] && dist[r] <= threshold) {
        if (cnt < cap) {
          out_rank[cnt] = r;
          out_time[cnt] = dist[r];
          out_len[cnt] = len[r];
        }
        ++cnt;
      }
  }
  return cnt;
}

// Bulk isochrone reachable sets: for origin i, bit r of row i is set iff rank
// r is settled with d <= T_i by run_phast_bounded_fast_seeded (the
// `reachable_edges` set of isochrone_handler.rs:1271-1278). Rows are
// ceil(n/64) u64 words. counts[i] = popcount of row i.
void orc_isochrone_bitsets(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                           const u64* dn_off, const u32* dn_tgt, const u32* dn_w,
                           const u32* origins, const u32* thresholds, u64 n_orig, u64* bits,
                           u64* counts, int n_threads) {
  u64 words = (n + 63) / 64;
  if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel num_threads(n_threads)
  {
    std::vector<u32> rk(n), ds(n);
#pragma omp for schedule(dynamic, 1)
    for (u64 i = 0; i < n_orig; ++i) {
      u32 zero = 0;
      u64 c = orc_phast_bounded_seeded(n, up_off, up_tgt, up_w, dn_off, dn_tgt, dn_w,
                                       &origins[i], &zero, 1, thresholds[i], rk.data(),
                                       ds.data(), n);
      u64* row = bits + i * words;
      std::memset(row, 0, words * 8);
      for (u64 j = 0; j < c; ++j) row[rk[j] >> 6] |= 1ull << (rk[j] & 63);
      counts[i] = c;
    }
  }
}

// Plain Dijkstra over the edge-based graph (validate/cch_correctness.rs
// pattern: an independent ground truth for the CCH pipeline).
void orc_dijkstra_ebg(u32 n, const u64* arc_off, const u32* arc_dst, const u32* arc_w,
                      u32 origin, u32* dist) {
  std::fill(dist, dist + n, INF);
  dist[origin] = 0;
  MinHeap pq;
  pq.push({0u, origin});
  while (!pq.empty()) {
    auto [d, u] = pq.top();
    pq.pop();
    if (d > dist[u]) continue;
    for (u64 i = arc_off[u]; i < arc_off[u + 1]; ++i) {
      u32 v = arc_dst[i], nd = sat_add(d, arc_w[i]);
      if (nd < dist[v]) {
        dist[v] = nd;
        pq.push({nd, v});
      }
    }
  }
}

// PhastEngine::query_block_gated_reverse (all-to-one) — phast.rs:879-1001.
// Upward over the DOWN-reverse flat (in-edges of DOWN, bucket_ch.rs:355-418),
// then a pull over UP edges in descending rank order. rev_off/rev_src/rev_w
// is the DownReverseAdjFlat; up_* the UpAdjFlat.
void orc_phast_reverse(u32 n, const u64* up_off, const u32* up_tgt, const u32* up_w,
                       const u64* rev_off, const u32* rev_src, const u32* rev_w, u32 target,
                       u32* dist) {
  std::fill(dist, dist + n, INF);
  dist[target] = 0;
  upward({rev_off, rev_src, rev_w}, target, dist, 1, false, INF);
  for (u32 r = n; r-- > 0;) {
    u32 best = dist[r];
    for (u64 i = up_off[r]; i < up_off[r + 1]; ++i) {
      u32 w = up_w[i];
      if (w == INF) continue;
      u32 dv = dist[up_tgt[i]];
      if (dv == INF) continue;
      best = std::min(best, sat_add(dv, w));
    }
    dist[r] = best;
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// CCH customization on the reference's directed rank-space topology
// (formats/cch_topo.rs:250-290, CchTopo): UP edges u -> v (v > u) and DOWN
// edges u -> v (v < u) as two CSRs, targets ascending within each node.
// Middle u32::MAX marks an original arc (cch_topo.rs:268).

namespace {
struct CTopo {
  u32 n;
  const u64* uo;
  const u32* ut;
  const u64* dof;
  const u32* dt;
};

// find_edge_index (customization.rs:1507-1521): binary search for target v
// in u's list; ~0 when absent.
u64 c_find(const u64* off, const u32* tgt, u32 u, u32 v) {
  const u32* lo = tgt + off[u];
  const u32* hi = tgt + off[u + 1];
  const u32* it = std::lower_bound(lo, hi, v);
  return (it != hi && *it == v) ? (u64)(it - tgt) : ~0ull;
}

// build_reverse_down_adj_for_relax (customization.rs:832-875): for every m
// the DOWN edges x -> m, sources in ascending x.
struct RevDown {
  std::vector<u64> off;
  std::vector<u32> src;
  std::vector<u64> eid;
};
RevDown c_rev_down(const CTopo& t) {
  RevDown r;
  r.off.assign((size_t)t.n + 1, 0);
  for (u64 i = 0; i < t.dof[t.n]; ++i) r.off[t.dt[i] + 1]++;
  for (u32 m = 0; m < t.n; ++m) r.off[m + 1] += r.off[m];
  r.src.resize(t.dof[t.n]);
  r.eid.resize(t.dof[t.n]);
  std::vector<u64> pos(r.off.begin(), r.off.end() - 1);
  for (u32 u = 0; u < t.n; ++u)
    for (u64 i = t.dof[u]; i < t.dof[u + 1]; ++i) {
      const u64 p = pos[t.dt[i]]++;
      r.src[p] = u;
      r.eid[p] = i;
    }
  return r;
}

// One apex-ordered pass over every triangle x -> m -> y (customization.rs
// :1110-1170): calls f(x, y, m, down edge x->m, up edge m->y, target edge,
// target is UP) for each pair with both legs present and y != x.
template <class F>
void c_triangles(const CTopo& t, const RevDown& r, F&& f) {
  for (u32 m = 0; m < t.n; ++m)
    for (u64 ir = r.off[m]; ir < r.off[m + 1]; ++ir) {
      const u32 x = r.src[ir];
      for (u64 j = t.uo[m]; j < t.uo[m + 1]; ++j) {
        const u32 y = t.ut[j];
        if (y == x) continue;
        if (y > x) {
          const u64 e = c_find(t.uo, t.ut, x, y);
          if (e != ~0ull) f(m, r.eid[ir], j, e, true);
        } else {
          const u64 e = c_find(t.dof, t.dt, x, y);
          if (e != ~0ull) f(m, r.eid[ir], j, e, false);
        }
      }
    }
}
}  // namespace

extern "C" {
// triangle_relax_parallel (customization.rs:1083-1200): packed
// (weight << 32 | middle) per edge, seeded from the given weights and
// middles; every pass offers each triangle's (w(x->m) + w(m->y), m) to edge
// x -> y (legs with weight u32::MAX skipped, the sum saturating) and keeps
// the smaller packed value; passes repeat until one changes nothing. The
// weight and middle arrays are updated in place. Returns the number of
// passes, 0 when 100 passes did not converge (the reference panics there).
u32 orc_cch_relax(u32 n, const u64* uo, const u32* ut, const u64* dof, const u32* dt, u32* up_w,
                  u32* dn_w, u32* up_mid, u32* dn_mid) {
  const CTopo t{n, uo, ut, dof, dt};
  const RevDown r = c_rev_down(t);
  const u64 nu = uo[n], nd = dof[n];
  std::vector<u64> pu(nu), pd(nd);
  for (u64 e = 0; e < nu; ++e) pu[e] = ((u64)up_w[e] << 32) | up_mid[e];
  for (u64 e = 0; e < nd; ++e) pd[e] = ((u64)dn_w[e] << 32) | dn_mid[e];
  u32 passes = 0;
  for (;;) {
    ++passes;
    u64 updates = 0;
    c_triangles(t, r, [&](u32 m, u64 exm, u64 emy, u64 e, bool up) {
      const u32 wxm = (u32)(pd[exm] >> 32), wmy = (u32)(pu[emy] >> 32);
      if (wxm == INF || wmy == INF) return;
      const u64 np = ((u64)sat_add(wxm, wmy) << 32) | m;
      u64& slot = up ? pu[e] : pd[e];
      if (np < slot) {
        slot = np;
        ++updates;
      }
    });
    if (!updates) break;
    if (passes >= 100) return 0;
  }
  for (u64 e = 0; e < nu; ++e) {
    up_w[e] = (u32)(pu[e] >> 32);
    up_mid[e] = (u32)pu[e];
  }
  for (u64 e = 0; e < nd; ++e) {
    dn_w[e] = (u32)(pd[e] >> 32);
    dn_mid[e] = (u32)pd[e];
  }
  return passes;
}

// triangle_relax_parallel as the reference runs it (customization.rs:1083-1200):
// each pass spreads the apexes over n_threads host threads (rayon's
// into_par_iter), every candidate lowers its target with an atomic fetch_min
// on the packed value, and passes repeat until one changes nothing. The
// fixed point is the same as orc_cch_relax's; this is the timed CPU
// baseline. Returns the number of passes (0: no convergence in 100).
u32 orc_cch_relax_par(u32 n, const u64* uo, const u32* ut, const u64* dof, const u32* dt,
                      u32* up_w, u32* dn_w, u32* up_mid, u32* dn_mid, int n_threads,
                      int* threads_used) {
  const CTopo t{n, uo, ut, dof, dt};
  const RevDown r = c_rev_down(t);
  const u64 nu = uo[n], nd = dof[n];
  std::vector<std::atomic<u64>> pu(nu), pd(nd);
  for (u64 e = 0; e < nu; ++e) pu[e].store(((u64)up_w[e] << 32) | up_mid[e], std::memory_order_relaxed);
  for (u64 e = 0; e < nd; ++e) pd[e].store(((u64)dn_w[e] << 32) | dn_mid[e], std::memory_order_relaxed);
  if (n_threads <= 0) n_threads = omp_get_max_threads();
  auto fetch_min = [](std::atomic<u64>& a, u64 v) {
    u64 cur = a.load(std::memory_order_relaxed);
    while (v < cur && !a.compare_exchange_weak(cur, v, std::memory_order_relaxed)) {
    }
    return v < cur;
  };
  u32 passes = 0;
  int used = 1;
  for (;;) {
    ++passes;
    u64 updates = 0;
#pragma omp parallel num_threads(n_threads) reduction(+ : updates)
    {
#pragma omp single
      used = omp_get_num_threads();
#pragma omp for schedule(dynamic, 256)
      for (long long mm = 0; mm < (long long)n; ++mm) {
        const u32 m = (u32)mm;
        for (u64 ir = r.off[m]; ir < r.off[m + 1]; ++ir) {
          const u32 x = r.src[ir];
          const u32 wxm = (u32)(pd[r.eid[ir]].load(std::memory_order_relaxed) >> 32);
          if (wxm == INF) continue;
          for (u64 j = uo[m]; j < uo[m + 1]; ++j) {
            const u32 y = ut[j];
            if (y == x) continue;
            const u32 wmy = (u32)(pu[j].load(std::memory_order_relaxed) >> 32);
            if (wmy == INF) continue;
            const u64 np = ((u64)sat_add(wxm, wmy) << 32) | m;
            if (y > x) {
              const u64 e = c_find(uo, ut, x, y);
              if (e != ~0ull && fetch_min(pu[e], np)) ++updates;
            } else {
              const u64 e = c_find(dof, dt, x, y);
              if (e != ~0ull && fetch_min(pd[e], np)) ++updates;
            }
          }
        }
      }
    }
    if (!updates) break;
    if (passes >= 100) return 0;
  }
  if (threads_used) *threads_used = used;
  for (u64 e = 0; e < nu; ++e) {
    const u64 v = pu[e].load(std::memory_order_relaxed);
    up_w[e] = (u32)(v >> 32);
    up_mid[e] = (u32)v;
  }
  for (u64 e = 0; e < nd; ++e) {
    const u64 v = pd[e].load(std::memory_order_relaxed);
    dn_w[e] = (u32)(v >> 32);
    dn_mid[e] = (u32)v;
  }
  return passes;
}

// triangle_relax_lex_parallel (customization.rs:1253-1436): packed
// (time << 32 | length) per edge, both components summed separately with
// saturation and compared as one u64 (time first, then length), passes until
// no update. Then, on the converged values, every SHORTCUT edge elects the
// smallest apex whose triangle sum equals its packed value; a shortcut with
// no such apex, and every original edge, keeps the given middle. Times and
// middles are updated in place; lengths are read only.
u32 orc_cch_relax_lex(u32 n, const u64* uo, const u32* ut, const u64* dof, const u32* dt,
                      const uint8_t* up_short, const uint8_t* dn_short, u32* up_t, u32* dn_t,
                      const u32* up_l, const u32* dn_l, u32* up_mid, u32* dn_mid) {
  const CTopo t{n, uo, ut, dof, dt};
  const RevDown r = c_rev_down(t);
  const u64 nu = uo[n], nd = dof[n];
  std::vector<u64> pu(nu), pd(nd);
  for (u64 e = 0; e < nu; ++e) pu[e] = ((u64)up_t[e] << 32) | up_l[e];
  for (u64 e = 0; e < nd; ++e) pd[e] = ((u64)dn_t[e] << 32) | dn_l[e];
  auto cand = [](u64 a, u64 b) {
    return ((u64)sat_add((u32)(a >> 32), (u32)(b >> 32)) << 32) | sat_add((u32)a, (u32)b);
  };
  u32 passes = 0;
  for (;;) {
    ++passes;
    u64 updates = 0;
    c_triangles(t, r, [&](u32, u64 exm, u64 emy, u64 e, bool up) {
      if ((u32)(pd[exm] >> 32) == INF || (u32)(pu[emy] >> 32) == INF) return;
      const u64 np = cand(pd[exm], pu[emy]);
      u64& slot = up ? pu[e] : pd[e];
      if (np < slot) {
        slot = np;
        ++updates;
      }
    });
    if (!updates) break;
    if (passes >= 100) return 0;
  }
  std::vector<u32> mu(nu, INF), md(nd, INF);
  c_triangles(t, r, [&](u32 m, u64 exm, u64 emy, u64 e, bool up) {
    if ((u32)(pd[exm] >> 32) == INF || (u32)(pu[emy] >> 32) == INF) return;
    const u64 np = cand(pd[exm], pu[emy]);
    if (up) {
      if (up_short[e] && np == pu[e]) mu[e] = std::min(mu[e], m);
    } else {
      if (dn_short[e] && np == pd[e]) md[e] = std::min(md[e], m);
    }
  });
  for (u64 e = 0; e < nu; ++e) {
    up_t[e] = (u32)(pu[e] >> 32);
    if (mu[e] != INF) up_mid[e] = mu[e];
  }
  for (u64 e = 0; e < nd; ++e) {
    dn_t[e] = (u32)(pd[e] >> 32);
    if (md[e] != INF) dn_mid[e] = md[e];
  }
  return passes;
}

// bottom_up_customize / bottom_up_with_external_middles
// (customization.rs:953-1052): ranks ascending; within a rank its DOWN edges
// by ascending target, then its UP edges. An original edge takes its
// original weight; a shortcut u -> v with middle m takes
// w(u -> m) + w(m -> v) (saturating), a missing leg reading u32::MAX. Every
// weight starts at u32::MAX, so a leg not yet computed in this order reads
// u32::MAX as well. Returns 0, or 1 when a shortcut's middle is not a rank
// (the reference indexes out of bounds there).
u32 orc_cch_bottom_up(u32 n, const u64* uo, const u32* ut, const u64* dof, const u32* dt,
                      const uint8_t* up_short, const uint8_t* dn_short, const u32* up_mid,
                      const u32* dn_mid, const u32* orig_up, const u32* orig_dn, u32* out_up,
                      u32* out_dn) {
  const u64 nu = uo[n], nd = dof[n];
  std::fill(out_up, out_up + nu, INF);
  std::fill(out_dn, out_dn + nd, INF);
  auto leg = [&](const u64* off, const u32* tgt, const u32* w, u32 a, u32 b) {
    const u64 e = c_find(off, tgt, a, b);
    return e == ~0ull ? INF : w[e];
  };
  for (u32 u = 0; u < n; ++u) {
    for (u64 i = dof[u]; i < dof[u + 1]; ++i) {  // targets ascend: already sorted
      if (!dn_short[i]) {
        out_dn[i] = orig_dn[i];
        continue;
      }
      const u32 m = dn_mid[i];
      if (m >= n) return 1;
      out_dn[i] = sat_add(leg(dof, dt, out_dn, u, m), leg(uo, ut, out_up, m, dt[i]));
    }
    for (u64 i = uo[u]; i < uo[u + 1]; ++i) {
      if (!up_short[i]) {
        out_up[i] = orig_up[i];
        continue;
      }
      const u32 m = up_mid[i];
      if (m >= n) return 1;
      out_up[i] = sat_add(leg(dof, dt, out_dn, u, m), leg(uo, ut, out_up, m, ut[i]));
    }
  }
  return 0;
}
}
