// cch_build.cpp — synthetic road graph -> edge-based graph -> nested
// dissection -> chordal CCH -> basic customization -> INF-filtered flats.
//
// See bf_cch.h for the reference steps each stage restates.

#include "bf_cch.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <functional>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

using u8 = uint8_t;
using u16 = uint16_t;
using u32 = uint32_t;
using u64 = uint64_t;
using i64 = int64_t;
constexpr u32 INF = 0xFFFFFFFFu;

thread_local std::string g_err;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

inline u32 sat_add(u32 a, u32 b) {
  u64 s = (u64)a + (u64)b;
  return s >= INF ? INF : (u32)s;
}

// splitmix64: portable, seedable, identical on every platform.
struct Rng {
  u64 s;
  explicit Rng(u64 seed) : s(seed) {}
  u64 next() {
    u64 z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform in [0, n) by multiply-shift of the high 32 bits
  u32 below(u32 n) { return (u32)(((next() >> 32) * (u64)n) >> 32); }
  bool chance_ppm(u32 ppm) { return below(1000000u) < ppm; }
};

u64 isqrt64(u64 v) {
  u64 r = 0, bit = 1ull << 62;
  while (bit > v) bit >>= 2;
  while (bit) {
    if (v >= r + bit) {
      v -= r + bit;
      r = (r >> 1) + bit;
    } else {
      r >>= 1;
    }
    bit >>= 2;
  }
  return r;
}

// round(num / den) with ties to even (weights.rs round_half_even_div)
u64 rhe_div(u64 num, u64 den) {
  u64 q = num / den, r = num % den;
  if (2 * r > den || (2 * r == den && (q & 1))) ++q;
  return q;
}

struct Road {
  u32 a, b;
  u16 speed_kmh;
  u8 cls;  // 0 local, 1 arterial, 2 motorway
  u8 dir;  // 0 both ways, 1 a->b only, 2 b->a only
};

}  // namespace

struct bfc_graph {
  // intersections
  u32 n_int = 0;
  std::vector<i64> ix, iy;
  u64 n_roads = 0;
  // EBG
  u32 n = 0;
  std::vector<u32> tail, head, nw;
  std::vector<u8> scls;
  std::vector<i64> sx, sy;  // state coordinates (segment midpoint)
  std::vector<u64> arc_off;
  std::vector<u32> arc_dst, arc_w;
  // CCH
  std::vector<u32> rank_of, state_at;
  u64 n_chordal = 0;
  std::vector<u64> up_off, dn_off;
  std::vector<u32> up_tgt, up_w, dn_tgt, dn_w;
  // chordal completion in upper-neighbour form (kept for customization tests)
  std::vector<u64> topo_off;           // [n + 1]
  std::vector<u32> topo_tgt;           // upper neighbours of each rank, ascending
  std::vector<u32> orig_up, orig_dn;   // original arc weights per edge (INF: none)
  std::vector<u32> cust_up, cust_dn;   // weights after this library's customization
  double t_gen = 0, t_order = 0, t_contract = 0, t_custom = 0;
};

namespace {

// ---------------------------------------------------------------------------
// Synthetic road network
// ---------------------------------------------------------------------------

void make_intersections(bfc_graph& g, u32 rows, u32 cols, u32 sp, u32 jit, Rng& rng) {
  g.n_int = rows * cols;
  g.ix.resize(g.n_int);
  g.iy.resize(g.n_int);
  for (u32 r = 0; r < rows; ++r)
    for (u32 c = 0; c < cols; ++c) {
      u32 id = r * cols + c;
      i64 jx = (i64)rng.below(2 * jit + 1) - (i64)jit;
      i64 jy = (i64)rng.below(2 * jit + 1) - (i64)jit;
      g.ix[id] = (i64)c * sp + jx;
      g.iy[id] = (i64)r * sp + jy;
    }
}

// Grid workload (100 x 100 in the tests): 4-neighbour grid; 5% of roads removed, 10% one-way; speed
// classes 30/50/90 km/h at 80/15/5 %.
std::vector<Road> roads_grid(u32 rows, u32 cols, Rng& rng) {
  std::vector<Road> roads;
  roads.reserve((size_t)rows * cols * 2);
  for (u32 r = 0; r < rows; ++r)
    for (u32 c = 0; c < cols; ++c) {
      u32 id = r * cols + c;
      if (c + 1 < cols) roads.push_back({id, id + 1, 0, 0, 0});
      if (r + 1 < rows) roads.push_back({id, id + cols, 0, 0, 0});
    }
  std::vector<Road> kept;
  kept.reserve(roads.size());
  for (Road rd : roads) {
    if (rng.chance_ppm(50000)) continue;  // 5% removed
    u32 k = rng.below(100);
    rd.speed_kmh = k < 80 ? 30 : (k < 95 ? 50 : 90);
    rd.cls = k < 80 ? 0 : (k < 95 ? 1 : 2);
    if (rng.chance_ppm(100000)) rd.dir = (u8)(1 + rng.below(2));  // 10% one-way
    kept.push_back(rd);
  }
  return kept;
}

// Country-scale workload: lattice with arterial lines every 10 rows/cols (70 km/h),
// motorway lines every 80 (120 km/h), and 9x9 local-street cells. Inside a
// cell the streets are a random spanning tree plus ~30% of the remaining
// lattice edges as loops (30-50 km/h); each cell joins the arterial on its
// north and west side at one random point. One-way: 10% of loop and arterial
// roads.
std::vector<Road> roads_country(u32 rows, u32 cols, Rng& rng) {
  const u32 A = 10, M = 80;
  std::vector<Road> roads;
  roads.reserve((size_t)rows * cols * 13 / 10);
  auto id = [cols](u32 r, u32 c) { return r * cols + c; };
  // arterial / motorway rows
  for (u32 r = 0; r < rows; r += A)
    for (u32 c = 0; c + 1 < cols; ++c) {
      bool mw = (r % M) == 0;
      Road rd{id(r, c), id(r, c + 1), (u16)(mw ? 120 : 70), (u8)(mw ? 2 : 1), 0};
      if (!mw && rng.chance_ppm(100000)) rd.dir = (u8)(1 + rng.below(2));
      roads.push_back(rd);
    }
  for (u32 c = 0; c < cols; c += A)
    for (u32 r = 0; r + 1 < rows; ++r) {
      bool mw = (c % M) == 0;
      Road rd{id(r, c), id(r + 1, c), (u16)(mw ? 120 : 70), (u8)(mw ? 2 : 1), 0};
      if (!mw && rng.chance_ppm(100000)) rd.dir = (u8)(1 + rng.below(2));
      roads.push_back(rd);
    }
  // local cells
  std::vector<u32> uf;
  auto find = [&uf](u32 x) {
    while (uf[x] != x) {
      uf[x] = uf[uf[x]];
      x = uf[x];
    }
    return x;
  };
  struct CE {
    u32 a, b;  // local indices
    u64 key;
  };
  std::vector<CE> ce;
  for (u32 r0 = 0; r0 < rows; r0 += A)
    for (u32 c0 = 0; c0 < cols; c0 += A) {
      u32 r1 = std::min(r0 + A, rows), c1 = std::min(c0 + A, cols);  // exclusive
      u32 h = r1 - r0 - 1, w = c1 - c0 - 1;                           // interior size
      if (h == 0 || w == 0) continue;
      auto lid = [w](u32 rr, u32 cc) { return rr * w + cc; };
      ce.clear();
      for (u32 rr = 0; rr < h; ++rr)
        for (u32 cc = 0; cc < w; ++cc) {
          if (cc + 1 < w) ce.push_back({lid(rr, cc), lid(rr, cc + 1), rng.next()});
          if (rr + 1 < h) ce.push_back({lid(rr, cc), lid(rr + 1, cc), rng.next()});
        }
      std::sort(ce.begin(), ce.end(), [](const CE& x, const CE& y) { return x.key < y.key; });
      uf.resize((size_t)h * w);
      std::iota(uf.begin(), uf.end(), 0u);
      auto gid = [&](u32 l) { return id(r0 + 1 + l / w, c0 + 1 + l % w); };
      for (const CE& e : ce) {
        u32 ra = find(e.a), rb = find(e.b);
        bool tree = ra != rb;
        if (tree) uf[ra] = rb;
        if (tree || rng.chance_ppm(300000)) {
          Road rd{gid(e.a), gid(e.b), (u16)(30 + rng.below(21)), 0, 0};
          if (!tree && rng.chance_ppm(100000)) rd.dir = (u8)(1 + rng.below(2));
          roads.push_back(rd);
        }
      }
      // attachments: north (to arterial row r0) and west (to arterial col c0)
      u32 cn = c0 + 1 + rng.below(w);
      roads.push_back({id(r0, cn), id(r0 + 1, cn), (u16)(30 + rng.below(21)), 0, 0});
      u32 rw = r0 + 1 + rng.below(h);
      roads.push_back({id(rw, c0), id(rw, c0 + 1), (u16)(30 + rng.below(21)), 0, 0});
    }
  return roads;
}

// Edge-based expansion (ebg/mod.rs:370-421): states are directed segments,
// arcs are turns at the shared intersection; a U-turn is allowed only at a
// dead end (one outgoing segment). Turn penalty uniform 0..50 ds; 2% of the
// turns are forbidden (removed). For the country graph, forbidden turns are
// drawn only at junctions with >= 3 outgoing segments.
void expand_ebg(bfc_graph& g, const std::vector<Road>& roads, bool forbid_only_junctions, Rng& rng) {
  g.n_roads = roads.size();
  std::vector<u32> tail, head, nw;
  std::vector<u8> cls;
  tail.reserve(roads.size() * 2);
  for (const Road& rd : roads) {
    i64 dx = g.ix[rd.a] - g.ix[rd.b], dy = g.iy[rd.a] - g.iy[rd.b];
    u64 len_cm = isqrt64((u64)(dx * dx + dy * dy));
    // time[ds] = 36 * length[m] / speed[km/h] = 36 * len_cm / (100 * speed)
    u32 w = (u32)std::max<u64>(1, rhe_div(len_cm * 36, (u64)rd.speed_kmh * 100));
    if (rd.dir != 2) {
      tail.push_back(rd.a);
      head.push_back(rd.b);
      nw.push_back(w);
      cls.push_back(rd.cls);
    }
    if (rd.dir != 1) {
      tail.push_back(rd.b);
      head.push_back(rd.a);
      nw.push_back(w);
      cls.push_back(rd.cls);
    }
  }
  const u32 n = (u32)tail.size();
  g.n = n;
  // outgoing states per intersection
  std::vector<u32> out_off(g.n_int + 1, 0), out_list(n);
  for (u32 s = 0; s < n; ++s) out_off[tail[s] + 1]++;
  for (u32 i = 0; i < g.n_int; ++i) out_off[i + 1] += out_off[i];
  {
    std::vector<u32> fill(out_off.begin(), out_off.end() - 1);
    for (u32 s = 0; s < n; ++s) out_list[fill[tail[s]]++] = s;
  }
  g.arc_off.assign(n + 1, 0);
  g.arc_dst.clear();
  g.arc_w.clear();
  g.arc_dst.reserve((size_t)n * 2);
  g.arc_w.reserve((size_t)n * 2);
  for (u32 s = 0; s < n; ++s) {
    u32 b = head[s];
    u32 deg = out_off[b + 1] - out_off[b];
    for (u32 k = out_off[b]; k < out_off[b + 1]; ++k) {
      u32 t = out_list[k];
      if (head[t] == tail[s] && deg > 1) continue;  // U-turn at a non-dead-end
      bool may_forbid = !forbid_only_junctions || deg >= 3;
      if (may_forbid && rng.chance_ppm(20000)) continue;  // 2% forbidden turns
      u32 pen = rng.below(51);
      g.arc_dst.push_back(t);
      g.arc_w.push_back(sat_add(nw[t], pen));
    }
    g.arc_off[s + 1] = g.arc_dst.size();
  }
  g.tail = std::move(tail);
  g.head = std::move(head);
  g.nw = std::move(nw);
  g.scls = std::move(cls);
  g.sx.resize(n);
  g.sy.resize(n);
  for (u32 s = 0; s < n; ++s) {
    g.sx[s] = (g.ix[g.tail[s]] + g.ix[g.head[s]]) / 2;
    g.sy[s] = (g.iy[g.tail[s]] + g.iy[g.head[s]]) / 2;
  }
}

// ---------------------------------------------------------------------------
// Nested dissection
// ---------------------------------------------------------------------------

struct Sub {
  std::vector<u32> gid;       // global state id per local node
  std::vector<u32> off, adj;  // local undirected CSR
};

struct NdCtx {
  const i64* X;
  const i64* Y;
  u32* rank_of;
};

Sub induce(const Sub& p, const std::vector<u32>& members, std::vector<int32_t>& map) {
  // map: parent-local -> child-local (-1 outside); caller guarantees map is -1
  Sub c;
  c.gid.resize(members.size());
  for (u32 i = 0; i < members.size(); ++i) {
    map[members[i]] = (int32_t)i;
    c.gid[i] = p.gid[members[i]];
  }
  c.off.assign(members.size() + 1, 0);
  for (u32 i = 0; i < members.size(); ++i) {
    u32 v = members[i], cnt = 0;
    for (u32 k = p.off[v]; k < p.off[v + 1]; ++k)
      if (map[p.adj[k]] >= 0) ++cnt;
    c.off[i + 1] = c.off[i] + cnt;
  }
  c.adj.resize(c.off.back());
  for (u32 i = 0; i < members.size(); ++i) {
    u32 v = members[i], pos = c.off[i];
    for (u32 k = p.off[v]; k < p.off[v + 1]; ++k) {
      int32_t m = map[p.adj[k]];
      if (m >= 0) c.adj[pos++] = (u32)m;
    }
  }
  for (u32 v : members) map[v] = -1;
  return c;
}

// Minimum-degree elimination on <= 64 nodes with bit masks.
void mindeg_leaf(const Sub& s, u32 lo, NdCtx& ctx) {
  const u32 n = (u32)s.gid.size();
  u64 adj[64];
  for (u32 i = 0; i < n; ++i) {
    adj[i] = 0;
    for (u32 k = s.off[i]; k < s.off[i + 1]; ++k) adj[i] |= 1ull << s.adj[k];
    adj[i] &= ~(1ull << i);
  }
  u64 alive = (n == 64) ? ~0ull : ((1ull << n) - 1);
  for (u32 step = 0; step < n; ++step) {
    u32 best = 64, bdeg = 65;
    for (u64 m = alive; m; m &= m - 1) {
      u32 v = (u32)__builtin_ctzll(m);
      u32 d = (u32)__builtin_popcountll(adj[v] & alive);
      if (d < bdeg) {
        bdeg = d;
        best = v;
      }
    }
    u64 nb = adj[best] & alive & ~(1ull << best);
    for (u64 m = nb; m; m &= m - 1) {
      u32 u = (u32)__builtin_ctzll(m);
      adj[u] |= nb;
      adj[u] &= ~(1ull << u);
    }
    alive &= ~(1ull << best);
    ctx.rank_of[s.gid[best]] = lo + step;
  }
}

void nd_rec(Sub s, u32 lo, NdCtx& ctx);

void nd_spawn(Sub&& s, u32 lo, NdCtx& ctx) {
  if (s.gid.size() > 20000) {
    Sub* heap = new Sub(std::move(s));
    NdCtx* c = &ctx;
#pragma omp task firstprivate(heap, lo, c)
    {
      nd_rec(std::move(*heap), lo, *c);
      delete heap;
    }
  } else {
    nd_rec(std::move(s), lo, ctx);
  }
}

void nd_rec(Sub s, u32 lo, NdCtx& ctx) {
  const u32 n = (u32)s.gid.size();
  if (n == 0) return;
  if (n <= 64) {
    mindeg_leaf(s, lo, ctx);
    return;
  }
  // connected components
  std::vector<int32_t> comp(n, -1);
  std::vector<u32> queue;
  queue.reserve(n);
  u32 ncomp = 0;
  for (u32 r = 0; r < n; ++r) {
    if (comp[r] >= 0) continue;
    comp[r] = (int32_t)ncomp;
    queue.clear();
    queue.push_back(r);
    for (size_t h = 0; h < queue.size(); ++h) {
      u32 v = queue[h];
      for (u32 k = s.off[v]; k < s.off[v + 1]; ++k)
        if (comp[s.adj[k]] < 0) {
          comp[s.adj[k]] = (int32_t)ncomp;
          queue.push_back(s.adj[k]);
        }
    }
    ++ncomp;
  }
  std::vector<int32_t> map(n, -1);
  if (ncomp > 1) {
    std::vector<std::vector<u32>> members(ncomp);
    for (u32 v = 0; v < n; ++v) members[comp[v]].push_back(v);
    u32 base = lo;
    for (u32 c = 0; c < ncomp; ++c) {
      Sub child = induce(s, members[c], map);
      u32 sz = (u32)members[c].size();
      nd_spawn(std::move(child), base, ctx);
      base += sz;
    }
    return;
  }
  // cut along the longer axis
  i64 minx = INT64_MAX, maxx = INT64_MIN, miny = INT64_MAX, maxy = INT64_MIN;
  for (u32 v = 0; v < n; ++v) {
    i64 x = ctx.X[s.gid[v]], y = ctx.Y[s.gid[v]];
    minx = std::min(minx, x);
    maxx = std::max(maxx, x);
    miny = std::min(miny, y);
    maxy = std::max(maxy, y);
  }
  const i64* C = (maxx - minx >= maxy - miny) ? ctx.X : ctx.Y;
  std::vector<u32> order(n);
  std::iota(order.begin(), order.end(), 0u);
  std::sort(order.begin(), order.end(), [&](u32 a, u32 b) {
    i64 ca = C[s.gid[a]], cb = C[s.gid[b]];
    return ca != cb ? ca < cb : s.gid[a] < s.gid[b];
  });
  std::vector<u32> pos(n);
  for (u32 i = 0; i < n; ++i) pos[order[i]] = i;
  std::vector<int64_t> diff(n + 1, 0);
  for (u32 v = 0; v < n; ++v)
    for (u32 k = s.off[v]; k < s.off[v + 1]; ++k) {
      u32 u = s.adj[k];
      if (u <= v) continue;
      u32 a = std::min(pos[u], pos[v]), b = std::max(pos[u], pos[v]);
      diff[a]++;
      diff[b]--;
    }
  // cut after sorted index i: crossing[i] = #edges with a <= i < b
  u32 wlo = n / 5, whi = n - 1 - n / 5;
  int64_t run = 0;
  double best_score = 1e300;
  u32 best_i = n / 2;
  for (u32 i = 0; i + 1 < n; ++i) {
    run += diff[i];
    if (i < wlo || i > whi) continue;
    double bal = (double)std::min(i + 1, n - i - 1) / (double)n;
    double score = (double)run / bal + 1e-9 * std::abs((double)i - n / 2.0);
    if (score < best_score) {
      best_score = score;
      best_i = i;
    }
  }
  // greedy vertex cover of the crossing edges
  std::vector<u32> cdeg(n, 0);
  std::vector<std::pair<u32, u32>> cross;
  for (u32 v = 0; v < n; ++v)
    for (u32 k = s.off[v]; k < s.off[v + 1]; ++k) {
      u32 u = s.adj[k];
      if (u <= v) continue;
      bool lv = pos[v] <= best_i, lu = pos[u] <= best_i;
      if (lv != lu) {
        cross.push_back({v, u});
        cdeg[v]++;
        cdeg[u]++;
      }
    }
  std::vector<u32> coff(n + 1, 0);
  for (u32 v = 0; v < n; ++v) coff[v + 1] = coff[v] + cdeg[v];
  std::vector<u32> cedge(coff[n]);
  {
    std::vector<u32> f(coff.begin(), coff.end() - 1);
    for (u32 e = 0; e < cross.size(); ++e) {
      cedge[f[cross[e].first]++] = e;
      cedge[f[cross[e].second]++] = e;
    }
  }
  std::vector<u32> cand;
  for (u32 v = 0; v < n; ++v)
    if (cdeg[v]) cand.push_back(v);
  std::sort(cand.begin(), cand.end(), [&](u32 a, u32 b) {
    return cdeg[a] != cdeg[b] ? cdeg[a] > cdeg[b] : a < b;
  });
  std::vector<u8> covered(cross.size(), 0), insep(n, 0);
  std::vector<u32> sep;
  for (u32 v : cand) {
    bool need = false;
    for (u32 k = coff[v]; k < coff[v + 1]; ++k)
      if (!covered[cedge[k]]) {
        need = true;
        break;
      }
    if (!need) continue;
    insep[v] = 1;
    sep.push_back(v);
    for (u32 k = coff[v]; k < coff[v + 1]; ++k) covered[cedge[k]] = 1;
  }
  std::vector<u32> left, right;
  for (u32 i = 0; i < n; ++i) {
    u32 v = order[i];
    if (insep[v]) continue;
    (i <= best_i ? left : right).push_back(v);
  }
  if (left.empty() || right.empty()) {
    // degenerate cut (should not happen on a connected graph with n > 64):
    // fall back to ordering by coordinate
    for (u32 i = 0; i < n; ++i) ctx.rank_of[s.gid[order[i]]] = lo + i;
    return;
  }
  u32 sep_lo = lo + (u32)left.size() + (u32)right.size();
  std::sort(sep.begin(), sep.end(), [&](u32 a, u32 b) { return pos[a] < pos[b]; });
  for (u32 i = 0; i < sep.size(); ++i) ctx.rank_of[s.gid[sep[i]]] = sep_lo + i;
  Sub sl = induce(s, left, map);
  Sub sr = induce(s, right, map);
  u32 lsz = (u32)left.size();
  s = Sub();  // release before recursing
  nd_spawn(std::move(sl), lo, ctx);
  nd_spawn(std::move(sr), lo + lsz, ctx);
}

// ---------------------------------------------------------------------------
// CCH: chordal completion along the elimination tree, then customization
// ---------------------------------------------------------------------------

void build_cch(bfc_graph& g, int n_threads) {
  const u32 n = g.n;
  double t0 = now_s();
  // undirected state graph
  std::vector<u32> deg(n + 1, 0);
  for (u32 s = 0; s < n; ++s)
    for (u64 k = g.arc_off[s]; k < g.arc_off[s + 1]; ++k) {
      u32 t = g.arc_dst[k];
      if (t == s) continue;
      deg[s]++;
      deg[t]++;
    }
  std::vector<u32> uoff(n + 1, 0);
  for (u32 v = 0; v < n; ++v) uoff[v + 1] = uoff[v] + deg[v];
  std::vector<u32> uadj(uoff[n]);
  {
    std::vector<u32> f(uoff.begin(), uoff.end() - 1);
    for (u32 s = 0; s < n; ++s)
      for (u64 k = g.arc_off[s]; k < g.arc_off[s + 1]; ++k) {
        u32 t = g.arc_dst[k];
        if (t == s) continue;
        uadj[f[s]++] = t;
        uadj[f[t]++] = s;
      }
  }
  // dedupe per node
  {
    std::vector<u32> noff(n + 1, 0);
#pragma omp parallel for schedule(dynamic, 4096)
    for (u32 v = 0; v < n; ++v) {
      std::sort(uadj.begin() + uoff[v], uadj.begin() + uoff[v + 1]);
      u32 m = (u32)(std::unique(uadj.begin() + uoff[v], uadj.begin() + uoff[v + 1]) -
                    (uadj.begin() + uoff[v]));
      noff[v + 1] = m;
    }
    for (u32 v = 0; v < n; ++v) noff[v + 1] += noff[v];
    std::vector<u32> nadj(noff[n]);
#pragma omp parallel for schedule(dynamic, 4096)
    for (u32 v = 0; v < n; ++v)
      std::copy(uadj.begin() + uoff[v], uadj.begin() + uoff[v] + (noff[v + 1] - noff[v]),
                nadj.begin() + noff[v]);
    uoff.swap(noff);
    uadj.swap(nadj);
  }
  // nested dissection
  g.rank_of.assign(n, INF);
  {
    Sub root;
    root.gid.resize(n);
    std::iota(root.gid.begin(), root.gid.end(), 0u);
    root.off = uoff;
    root.adj = uadj;
    NdCtx ctx{g.sx.data(), g.sy.data(), g.rank_of.data()};
#pragma omp parallel num_threads(n_threads)
#pragma omp single
    nd_rec(std::move(root), 0, ctx);
  }
  g.state_at.assign(n, INF);
  for (u32 v = 0; v < n; ++v) {
    if (g.rank_of[v] >= n || g.state_at[g.rank_of[v]] != INF)
      throw std::runtime_error("nested dissection produced an invalid permutation");
    g.state_at[g.rank_of[v]] = v;
  }
  double t1 = now_s();
  g.t_order = t1 - t0;

  // rank-space adjacency (lower neighbours only, for the elimination tree)
  std::vector<u32> loff(n + 1, 0);
  for (u32 r = 0; r < n; ++r) {
    u32 v = g.state_at[r], c = 0;
    for (u32 k = uoff[v]; k < uoff[v + 1]; ++k)
      if (g.rank_of[uadj[k]] < r) ++c;
    loff[r + 1] = loff[r] + c;
  }
  std::vector<u32> ladj(loff[n]);
#pragma omp parallel for schedule(dynamic, 4096)
  for (u32 r = 0; r < n; ++r) {
    u32 v = g.state_at[r], p = loff[r];
    for (u32 k = uoff[v]; k < uoff[v + 1]; ++k) {
      u32 q = g.rank_of[uadj[k]];
      if (q < r) ladj[p++] = q;
    }
    std::sort(ladj.begin() + loff[r], ladj.begin() + loff[r + 1]);
  }
  uoff.clear();
  uoff.shrink_to_fit();
  uadj.clear();
  uadj.shrink_to_fit();
  // elimination tree (Liu, path compression)
  std::vector<u32> parent(n, INF), anc(n, INF);
  for (u32 i = 0; i < n; ++i) {
    for (u32 k = loff[i]; k < loff[i + 1]; ++k) {
      u32 j = ladj[k];
      while (j != INF && j < i) {
        u32 nx = anc[j];
        anc[j] = i;
        if (nx == INF) parent[j] = i;
        j = nx;
      }
    }
  }
  anc.clear();
  anc.shrink_to_fit();
  // row structures: row(i) = {j < i : (j, i) in the chordal completion}
  std::vector<u64> roff(n + 1, 0);
  {
    std::vector<u32> cnt(n, 0);
#pragma omp parallel num_threads(n_threads)
    {
      std::vector<u32> mark(n, INF);
#pragma omp for schedule(dynamic, 1024)
      for (u32 i = 0; i < n; ++i) {
        u32 c = 0;
        mark[i] = i;
        for (u32 k = loff[i]; k < loff[i + 1]; ++k)
          for (u32 j = ladj[k]; mark[j] != i; j = parent[j]) {
            mark[j] = i;
            ++c;
          }
        cnt[i] = c;
      }
    }
    for (u32 i = 0; i < n; ++i) roff[i + 1] = roff[i] + cnt[i];
  }
  const u64 L = roff[n];
  std::vector<u32> rowj(L);
#pragma omp parallel num_threads(n_threads)
  {
    std::vector<u32> mark(n, INF);
#pragma omp for schedule(dynamic, 1024)
    for (u32 i = 0; i < n; ++i) {
      u64 p = roff[i];
      mark[i] = i;
      for (u32 k = loff[i]; k < loff[i + 1]; ++k)
        for (u32 j = ladj[k]; mark[j] != i; j = parent[j]) {
          mark[j] = i;
          rowj[p++] = j;
        }
      std::sort(rowj.begin() + roff[i], rowj.begin() + roff[i + 1]);
    }
  }
  loff.clear();
  loff.shrink_to_fit();
  ladj.clear();
  ladj.shrink_to_fit();
  // transpose: U(j) = {i > j : j in row(i)}, ascending; remember slots
  std::vector<u64> Uoff(n + 1, 0);
  for (u64 p = 0; p < L; ++p) Uoff[rowj[p] + 1]++;
  for (u32 j = 0; j < n; ++j) Uoff[j + 1] += Uoff[j];
  std::vector<u32> Ut(L);
  std::vector<u64> rowslot(L);
  {
    std::vector<u64> f(Uoff.begin(), Uoff.end() - 1);
    for (u32 i = 0; i < n; ++i)
      for (u64 p = roff[i]; p < roff[i + 1]; ++p) {
        u32 j = rowj[p];
        rowslot[p] = f[j];
        Ut[f[j]++] = i;
      }
  }
  g.n_chordal = L;
  double t2 = now_s();
  g.t_contract = t2 - t1;

  // customization: wup[e] = w(j -> U(j)[e]), wdn[e] = w(U(j)[e] -> j)
  std::vector<u32> wup(L, INF), wdn(L, INF);
  auto slot_of = [&](u32 j, u32 i) -> u64 {
    auto b = Ut.begin() + Uoff[j], e = Ut.begin() + Uoff[j + 1];
    auto it = std::lower_bound(b, e, i);
    return (u64)(it - Ut.begin());
  };
  for (u32 s = 0; s < n; ++s) {
    u32 rs = g.rank_of[s];
    for (u64 k = g.arc_off[s]; k < g.arc_off[s + 1]; ++k) {
      u32 rt = g.rank_of[g.arc_dst[k]];
      if (rt == rs) continue;
      u32 w = g.arc_w[k];
      if (rs < rt) {
        u64 e = slot_of(rs, rt);
        wup[e] = std::min(wup[e], w);
      } else {
        u64 e = slot_of(rt, rs);
        wdn[e] = std::min(wdn[e], w);
      }
    }
  }
  g.orig_up = wup;
  g.orig_dn = wdn;
  // etree heights (children before parents)
  std::vector<u32> height(n, 0);
  u32 max_h = 0;
  for (u32 i = 0; i < n; ++i) {
    if (parent[i] != INF) height[parent[i]] = std::max(height[parent[i]], height[i] + 1);
    max_h = std::max(max_h, height[i]);
  }
  std::vector<u32> hoff(max_h + 2, 0), hnodes(n);
  for (u32 i = 0; i < n; ++i) hoff[height[i] + 1]++;
  for (u32 h = 0; h <= max_h; ++h) hoff[h + 1] += hoff[h];
  {
    std::vector<u32> f(hoff.begin(), hoff.end() - 1);
    for (u32 i = 0; i < n; ++i) hnodes[f[height[i]]++] = i;
  }
  // node x pulls every lower triangle (z, x, y), z in row(x), y in U(z), y > x
#pragma omp parallel num_threads(n_threads)
  {
    std::vector<u64> where(n, ~0ull);
    for (u32 h = 0; h <= max_h; ++h) {
#pragma omp for schedule(dynamic, 64)
      for (u32 q = hoff[h]; q < hoff[h + 1]; ++q) {
        u32 x = hnodes[q];
        for (u64 e = Uoff[x]; e < Uoff[x + 1]; ++e) where[Ut[e]] = e;
        for (u64 p = roff[x]; p < roff[x + 1]; ++p) {
          u32 z = rowj[p];
          u64 ezx = rowslot[p];
          u32 w_xz = wdn[ezx], w_zx = wup[ezx];
          if (w_xz == INF && w_zx == INF) continue;
          for (u64 ezy = ezx + 1; ezy < Uoff[z + 1]; ++ezy) {
            u64 f = where[Ut[ezy]];
            u32 a = sat_add(w_xz, wup[ezy]);
            if (a < wup[f]) wup[f] = a;
            u32 b = sat_add(wdn[ezy], w_zx);
            if (b < wdn[f]) wdn[f] = b;
          }
        }
      }
    }
  }
  double t3 = now_s();
  g.t_custom = t3 - t2;
  g.topo_off = Uoff;
  g.topo_tgt = Ut;
  g.cust_up = wup;
  g.cust_dn = wdn;
  rowj.clear();
  rowj.shrink_to_fit();
  rowslot.clear();
  rowslot.shrink_to_fit();

  // INF-filtered flats (bucket_ch.rs:191-338): up by source, down by source
  g.up_off.assign(n + 1, 0);
  g.dn_off.assign(n + 1, 0);
  for (u32 j = 0; j < n; ++j)
    for (u64 e = Uoff[j]; e < Uoff[j + 1]; ++e) {
      if (wup[e] != INF) g.up_off[j + 1]++;
      if (wdn[e] != INF) g.dn_off[Ut[e] + 1]++;
    }
  for (u32 j = 0; j < n; ++j) {
    g.up_off[j + 1] += g.up_off[j];
    g.dn_off[j + 1] += g.dn_off[j];
  }
  g.up_tgt.resize(g.up_off[n]);
  g.up_w.resize(g.up_off[n]);
  g.dn_tgt.resize(g.dn_off[n]);
  g.dn_w.resize(g.dn_off[n]);
  {
    std::vector<u64> fu(g.up_off.begin(), g.up_off.end() - 1);
    std::vector<u64> fd(g.dn_off.begin(), g.dn_off.end() - 1);
    for (u32 j = 0; j < n; ++j)
      for (u64 e = Uoff[j]; e < Uoff[j + 1]; ++e) {
        u32 i = Ut[e];
        if (wup[e] != INF) {
          g.up_tgt[fu[j]] = i;
          g.up_w[fu[j]++] = wup[e];
        }
        if (wdn[e] != INF) {
          g.dn_tgt[fd[i]] = j;
          g.dn_w[fd[i]++] = wdn[e];
        }
      }
  }
}

int guard(const std::function<void()>& fn) {
  try {
    fn();
    return 0;
  } catch (const std::bad_alloc&) {
    g_err = "out of host memory";
  } catch (const std::exception& e) {
    g_err = e.what();
  }
  return 1;
}
}  // namespace

extern "C" {

int bfc_build_synthetic(const bfc_synth_params* p, int n_threads, bfc_graph** out) {
  if (out) *out = nullptr;
  if (!p || !out) {
    g_err = "null argument";
    return 1;
  }
  if (p->rows < 2 || p->cols < 2 || (u64)p->rows * p->cols > 400000000ull) {
    g_err = "rows/cols out of range";
    return 1;
  }
  if (p->kind != BFC_KIND_GRID && p->kind != BFC_KIND_COUNTRY) {
    g_err = "unknown graph kind";
    return 1;
  }
  if (n_threads <= 0) n_threads = omp_get_max_threads();
  bfc_graph* g = new (std::nothrow) bfc_graph();
  if (!g) {
    g_err = "out of host memory";
    return 1;
  }
  int rc = guard([&] {
    omp_set_num_threads(n_threads);
    double t0 = now_s();
    u32 sp = p->spacing_cm ? p->spacing_cm : 10000;
    u32 jit = p->jitter_cm ? p->jitter_cm : sp / 4;
    Rng rng(p->seed);
    make_intersections(*g, p->rows, p->cols, sp, jit, rng);
    std::vector<Road> roads = p->kind == BFC_KIND_GRID ? roads_grid(p->rows, p->cols, rng)
                                                        : roads_country(p->rows, p->cols, rng);
    expand_ebg(*g, roads, p->kind == BFC_KIND_COUNTRY, rng);
    g->t_gen = now_s() - t0;
    build_cch(*g, n_threads);
  });
  if (rc) {
    delete g;
    return rc;
  }
  *out = g;
  return 0;
}

int bfc_build_from_arcs(uint32_t n_states, uint64_t n_arcs, const uint32_t* arc_src,
                        const uint32_t* arc_dst, const uint32_t* arc_w, const int64_t* sx,
                        const int64_t* sy, int n_threads, bfc_graph** out) {
  if (out) *out = nullptr;
  if (!out || n_states == 0 || (n_arcs && (!arc_src || !arc_dst || !arc_w)) || !sx || !sy) {
    g_err = "invalid argument";
    return 1;
  }
  for (u64 k = 0; k < n_arcs; ++k)
    if (arc_src[k] >= n_states || arc_dst[k] >= n_states) {
      g_err = "arc endpoint out of range";
      return 1;
    }
  if (n_threads <= 0) n_threads = omp_get_max_threads();
  bfc_graph* g = new (std::nothrow) bfc_graph();
  if (!g) {
    g_err = "out of host memory";
    return 1;
  }
  int rc = guard([&] {
    omp_set_num_threads(n_threads);
    g->n = n_states;
    g->n_int = 0;
    g->sx.assign(sx, sx + n_states);
    g->sy.assign(sy, sy + n_states);
    g->arc_off.assign(n_states + 1, 0);
    for (u64 k = 0; k < n_arcs; ++k) g->arc_off[arc_src[k] + 1]++;
    for (u32 s = 0; s < n_states; ++s) g->arc_off[s + 1] += g->arc_off[s];
    g->arc_dst.resize(n_arcs);
    g->arc_w.resize(n_arcs);
    std::vector<u64> f(g->arc_off.begin(), g->arc_off.end() - 1);
    for (u64 k = 0; k < n_arcs; ++k) {
      u64 q = f[arc_src[k]]++;
      g->arc_dst[q] = arc_dst[k];
      g->arc_w[q] = arc_w[k];
    }
    g->nw.assign(n_states, 0);
    g->tail.assign(n_states, 0);
    g->head.assign(n_states, 0);
    g->scls.assign(n_states, 0);
    build_cch(*g, n_threads);
  });
  if (rc) {
    delete g;
    return rc;
  }
  *out = g;
  return 0;
}

void bfc_free(bfc_graph* g) { delete g; }

void bfc_ebg(const bfc_graph* g, bfc_ebg_view* o) {
  std::memset(o, 0, sizeof(*o));
  if (!g) return;
  o->n_intersections = g->n_int;
  o->n_states = g->n;
  o->n_roads = g->n_roads;
  o->n_arcs = g->arc_dst.size();
  o->arc_off = g->arc_off.data();
  o->arc_dst = g->arc_dst.data();
  o->arc_w = g->arc_w.data();
  o->node_weight = g->nw.data();
  o->state_tail = g->tail.data();
  o->state_head = g->head.data();
  o->state_class = g->scls.data();
  o->ix = g->ix.data();
  o->iy = g->iy.data();
}

void bfc_topo(const bfc_graph* g, bfc_topo_view* o) {
  std::memset(o, 0, sizeof(*o));
  o->n_nodes = g->n;
  o->n_edges = g->topo_tgt.size();
  o->off = g->topo_off.data();
  o->tgt = g->topo_tgt.data();
  o->orig_up = g->orig_up.data();
  o->orig_down = g->orig_dn.data();
  o->cust_up = g->cust_up.data();
  o->cust_down = g->cust_dn.data();
}

void bfc_cch(const bfc_graph* g, bfc_cch_view* o) {
  std::memset(o, 0, sizeof(*o));
  if (!g) return;
  o->n_nodes = g->n;
  o->n_up = g->up_tgt.size();
  o->n_down = g->dn_tgt.size();
  o->n_chordal = g->n_chordal;
  o->up_off = g->up_off.data();
  o->up_tgt = g->up_tgt.data();
  o->up_w = g->up_w.data();
  o->down_off = g->dn_off.data();
  o->down_tgt = g->dn_tgt.data();
  o->down_w = g->dn_w.data();
  o->rank_to_state = g->state_at.data();
  o->state_to_rank = g->rank_of.data();
  o->t_generate_s = g->t_gen;
  o->t_order_s = g->t_order;
  o->t_contract_s = g->t_contract;
  o->t_customize_s = g->t_custom;
}

const char* bfc_last_error(void) { return g_err.c_str(); }

}  // extern "C"
