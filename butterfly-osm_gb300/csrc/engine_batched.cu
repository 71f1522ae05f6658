// engine_batched.cu — the batched GPU PHAST engine.
//
// All sources of a call (up to the HBM budget) run as the lanes of ONE
// level-synchronous sweep over a [row][lane] u32 slab, instead of the
// reference's chunks of K_LANES = 8 (batched_phast.rs:33, :667-706):
//
//   * target restriction (RPHAST): only rows that reach a requested target
//     through DOWN edges are swept. They are found by one descending scan of
//     the level-ordered pull CSR (in-edge sources always sit at lower slab
//     positions). Their distances at the targets are exactly the unrestricted
//     ones: every DOWN path into a target stays inside the restricted set.
//   * upward: the k_upward path walk writes each source's settled ancestors
//     straight into its lane of the (INF-initialised) slab.
//   * sweep: one launch per level of the restricted DAG; a work item is a
//     node (or a slice of at most SPLIT in-edges of a high in-degree node);
//     a thread owns 4 consecutive lanes, so every gathered source row is a
//     contiguous, coalesced uint4 stream. Sliced nodes combine with atomicMin.
//   * extract: target rows -> row-major S x T matrix via a shared-memory
//     transpose; cells above the threshold become INF.

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <thread>

#include "engine.cuh"

namespace bf {

namespace {


// Hash of a target list: only a fast pre-check before the exact comparison
// of the cached schedule's targets. Setting BF_TEST_SCHED_KEY_COLLIDE in the
// environment makes every list hash alike (a test hook: schedules must then
// still be told apart by the comparison).
uint64_t hash_targets(const uint32_t* t, uint64_t T) {
  static const bool collide = std::getenv("BF_TEST_SCHED_KEY_COLLIDE") != nullptr;
  if (collide) return 0x5EEDull;
  uint64_t h = 1469598103934665603ull ^ T;
  for (uint64_t i = 0; i < T; ++i) {
    h ^= t[i];
    h *= 1099511628211ull;
  }
  return h;
}

// Grow a device array to `need` elements (1/8 more with `slack`, for arrays
// sized by a schedule's rows, items or edges, which vary between targets).
template <class T>
bf_status ensure(T** p, size_t& cap, size_t need, Graph* g, bool slack = false) {
  if (need <= cap && *p) return BF_OK;
  if (*p) {
    cudaFree(*p);
    g->device_bytes -= cap * sizeof(T);
  }
  *p = nullptr;
  cap = 0;
  size_t n = std::max<size_t>(slack ? need + need / 8 : need, 1);
  if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_error("cudaMalloc for the restricted schedule failed");
    return BF_ERR_OOM;
  }
  cap = n;
  g->device_bytes += n * sizeof(T);
  return BF_OK;
}

// Run f(b, e) over [0, n) split into contiguous chunks on host threads
// (single-threaded below `grain` units per thread).
// f(t, b, e) for nt equal contiguous slices of [0, n), slice t on thread t.
template <class F>
void parallel_slices(uint64_t n, uint32_t nt, F f) {
  const uint64_t step = (n + nt - 1) / nt;
  std::vector<std::thread> th;
  for (uint32_t t = 1; t < nt; ++t) {
    const uint64_t b = std::min(n, t * step), e = std::min(n, (t + 1) * step);
    th.emplace_back([&f, t, b, e] { f(t, b, e); });
  }
  f(0, 0, std::min(n, step));
  for (auto& x : th) x.join();
}

template <class F>
void parallel_chunks(uint64_t n, uint64_t grain, F f, uint64_t max_threads = 16) {
  uint64_t nt = std::min<uint64_t>(std::max(1u, std::thread::hardware_concurrency()), max_threads);
  nt = std::min<uint64_t>(nt, std::max<uint64_t>(1, n / std::max<uint64_t>(grain, 1)));
  if (nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const uint64_t step = (n + nt - 1) / nt;
  for (uint64_t t = 1; t < nt; ++t) {
    const uint64_t b = std::min(n, t * step), e = std::min(n, (t + 1) * step);
    th.emplace_back([&f, b, e] { f(b, e); });
  }
  f(0, std::min(n, step));
  for (auto& x : th) x.join();
}

}  // namespace

__global__ void k_scatter_pairs(const uint2* __restrict__ pr, uint64_t m,
                                uint32_t* __restrict__ out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[pr[i].x] = pr[i].y;
}

// Build (or reuse) a sweep schedule: restricted to the DOWN ancestry of the
// targets h_tgt[0..T) (ranks, on the host), or over every node when all is
// set (then h_tgt may be null and T is 0). The restricted set is collected by
// walking in-edges from the targets in descending slab position (a max-heap:
// in-edge sources always have lower positions), so the cost is proportional
// to the restricted nodes and edges, not to the graph. The device rank->row
// map is patched in place: entries of the previous schedule are reset to
// NONE and the new ones set.
bf_status build_schedule(Graph* g, Ctx& c, Sched& sc, const uint32_t* h_tgt, uint64_t T, bool all,
                         cudaStream_t st, const uint32_t* d_tgt) {
  const uint32_t SPLIT = std::max<uint32_t>(1, g->tune.split);
  const uint32_t SMALL_ROWS = g->tune.small_rows;
  const uint32_t SMALL_SPLIT = std::max<uint32_t>(1, std::min(SPLIT, g->tune.small_split));
  const uint64_t key = (all ? 0x9E3779B97F4A7C15ull : hash_targets(h_tgt, T)) ^
                       ((uint64_t)SPLIT << 56) ^ ((uint64_t)SMALL_SPLIT << 48) ^
                       ((uint64_t)SMALL_ROWS << 20);
  // reuse only for the same split settings and exactly the same targets
  if (sc.valid && sc.key == key && sc.T == T &&
      (all || (sc.tgt.size() == T && (T == 0 || std::memcmp(sc.tgt.data(), h_tgt, T * 4) == 0)))) {
    ++sc.uses;
    return BF_OK;
  }
  sc.valid = false;
  sc.uses = 0;
  if (sc.gexec) {
    cudaGraphExecDestroy(sc.gexec);
    sc.gexec = nullptr;
  }
  if (sc.one_exec) {
    cudaGraphExecDestroy(sc.one_exec);
    sc.one_exec = nullptr;
  }
  // restricted schedules are built on the device (schedule.cu) unless turned
  // off; the totals it reads back carry edges in 32 bits
  if (!all && T && g->tune.dev_sched && g->n_down < 0xFFFFFFFFull)
    return build_schedule_device(g, c, sc, h_tgt, d_tgt, T, key, st);
  sc.dev_built = false;
  if (sc.cidx_dirty) {  // the device build wrote every rank: reset the map whole
    sc.ranks.clear();
    sc.cidx_ready = false;
    sc.cidx_dirty = false;
  }
  const uint32_t n = g->n;
  if (c.rowmap.size() != n) c.rowmap.assign(n, NONE);
  // restricted positions grouped by level, levels ascending (the order inside
  // a level does not matter: no edge joins two rows of one level)
  std::vector<uint32_t> R;
  if (all) {
    R.resize(n);
    for (uint32_t p = 0; p < n; ++p) R[p] = p;
  } else {
    // The restricted set is everything that reaches a target along in-edges.
    // Host threads each walk (depth first) from their share of the targets; a
    // node is expanded by the thread that claims it (atomic OR on a bitmap of
    // n bits, small enough to stay in the host caches), so every node is
    // expanded once. The claimed nodes are then grouped by level.
    if (c.markbits.size() != (n + 63) / 64) c.markbits.assign((n + 63) / 64, 0);
    uint64_t* mb = c.markbits.data();
    auto claim = [mb](uint32_t u) {
      const uint64_t bit = 1ull << (u & 63);
      if (__atomic_load_n(&mb[u >> 6], __ATOMIC_RELAXED) & bit) return false;
      return (__atomic_fetch_or(&mb[u >> 6], bit, __ATOMIC_RELAXED) & bit) == 0;
    };
    const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t nth = T >= 512 ? std::min(16u, hw) : 1u;
    std::vector<std::vector<uint32_t>> found(nth);
    parallel_slices(T, nth, [&](uint32_t t, uint64_t b, uint64_t e) {
      std::vector<uint32_t>& out = found[t];
      std::vector<uint32_t> stack;
      for (uint64_t i = b; i < e; ++i) {
        const uint32_t p0 = g->pos_of[h_tgt[i]];
        if (!claim(p0)) continue;
        out.push_back(p0);
        stack.push_back(p0);
        while (!stack.empty()) {
          const uint32_t p = stack.back();
          stack.pop_back();
          for (uint64_t k = g->h_in_off[p]; k < g->h_in_off[p + 1]; ++k) {
            const uint32_t u = g->h_in_rec[k].x;
            if (claim(u)) {
              out.push_back(u);
              stack.push_back(u);
            }
          }
        }
      }
    });
    // group by level, levels ascending (a counting sort on the level index)
    const uint32_t L = g->n_levels;
    std::vector<uint32_t> lvl_cnt(L + 1, 0);
    size_t tot = 0;
    for (auto& f : found) tot += f.size();
    std::vector<uint32_t> lv(tot);
    {
      size_t j = 0;
      for (auto& f : found)
        for (uint32_t p : f) {
          const uint32_t l = (uint32_t)(std::upper_bound(g->lvl_start.begin(), g->lvl_start.end(), p) -
                                        g->lvl_start.begin() - 1);
          lv[j++] = l;
          ++lvl_cnt[l + 1];
        }
    }
    for (uint32_t l = 0; l < L; ++l) lvl_cnt[l + 1] += lvl_cnt[l];
    R.resize(tot);
    {
      size_t j = 0;
      for (auto& f : found)
        for (uint32_t p : f) R[lvl_cnt[lv[j++]]++] = p;
    }
    for (uint32_t p : R) mb[p >> 6] = 0;
  }
  const uint32_t n_r = (uint32_t)R.size();
  for (uint32_t i = 0; i < n_r; ++i) c.rowmap[R[i]] = i;
  const bool two = g->has_len;
  // rows per level; small levels get short work items
  std::vector<uint32_t> row_lvl(g->n_levels + 1, 0);
  {
    uint32_t l = 0;
    for (uint32_t i = 0; i < n_r; ++i) {
      while (R[i] >= g->lvl_start[l + 1]) row_lvl[++l] = i;
    }
    while (l < g->n_levels) row_lvl[++l] = n_r;
  }
  // per row: edge and item offsets (prefix sums), then a parallel fill
  std::vector<uint64_t> eoff(n_r + 1, 0), ioff(n_r + 1, 0);
  std::vector<uint32_t> split_of(n_r);
  for (uint32_t l = 0; l < g->n_levels; ++l) {
    const uint32_t rows_l = row_lvl[l + 1] - row_lvl[l];
    const uint32_t split_l = rows_l < SMALL_ROWS ? SMALL_SPLIT : SPLIT;
    for (uint32_t i = row_lvl[l]; i < row_lvl[l + 1]; ++i) {
      const uint32_t p = R[i];
      const uint64_t deg = g->h_in_off[p + 1] - g->h_in_off[p];
      split_of[i] = split_l;
      eoff[i + 1] = eoff[i] + deg;
      ioff[i + 1] = ioff[i] + (deg + split_l - 1) / split_l;
    }
  }
  if (eoff[n_r] > 0xFFFFFFFFull) {
    for (uint32_t p : R) c.rowmap[p] = NONE;
    set_error("restricted edge set exceeds 2^32 edges");
    return BF_ERR_UNSUPPORTED;
  }
  // items, edge records (and length weights) are filled in place in the
  // context's page-locked staging arena, so their upload is a plain DMA
  const size_t n_e = eoff[n_r], n_i = ioff[n_r];
  {
    const size_t need = n_i * sizeof(uint4) + n_e * sizeof(uint2) + (two ? n_e * 4 : 0) + 64;
    if (need > c.stage_bytes) {
      if (c.h_stage) cudaFreeHost(c.h_stage);
      c.h_stage = nullptr;
      c.stage_bytes = 0;
      if (cudaHostAlloc(&c.h_stage, need, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        for (uint32_t p : R) c.rowmap[p] = NONE;
        set_error("cannot allocate the page-locked schedule staging buffer");
        return BF_ERR_OOM;
      }
      c.stage_bytes = need;
    }
  }
  uint4* items = static_cast<uint4*>(c.h_stage);
  uint2* erec = reinterpret_cast<uint2*>(items + n_i);
  uint32_t* elen = reinterpret_cast<uint32_t*>(erec + n_e);  // length weight per erec entry
  std::vector<uint32_t> split_bits((n_r + 31) / 32 + 1, 0);
  // chunks of whole 32-row groups, so no two threads share a split_bits word
  parallel_chunks((n_r + 31) / 32, 256, [&](uint64_t w0, uint64_t w1) {
    const uint32_t i1 = (uint32_t)std::min<uint64_t>(n_r, w1 * 32);
    for (uint32_t i = (uint32_t)(w0 * 32); i < i1; ++i) {
      const uint32_t p = R[i];
      const uint64_t k0 = g->h_in_off[p], k1 = g->h_in_off[p + 1];
      if (k0 == k1) {  // no in-edges: the row is its seed (or INF): reset every wave
        split_bits[i >> 5] |= 1u << (i & 31);
        continue;
      }
      const uint32_t e0 = (uint32_t)eoff[i];
      for (uint64_t k = k0; k < k1; ++k) {
        erec[e0 + (k - k0)] = make_uint2(c.rowmap[g->h_in_rec[k].x], g->h_in_rec[k].y);
        if (two) elen[e0 + (k - k0)] = g->h_in_len[k];
      }
      const uint32_t deg = (uint32_t)(k1 - k0), sp = split_of[i];
      const uint32_t split = deg > sp ? 1u : 0u;
      if (split) split_bits[i >> 5] |= 1u << (i & 31);
      uint64_t it = ioff[i];
      for (uint32_t a = 0; a < deg; a += sp)
        items[it++] = make_uint4(i, e0 + a, e0 + std::min(deg, a + sp), split);
    }
  });
  sc.lvl_item.assign(g->n_levels + 1, 0);
  for (uint32_t l = 0; l <= g->n_levels; ++l) sc.lvl_item[l] = (uint32_t)ioff[row_lvl[l]];
  // the edge records of a level's rows are contiguous: level -> first record
  std::vector<uint32_t> lvl_erec(g->n_levels + 1);
  for (uint32_t l = 0; l <= g->n_levels; ++l) lvl_erec[l] = (uint32_t)eoff[row_lvl[l]];
  sc.lvl_erec_ready = true;
  sc.lvl_row = row_lvl;
  sc.lvl_edge = lvl_erec;
  // rows by gather count, most-used first (up to 65536 of them): the matrix
  // sweep keeps the head of this list in L2. A counting sort by count; the
  // full-graph schedule (isochrones, bounded queries) does not use it.
  sc.hub_order.clear();
  sc.hub_rows = NONE;  // bitmap to be (re)built for this schedule
  if (!all && n_r) {
    std::vector<uint32_t> uses(n_r, 0);
    for (size_t k = 0; k < n_e; ++k) ++uses[erec[k].x];
    uint32_t top = 0;
    for (uint32_t u : uses) top = std::max(top, u);
    std::vector<uint32_t> at(top + 2, 0);  // rows per count, then start offsets (descending)
    for (uint32_t u : uses) ++at[u];
    const uint32_t keep = std::min<uint32_t>(n_r, 65536);
    uint32_t acc = 0;
    for (uint32_t u = top + 1; u-- > 0;) {
      const uint32_t c = at[u];
      at[u] = acc;
      acc += c;
    }
    sc.hub_order.assign(keep, 0);
    for (uint32_t i = 0; i < n_r; ++i) {
      const uint32_t slot = at[uses[i]]++;
      if (slot < keep) sc.hub_order[slot] = i;
    }
  }
  // items of a level, heaviest first, so the level's last blocks are short
  parallel_chunks(g->n_levels, 16, [&](uint64_t l0, uint64_t l1) {
    for (uint64_t l = l0; l < l1; ++l)
      std::stable_sort(items + sc.lvl_item[l], items + sc.lvl_item[l + 1],
                       [](const uint4& a, const uint4& b) { return a.z - a.y > b.z - b.y; });
  });
  std::vector<uint32_t> trow(T);
  for (uint64_t i = 0; i < T; ++i) trow[i] = c.rowmap[g->pos_of[h_tgt[i]]];
  // device rank -> row map: reset the previous schedule's entries, set ours
  std::vector<uint2> pairs;
  pairs.reserve(sc.ranks.size() + n_r);
  for (uint32_t r : sc.ranks) pairs.push_back(make_uint2(r, NONE));
  const size_t n_reset = pairs.size();
  std::vector<uint32_t> ranks(n_r);
  for (uint32_t i = 0; i < n_r; ++i) {
    ranks[i] = g->rank_at[R[i]];
    pairs.push_back(make_uint2(ranks[i], i));
  }
  for (uint32_t p : R) c.rowmap[p] = NONE;
  bf_status s;
  if ((s = ensure(&sc.d_cidx, sc.cap_cidx, n, g))) return s;
  if ((s = ensure(&sc.d_item, sc.cap_items, n_i, g, true))) return s;
  // two records of padding: a bulk copy of a level's records rounds its end
  // up to 16 bytes
  if ((s = ensure(&sc.d_erec, sc.cap_edges, n_e + 2, g, true))) return s;
  if (two && (s = ensure(&sc.d_elen, sc.cap_elen, n_e, g, true))) return s;
  if ((s = ensure(&sc.d_trow, sc.cap_t, T, g, true))) return s;
  if ((s = ensure(&c.d_pairs, c.cap_pairs, pairs.size() * 2, g, true))) return s;
  if ((s = ensure(&sc.d_split, sc.cap_split, split_bits.size(), g))) return s;
  if ((s = ensure(&sc.d_lvl_erec, sc.cap_lvl_erec, lvl_erec.size(), g, true))) return s;
  BF_CUDA(cudaMemcpyAsync(sc.d_lvl_erec, lvl_erec.data(), lvl_erec.size() * 4,
                          cudaMemcpyHostToDevice, st));
  if ((s = ensure(&sc.d_lvl, sc.cap_lvl, sc.lvl_item.size(), g))) return s;
  BF_CUDA(cudaMemcpyAsync(sc.d_lvl, sc.lvl_item.data(), sc.lvl_item.size() * 4,
                          cudaMemcpyHostToDevice, st));
  BF_CUDA(cudaMemcpyAsync(sc.d_split, split_bits.data(), split_bits.size() * 4,
                          cudaMemcpyHostToDevice, st));
  if (!sc.cidx_ready) {
    BF_CUDA(cudaMemsetAsync(sc.d_cidx, 0xFF, (size_t)n * 4, st));
    sc.cidx_ready = true;
  }
  if (!pairs.empty()) {
    BF_CUDA(cudaMemcpyAsync(c.d_pairs, pairs.data(), pairs.size() * sizeof(uint2),
                            cudaMemcpyHostToDevice, st));
    const uint2* dp = reinterpret_cast<const uint2*>(c.d_pairs);
    if (n_reset)
      k_scatter_pairs<<<(unsigned)((n_reset + 255) / 256), 256, 0, st>>>(dp, n_reset, sc.d_cidx);
    if (n_r)
      k_scatter_pairs<<<(unsigned)((n_r + 255) / 256), 256, 0, st>>>(dp + n_reset, n_r,
                                                                      sc.d_cidx);
    BF_CUDA(cudaGetLastError());
  }
  if (n_i)
    BF_CUDA(cudaMemcpyAsync(sc.d_item, items, n_i * sizeof(uint4), cudaMemcpyHostToDevice, st));
  if (n_e)
    BF_CUDA(cudaMemcpyAsync(sc.d_erec, erec, n_e * sizeof(uint2), cudaMemcpyHostToDevice, st));
  if (two && n_e)
    BF_CUDA(cudaMemcpyAsync(sc.d_elen, elen, n_e * 4, cudaMemcpyHostToDevice, st));
  if (T) BF_CUDA(cudaMemcpyAsync(sc.d_trow, trow.data(), T * 4, cudaMemcpyHostToDevice, st));
  BF_CUDA(cudaStreamSynchronize(st));  // host vectors are freed on return
  sc.ranks.swap(ranks);
  sc.n_r = n_r;
  sc.n_items = n_i;
  sc.n_edges = n_e;
  sc.T = T;
  sc.key = key;
  if (all)
    sc.tgt.clear();
  else
    sc.tgt.assign(h_tgt, h_tgt + T);
  sc.valid = true;
  return BF_OK;
}

namespace {

// min-combine one warp's 128 lanes (thread t holds lanes 4t..4t+3 of the
// group starting at wbase) into a row with atomicMin, transposed through the
// warp's 512-byte shared-memory slice so that atomic instruction j covers the
// 32 consecutive lanes wbase + 32j .. +31: one 128-byte line per instruction
// instead of 16 sectors. Every thread of the warp must call it.
__device__ __forceinline__ void atomic_min_lanes(uint32_t* row, uint32_t wbase, uint4 acc,
                                                 uint32_t Kp, uint32_t* wbuf) {
  const uint32_t t = threadIdx.x & 31;
  reinterpret_cast<uint4*>(wbuf)[t] = acc;
  __syncwarp();
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint32_t v = wbuf[32 * j + t];
    const uint32_t L = wbase + 32 * j + t;
    if (L < Kp && v != INF) atomicMin(row + L, v);
  }
}

// One level of the restricted sweep. blockIdx.x = work item, a thread owns
// 4 consecutive lanes starting at lane; rows are Kp lanes wide (Kp % 4 == 0).
__global__ void __launch_bounds__(256)
    k_sweep_items(const uint4* __restrict__ item, uint32_t i0, const uint2* __restrict__ erec,
                  uint32_t* __restrict__ slab, uint32_t Kp, const uint32_t* __restrict__ seeded,
                  const uint32_t* __restrict__ hub, uint32_t hinted) {
  // launched as a programmatic dependent of the previous level: let the next
  // level's blocks get scheduled, read the static schedule, then wait for the
  // previous level's rows (no-ops for a plain launch)
  asm volatile("griddepcontrol.launch_dependents;");
  const uint4 it = item[i0 + blockIdx.x];
  const uint32_t lane = (blockIdx.y * blockDim.x + threadIdx.x) * 4;
  const uint32_t wbase = lane - 4 * (threadIdx.x & 31);
  if (wbase >= Kp) return;  // the whole warp is past the last lane
  const bool live = lane < Kp;
  // when the slab is much larger than L2, rows gathered most often (hub
  // rows) stay in L2: their loads and stores carry an evict-last policy,
  // every other row evict-first; a slab of L2 scale keeps normal eviction
  const uint64_t pl = l2_policy_last(), pf = hinted ? l2_policy_first() : l2_policy_normal();
  asm volatile("griddepcontrol.wait;" ::: "memory");
  uint4 acc = make_uint4(INF, INF, INF, INF);
  if (live) {
    uint32_t e = it.y;
    for (; e + 2 <= it.z; e += 2) {
      const uint2 r0 = erec[e], r1 = erec[e + 1];
      const uint4 a = ld_hint(slab + (size_t)r0.x * Kp + lane, is_hub(hub, r0.x) ? pl : pf);
      const uint4 b = ld_hint(slab + (size_t)r1.x * Kp + lane, is_hub(hub, r1.x) ? pl : pf);
      acc.x = min(acc.x, min(sat_add(a.x, r0.y), sat_add(b.x, r1.y)));
      acc.y = min(acc.y, min(sat_add(a.y, r0.y), sat_add(b.y, r1.y)));
      acc.z = min(acc.z, min(sat_add(a.z, r0.y), sat_add(b.z, r1.y)));
      acc.w = min(acc.w, min(sat_add(a.w, r0.y), sat_add(b.w, r1.y)));
    }
    if (e < it.z) {
      const uint2 r0 = erec[e];
      const uint4 a = ld_hint(slab + (size_t)r0.x * Kp + lane, is_hub(hub, r0.x) ? pl : pf);
      acc.x = min(acc.x, sat_add(a.x, r0.y));
      acc.y = min(acc.y, sat_add(a.y, r0.y));
      acc.z = min(acc.z, sat_add(a.z, r0.y));
      acc.w = min(acc.w, sat_add(a.w, r0.y));
    }
  }
  uint32_t* row = slab + (size_t)it.x * Kp;
  if (it.w) {  // one slice of a high in-degree node: combine atomically
    __shared__ __align__(16) uint32_t sbuf[256 * 4];
    atomic_min_lanes(row, wbase, acc, Kp, sbuf + (threadIdx.x & ~31u) * 4);
  } else if (live) {
    const uint64_t pw = is_hub(hub, it.x) ? pl : pf;
    // rows that got no seed this wave hold stale data: their value is the pull
    uint4 c = ((seeded[it.x >> 5] >> (it.x & 31)) & 1u) ? ld_hint(row + lane, pf)
                                                        : make_uint4(INF, INF, INF, INF);
    c.x = min(c.x, acc.x);
    c.y = min(c.y, acc.y);
    c.z = min(c.z, acc.z);
    c.w = min(c.w, acc.w);
    st_hint(row + lane, c, pw);
  }
}

// Gated variant for bounded sweeps with a threshold per lane: a row is
// "active" when some lane holds a value within that lane's threshold (bit in
// `active`). An item none of whose in-edge sources is active is skipped (its
// row keeps its seed or INF), and inactive source rows are not gathered: a
// value above a lane's threshold can only produce values above it, so every
// distance within the threshold is still exact. This is the GPU form of the
// reference's block gating (isochrone_handler.rs:419-452, batched_phast.rs:1093-1160).
__global__ void __launch_bounds__(128)
    k_sweep_gated(const uint4* __restrict__ item, uint32_t i0, const uint2* __restrict__ erec,
                  uint32_t* __restrict__ slab, uint32_t Kp, uint32_t* __restrict__ active,
                  const uint32_t* __restrict__ thr, uint32_t kw,
                  const uint32_t* __restrict__ seeded) {
  asm volatile("griddepcontrol.launch_dependents;");
  const uint4 it = item[i0 + blockIdx.x];
  asm volatile("griddepcontrol.wait;" ::: "memory");
  bool any = false;
  for (uint32_t e = it.y; e < it.z; ++e) {
    const uint32_t r = erec[e].x;
    any |= (active[r >> 5] >> (r & 31)) & 1u;
  }
  if (!any) return;  // uniform across the block
  const uint32_t lane = (blockIdx.y * blockDim.x + threadIdx.x) * 4;
  const uint32_t wbase = lane - 4 * (threadIdx.x & 31);
  if (wbase >= Kp) return;  // the whole warp is past the last lane
  const bool live = lane < Kp;
  uint4 acc = make_uint4(INF, INF, INF, INF);
  if (live)
    for (uint32_t e = it.y; e < it.z; ++e) {
      const uint2 r = erec[e];
      if (!((active[r.x >> 5] >> (r.x & 31)) & 1u)) continue;
      const uint4 a = *reinterpret_cast<const uint4*>(slab + (size_t)r.x * Kp + lane);
      acc.x = min(acc.x, sat_add(a.x, r.y));
      acc.y = min(acc.y, sat_add(a.y, r.y));
      acc.z = min(acc.z, sat_add(a.z, r.y));
      acc.w = min(acc.w, sat_add(a.w, r.y));
    }
  uint32_t* row = slab + (size_t)it.x * Kp;
  uint4 v = acc;
  if (it.w) {
    __shared__ __align__(16) uint32_t sbuf[128 * 4];
    atomic_min_lanes(row, wbase, acc, Kp, sbuf + (threadIdx.x & ~31u) * 4);
  } else if (live) {
    // without a full slab reset only seeded rows hold valid data here
    const bool valid = !seeded || ((seeded[it.x >> 5] >> (it.x & 31)) & 1u);
    v = valid ? *reinterpret_cast<const uint4*>(row + lane) : make_uint4(INF, INF, INF, INF);
    v.x = min(v.x, acc.x);
    v.y = min(v.y, acc.y);
    v.z = min(v.z, acc.z);
    v.w = min(v.w, acc.w);
    *reinterpret_cast<uint4*>(row + lane) = v;
  }
  const bool act = live && ((lane + 0 < kw && v.x <= thr[lane + 0]) ||
                            (lane + 1 < kw && v.y <= thr[lane + 1]) ||
                            (lane + 2 < kw && v.z <= thr[lane + 2]) ||
                            (lane + 3 < kw && v.w <= thr[lane + 3]));
  const unsigned m = __ballot_sync(0xFFFFFFFFu, act);
  if (m && (threadIdx.x & 31) == (unsigned)(__ffs(m) - 1))
    atomicOr(&active[it.x >> 5], 1u << (it.x & 31));
}

// Mark the slab rows of every origin's ancestor path (the rows the upward
// pass will seed): one warp per origin, whole runs of consecutive ranks at once.
__global__ void __launch_bounds__(128)
    k_mark_paths(const uint32_t* __restrict__ orig, uint32_t k, const uint32_t* __restrict__ parent,
                 const uint32_t* __restrict__ run_end, const uint32_t* __restrict__ cidx,
                 uint32_t* __restrict__ seeded) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= k) return;
  uint32_t x = orig[w];
  for (uint32_t guard = 0; x != NONE && guard < (1u << 30); ++guard) {
    // ancestors are shared: once a run's first node is marked, the warp that
    // marked it covers the rest of this same path
    const uint32_t r0 = cidx[x];
    if (r0 != NONE && ((*(volatile uint32_t*)&seeded[r0 >> 5] >> (r0 & 31)) & 1u)) break;
    const uint32_t e = run_end[x];
    for (uint32_t r = x + lane; r <= e; r += 32) {
      const uint32_t row = cidx[r];
      if (row != NONE) atomicOr(&seeded[row >> 5], 1u << (row & 31));
    }
    __syncwarp();
    x = parent[e];
  }
}

// Reset to INF the rows that are read before being fully written: rows that
// get seeds (seeded bits), rows without in-edges and rows whose in-edges are
// split over items (combined by atomicMin). All other rows are fully written
// by the sweep before anything reads them. One block per 32-row group.
__global__ void __launch_bounds__(256)
    k_init_rows(const uint32_t* __restrict__ seeded, const uint32_t* __restrict__ split,
                uint32_t words, uint32_t* __restrict__ slab, uint32_t Kp) {
  for (uint32_t gw = blockIdx.x; gw < words; gw += gridDim.x) {
    uint32_t m = seeded[gw] | split[gw];
    while (m) {
      const uint32_t b = __ffs(m) - 1;
      m &= m - 1;
      uint32_t* row = slab + (size_t)(gw * 32 + b) * Kp;
      for (uint32_t l = threadIdx.x * 4; l < Kp; l += blockDim.x * 4)
        *reinterpret_cast<uint4*>(row + l) = make_uint4(INF, INF, INF, INF);
    }
  }
}

// Same rows as k_init_rows for wide rows, stored by the bulk-copy engine from
// a shared-memory run of `ch` INF lanes: one thread per block issues one copy
// per row chunk, so the stores take no issue slots from the upward pass that
// runs beside them (10k x 10k: its phase 2.78 -> 2.66 ms). Rows are Kp * 4
// bytes with Kp % 4 == 0 and ch % 4 == 0, so every chunk starts on a 16-byte
// boundary of the (16-byte aligned) slab and is a multiple of 16 bytes long.
__global__ void __launch_bounds__(128)
    k_init_rows_bulk(const uint32_t* __restrict__ seeded, const uint32_t* __restrict__ split,
                     uint32_t words, uint32_t* __restrict__ slab, uint32_t Kp, uint32_t ch) {
  extern __shared__ __align__(128) uint4 infbuf[];
  for (uint32_t i = threadIdx.x; i < ch / 4; i += blockDim.x)
    infbuf[i] = make_uint4(INF, INF, INF, INF);
  // generic-proxy writes of the run made visible to the bulk copies
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (threadIdx.x != 0) return;
  const uint32_t sa = static_cast<uint32_t>(__cvta_generic_to_shared(infbuf));
  for (uint32_t gw = blockIdx.x; gw < words; gw += gridDim.x) {
    uint32_t m = seeded[gw] | split[gw];
    while (m) {
      const uint32_t b = __ffs(m) - 1;
      m &= m - 1;
      uint32_t* row = slab + (size_t)(gw * 32 + b) * Kp;
      for (uint32_t l = 0; l < Kp; l += ch) {
        const uint32_t nb = min(ch, Kp - l) * 4;
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                     :: "l"(row + l), "r"(sa), "r"(nb) : "memory");
      }
    }
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  }
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  // the shared run must outlive every copy reading it
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// out[s * T + t] = slab[trow[t]][s] (INF above the threshold); 32 x 32 tiles.
__global__ void __launch_bounds__(256)
    k_extract_lanes(const uint32_t* __restrict__ slab, uint32_t Kp,
                    const uint32_t* __restrict__ trow, uint64_t T, uint32_t S,
                    uint32_t threshold, uint32_t* __restrict__ out) {
  __shared__ uint32_t tile[32][33];
  const uint64_t t0 = (uint64_t)blockIdx.x * 32;
  const uint32_t l0 = blockIdx.y * 32;
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint64_t t = t0 + r;
    const uint32_t l = l0 + threadIdx.x;
    tile[r][threadIdx.x] = (t < T && l < S) ? slab[(size_t)trow[t] * Kp + l] : INF;
  }
  __syncthreads();
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint32_t l = l0 + r;
    const uint64_t t = t0 + threadIdx.x;
    if (l < S && t < T) {
      const uint32_t v = tile[threadIdx.x][r];
      out[(uint64_t)l * T + t] = v > threshold ? INF : v;
    }
  }
}

}  // namespace

}  // namespace bf

namespace bf {

// Grow the context's distance slab to at least `need` bytes.
// A slab that grows takes 1/16 more than asked when the budget allows:
// restricted row counts vary by a few percent between target sets, and each
// regrowth (cudaFree + cudaMalloc of gigabytes) stalls the stream.
bf_status ensure_slab(Graph* g, Ctx& c, size_t need) {
  if (need <= c.slab_bytes) return BF_OK;
  const size_t roomy = need + need / 16;
  const size_t alloc = roomy <= ctx_budget(g, c) ? roomy : need;
  if (c.d_slab) {
    cudaFree(c.d_slab);
    g->device_bytes -= c.slab_bytes;
    c.d_slab = nullptr;
    c.slab_bytes = 0;
  }
  if (alloc > need && cudaMalloc(&c.d_slab, alloc) == cudaSuccess) {
    c.slab_bytes = alloc;
    g->device_bytes += alloc;
    return BF_OK;
  }
  cudaGetLastError();
  c.d_slab = nullptr;
  if (cudaMalloc(&c.d_slab, need) != cudaSuccess) {
    cudaGetLastError();
    set_error("cannot allocate the batched distance slab (" + std::to_string(need) + " bytes)");
    return BF_ERR_OOM;
  }
  c.slab_bytes = need;
  g->device_bytes += need;
  return BF_OK;
}

// Slab bytes available to a context: its own budget, or what the graph's
// budget leaves (the context's current slab is reusable).
uint64_t ctx_budget(Graph* g, Ctx& c) {
  if (c.budget) return c.budget;
  const uint64_t used = g->device_bytes;
  return (g->hbm_budget > used ? g->hbm_budget - used : 0) + c.slab_bytes;
}

static void free_sched(Sched& sc) {
  void* p[] = {sc.d_cidx, sc.d_item, sc.d_erec, sc.d_elen, sc.d_trow, sc.d_split, sc.d_hub,
               sc.d_lvl, sc.d_uses, sc.d_hub_h, sc.d_lvl_erec};
  for (void* q : p)
    if (q) cudaFree(q);
  if (sc.gexec) cudaGraphExecDestroy(sc.gexec);
  if (sc.one_exec) cudaGraphExecDestroy(sc.one_exec);
  sc = Sched();
}

void free_ctx(Ctx& c) {
  free_sched(c.sc);
  free_sched(c.full);
  if (c.d_pairs) cudaFree(c.d_pairs);
  if (c.d_seeded) cudaFree(c.d_seeded);
  if (c.d_slab) cudaFree(c.d_slab);
  if (c.d_iso_tmp) cudaFree(c.d_iso_tmp);
  if (c.d_cseed) cudaFree(c.d_cseed);
  if (c.d_one) cudaFree(c.d_one);
  if (c.d_iso_prog) cudaFree(c.d_iso_prog);
  if (c.d_count) cudaFree(c.d_count);
  if (c.h_stage) cudaFreeHost(c.h_stage);
  free_sched_scratch(c.sd);
  for (auto& e : c.ev)
    if (e) cudaEventDestroy(e);
  if (c.fork) cudaEventDestroy(c.fork);
  if (c.join) cudaEventDestroy(c.join);
  if (c.aux) cudaStreamDestroy(c.aux);
  c = Ctx();
}

bf_status init_ctx(Ctx& c) {
  for (auto& e : c.ev) BF_CUDA(cudaEventCreate(&e));
  BF_CUDA(cudaStreamCreateWithFlags(&c.aux, cudaStreamNonBlocking));
  BF_CUDA(cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming));
  BF_CUDA(cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming));
  return BF_OK;
}

bf_status batched_prepare(Graph* g, uint32_t) {
  (void)g;
  return BF_OK;
}

// Hub rows of a schedule for rows of row_bytes: as many of the most-gathered
// rows as fit the tune's L2 share, as a device bitmap (*hub = null when off).
bf_status hub_rows(Graph* g, Sched& sc, uint64_t row_bytes, cudaStream_t st, const uint32_t** hub) {
  *hub = nullptr;
  uint32_t H = 0;
  const uint64_t ranked = sc.dev_built ? std::min<uint32_t>(sc.n_r, 65536) : sc.hub_order.size();
  if (g->tune.hub_mb && row_bytes)
    H = (uint32_t)std::min<uint64_t>(ranked, ((uint64_t)g->tune.hub_mb << 20) / row_bytes);
  if (!H) return BF_OK;
  if (H != sc.hub_rows && sc.dev_built) {
    bf_status rc;
    if ((rc = hub_rows_device(g, sc, H, st))) return rc;
    sc.hub_rows = H;
  } else if (H != sc.hub_rows) {
    std::vector<uint32_t> bits((std::max<uint32_t>(sc.n_r, 1) + 31) / 32, 0);
    for (uint32_t i = 0; i < H; ++i) bits[sc.hub_order[i] >> 5] |= 1u << (sc.hub_order[i] & 31);
    bf_status s;
    if ((s = ensure(&sc.d_hub, sc.cap_hub, bits.size(), g))) return s;
    BF_CUDA(cudaMemcpyAsync(sc.d_hub, bits.data(), bits.size() * 4, cudaMemcpyHostToDevice, st));
    sc.hub_rows = H;
  }
  *hub = sc.d_hub;
  return BF_OK;
}

// Launch the restricted sweep's level schedule. From the second call on the
// same schedule and slab geometry the launches are replayed from a captured
// CUDA graph instead of being issued one by one.
bf_status sweep_levels(Graph* g, Sched& sc, uint32_t* slab, uint32_t Kp, unsigned lane_blocks,
                       unsigned tpb, cudaStream_t st, uint64_t* launches,
                       const uint32_t* seeded) {
  const bool pdl = g->tune.pdl != 0;
  // cache hints only pay when the slab is well beyond L2 (otherwise
  // evict-first would drop lines that the sweep reads again)
  const bool hinted = (uint64_t)std::max<uint32_t>(sc.n_r, 1) * Kp * 4 > 4 * g->l2_bytes;
  const uint32_t* hub = nullptr;
  bf_status hs;
  if (hinted && (hs = hub_rows(g, sc, (uint64_t)Kp * 4, st, &hub))) return hs;
  auto issue = [&](cudaStream_t s, uint64_t* count) -> cudaError_t {
    for (uint32_t l = 0; l < g->n_levels; ++l) {
      const uint32_t i0 = sc.lvl_item[l], i1 = sc.lvl_item[l + 1];
      if (i1 == i0) continue;
      cudaError_t e = launch_level(k_sweep_items, dim3(i1 - i0, lane_blocks), tpb, pdl, s,
                                   (const uint4*)sc.d_item, i0, (const uint2*)sc.d_erec, slab, Kp,
                                   seeded, hub, hinted ? 1u : 0u);
      if (e != cudaSuccess) return e;
      ++*count;
    }
    return cudaSuccess;
  };
  const bool geom = sc.g_kp == Kp && sc.g_lb == lane_blocks && sc.g_tpb == tpb &&
                    sc.g_slab == slab && sc.g_stream == st && sc.g_seeded == seeded &&
                    sc.g_pdl == pdl && sc.g_hub == hub && sc.g_hinted == hinted;
  if (sc.gexec && !geom) {
    cudaGraphExecDestroy(sc.gexec);
    sc.gexec = nullptr;
  }
  if (!sc.gexec && sc.uses >= 1 && g->tune.graphs) {
    cudaStreamCaptureStatus cs;
    BF_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusNone) {
      uint64_t dummy = 0;
      cudaGraph_t graph;
      BF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      const cudaError_t le = issue(st, &dummy);
      const cudaError_t ce = cudaStreamEndCapture(st, &graph);
      if (le != cudaSuccess) {
        if (ce == cudaSuccess) cudaGraphDestroy(graph);
        return cuda_status(le, "level launch during capture");
      }
      if (ce != cudaSuccess) return cuda_status(ce, "cudaStreamEndCapture");
      cudaError_t e = cudaGraphInstantiate(&sc.gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate");
      sc.g_kp = Kp;
      sc.g_lb = lane_blocks;
      sc.g_tpb = tpb;
      sc.g_slab = slab;
      sc.g_stream = st;
      sc.g_seeded = seeded;
      sc.g_pdl = pdl;
      sc.g_hub = hub;
      sc.g_hinted = hinted;
    }
  }
  if (sc.gexec && g->tune.graphs) {
    BF_CUDA(cudaGraphLaunch(sc.gexec, st));
    for (uint32_t l = 0; l < g->n_levels; ++l)
      if (sc.lvl_item[l + 1] != sc.lvl_item[l]) ++*launches;
  } else {
    BF_CUDA(issue(st, launches));
  }
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

// Gated level schedule (launched directly: the skip decisions depend on the
// data of each call).
bf_status sweep_levels_gated(Graph* g, Sched& sc, uint32_t* slab, uint32_t Kp, unsigned lane_blocks,
                             unsigned tpb, uint32_t* active, const uint32_t* thr, uint32_t kw,
                             cudaStream_t st, uint64_t* launches, const uint32_t* seeded) {
  const bool pdl = g->tune.pdl != 0;
  for (uint32_t l = 0; l < g->n_levels; ++l) {
    const uint32_t i0 = sc.lvl_item[l], i1 = sc.lvl_item[l + 1];
    if (i1 == i0) continue;
    BF_CUDA(launch_level(k_sweep_gated, dim3(i1 - i0, lane_blocks), tpb, pdl, st,
                         (const uint4*)sc.d_item, i0, (const uint2*)sc.d_erec, slab, Kp, active,
                         thr, kw, seeded));
    ++*launches;
  }
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

void launch_extract_lanes(const uint32_t* slab, uint32_t Kp, const uint32_t* trow, uint64_t T,
                          uint32_t S, uint32_t threshold, uint32_t* out, cudaStream_t st) {
  dim3 eg((unsigned)((T + 31) / 32), (unsigned)((S + 31) / 32)), eb(32, 8);
  k_extract_lanes<<<eg, eb, 0, st>>>(slab, Kp, trow, T, S, threshold, out);
}

void launch_mark_paths(Graph* g, const uint32_t* d_src, uint64_t k, const uint32_t* cidx,
                       uint32_t* seeded, cudaStream_t st) {
  if (!k) return;
  k_mark_paths<<<(unsigned)((k + 3) / 4), 128, 0, st>>>(d_src, (uint32_t)k, g->d_parent,
                                                        g->d_run_end, cidx, seeded);
}

void launch_init_rows(const uint32_t* seeded, const uint32_t* split, uint32_t words,
                      uint32_t* slab, uint32_t Kp, cudaStream_t st) {
  const uint32_t grid = std::min<uint32_t>(words, 152 * 32);
  if (Kp >= 1024 && Kp % 4 == 0 && (reinterpret_cast<uintptr_t>(slab) & 15) == 0) {
    const uint32_t ch = std::min<uint32_t>(Kp, 8192);  // 32 KB of shared memory at most
    k_init_rows_bulk<<<grid, 128, ch * 4, st>>>(seeded, split, words, slab, Kp, ch);
    return;
  }
  k_init_rows<<<grid, Kp >= 1024 ? 256 : 64, 0, st>>>(seeded, split, words, slab, Kp);
}

bf_status prepare_rows(Graph* g, Ctx& c, Sched& sc, const uint32_t* d_src, uint64_t kw,
                       uint32_t Kp, cudaStream_t st, uint64_t* launches) {
  const uint32_t words = (std::max<uint32_t>(sc.n_r, 1) + 31) / 32;
  bf_status s;
  if ((s = ensure(&c.d_seeded, c.cap_seeded, words, g))) return s;
  BF_CUDA(cudaMemsetAsync(c.d_seeded, 0, (size_t)words * 4, st));
  launch_mark_paths(g, d_src, kw, sc.d_cidx, c.d_seeded, st);
  // only rows the sweep does not overwrite whole need INF first (seeded,
  // split and in-edge-free rows; 10k x 10k: 2.8 against 3.5 ms for a reset
  // of the whole slab beside the upward pass)
  launch_init_rows(c.d_seeded, sc.d_split, words, c.d_slab, Kp, st);
  BF_CUDA(cudaGetLastError());
  *launches += 2;
  return BF_OK;
}

// One wave on the context's current target-restricted schedule: reset the
// slab, upward pass for kw sources, restricted sweep. Records c.ev[0..2]
// around the phases when `timed`.
bf_status batched_wave(Graph* g, Ctx& c, const uint32_t* d_src, uint64_t kw, uint32_t Kp,
                       cudaStream_t st, uint64_t* launches, bool timed, uint64_t pre_stride,
                       uint64_t pre_col) {
  bf_status s;
  Sched& sc = c.sc;
  const uint64_t rows = std::max<uint32_t>(sc.n_r, 1);
  const unsigned tpb = std::min<uint32_t>(g->tune.tpb, ((Kp / 4 + 31) / 32) * 32);
  const unsigned lane_blocks = (Kp / 4 + tpb - 1) / tpb;
  (void)rows;
  if (timed) BF_CUDA(cudaEventRecord(c.ev[0], st));
  // the upward pass is latency-bound and the row reset bandwidth-bound: with
  // a shallow enough tree the pass runs on the side stream into a compact
  // buffer of ranks while the reset runs here, and a scatter maps them to
  // rows (the pass may also have run before the schedule was built)
  const uint32_t dcap = ((g->max_depth + 1) + 31) & ~31u;
  const bool overlap =
      pre_stride || (g->tune.overlap_up && c.aux && (size_t)UPWARD_WARPS * 2 * dcap * 4 <= 200 * 1024);
  if (overlap) {
    const uint32_t words = (std::max<uint32_t>(sc.n_r, 1) + 31) / 32;
    if ((s = ensure(&c.d_seeded, c.cap_seeded, words, g))) return s;
    if (!pre_stride && (s = ensure(&c.d_cseed, c.cap_cseed, kw * (g->max_depth + 1), g))) return s;
    BF_CUDA(cudaMemsetAsync(c.d_seeded, 0, (size_t)words * 4, st));
    launch_mark_paths(g, d_src, kw, sc.d_cidx, c.d_seeded, st);
    if (!pre_stride) {
      BF_CUDA(cudaEventRecord(c.fork, st));
      BF_CUDA(cudaStreamWaitEvent(c.aux, c.fork, 0));
      if ((s = launch_upward(g, d_src, kw, INF, nullptr, reinterpret_cast<uint32_t*>(c.d_cseed),
                             (uint32_t)kw, nullptr, c.aux, nullptr, nullptr, nullptr,
                             UPWARD_OUT_COMPACT)))
        return s;
      BF_CUDA(cudaEventRecord(c.join, c.aux));
      ++*launches;
    }
    // only rows the sweep does not overwrite whole need INF first: seeded
    // rows (read back by their item), split rows (atomicMin targets) and rows
    // without in-edges (read, never written) - sc.d_split marks the last two
    launch_init_rows(c.d_seeded, sc.d_split, words, c.d_slab, Kp, st);
    BF_CUDA(cudaStreamWaitEvent(st, c.join, 0));
    if ((s = launch_scatter_seeds(g, c.d_cseed, kw, d_src, c.d_slab, Kp, st,
                                  pre_stride ? pre_stride : kw, pre_col, sc.d_cidx)))
      return s;
    *launches += 3;
  } else {
    if ((s = prepare_rows(g, c, sc, d_src, kw, Kp, st, launches))) return s;
    if ((s = launch_upward(g, d_src, kw, INF, sc.d_cidx, c.d_slab, Kp, nullptr, st))) return s;
    ++*launches;
  }
  if (timed) BF_CUDA(cudaEventRecord(c.ev[1], st));
  return sweep_levels(g, sc, c.d_slab, Kp, lane_blocks, tpb, st, launches, c.d_seeded);
}

bf_status batched_matrix(Graph* g, Ctx& c, const uint32_t* d_src, uint64_t S, const uint32_t* d_tgt,
                         uint64_t T, uint32_t threshold, uint32_t* d_out, cudaStream_t st,
                         bf_stats* stats) {
  bf_status s;
  // the upward pass needs only the sources: with a shallow tree it runs on
  // the side stream from here, beside the target check and the restricted
  // schedule's build, into a compact buffer of ranks for all S sources
  const uint32_t dcap = ((g->max_depth + 1) + 31) & ~31u;
  const uint64_t pre_entries = S * (uint64_t)(g->max_depth + 1);
  const bool pre = S && g->tune.overlap_up && c.aux &&
                   (size_t)UPWARD_WARPS * 2 * dcap * 4 <= 200 * 1024 &&
                   pre_entries * sizeof(uint2) <= (1ull << 30);
  uint64_t pre_launches = 0;
  if (pre) {
    if ((s = ensure(&c.d_cseed, c.cap_cseed, pre_entries, g))) return s;
    BF_CUDA(cudaEventRecord(c.fork, st));
    BF_CUDA(cudaStreamWaitEvent(c.aux, c.fork, 0));
    if ((s = launch_upward(g, d_src, S, INF, nullptr, reinterpret_cast<uint32_t*>(c.d_cseed),
                           (uint32_t)S, nullptr, c.aux, nullptr, nullptr, nullptr,
                           UPWARD_OUT_COMPACT)))
      return s;
    BF_CUDA(cudaEventRecord(c.join, c.aux));
    pre_launches = 1;
  }
  std::vector<uint32_t> h_tgt(T);
  BF_CUDA(cudaMemcpyAsync(h_tgt.data(), d_tgt, T * 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  for (uint64_t i = 0; i < T; ++i)
    if (h_tgt[i] >= g->n) {
      set_error("targets[" + std::to_string(i) + "] is not a node of the graph");
      return BF_ERR_INVALID;
    }
  const auto tb = std::chrono::steady_clock::now();
  if ((s = build_schedule(g, c, c.sc, h_tgt.data(), T, false, st, d_tgt))) return s;
  if (stats)
    stats->schedule_ms +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
  Sched& sc = c.sc;
  const uint64_t rows = std::max<uint32_t>(sc.n_r, 1);
  // lanes per wave: all sources if the slab fits the budget, else waves
  uint64_t max_lanes = ctx_budget(g, c) / (rows * 4);
  max_lanes = max_lanes >= 32 ? max_lanes & ~31ull : 0;
  if (max_lanes == 0) {
    set_error("HBM budget too small for one 32-lane wave of the restricted slab");
    return BF_ERR_OOM;
  }
  if (g->tune.max_lanes) max_lanes = std::min<uint64_t>(max_lanes, g->tune.max_lanes);
  const uint64_t wave = std::min<uint64_t>(max_lanes, (S + 3) & ~3ull);
  const uint32_t Kp = (uint32_t)((wave + 3) & ~3ull);
  if ((s = ensure_slab(g, c, (size_t)rows * Kp * 4))) return s;
  uint64_t launches = pre_launches;
  float t_up = 0, t_dn = 0, t_ex = 0;
  for (uint64_t s0 = 0; s0 < S; s0 += wave) {
    const uint64_t kw = std::min<uint64_t>(wave, S - s0);
    if ((s = batched_wave(g, c, d_src + s0, kw, Kp, st, &launches, stats != nullptr,
                          pre ? S : 0, s0)))
      return s;
    if (stats) BF_CUDA(cudaEventRecord(c.ev[2], st));
    dim3 eg((unsigned)((T + 31) / 32), (unsigned)((kw + 31) / 32)), eb(32, 8);
    k_extract_lanes<<<eg, eb, 0, st>>>(c.d_slab, Kp, sc.d_trow, T, (uint32_t)kw, threshold,
                                       d_out + s0 * T);
    BF_CUDA(cudaGetLastError());
    ++launches;
    if (stats) {
      BF_CUDA(cudaEventRecord(c.ev[3], st));
      BF_CUDA(cudaEventSynchronize(c.ev[3]));
      float ea, eb, ec;
      BF_CUDA(cudaEventElapsedTime(&ea, c.ev[0], c.ev[1]));
      BF_CUDA(cudaEventElapsedTime(&eb, c.ev[1], c.ev[2]));
      BF_CUDA(cudaEventElapsedTime(&ec, c.ev[2], c.ev[3]));
      t_up += ea;
      t_dn += eb;
      t_ex += ec;
    }
  }
  if (stats) {
    stats->n_batches += (S + wave - 1) / wave;
    stats->waves += (S + wave - 1) / wave;
    stats->swept_nodes = sc.n_r;
    stats->swept_edges = sc.n_edges;
    stats->lanes = Kp;
    stats->kernel_launches += launches;
    stats->upward_ms += t_up;
    stats->downward_ms += t_dn;
    stats->extract_ms += t_ex;
  }
  return BF_OK;
}

}  // namespace bf
