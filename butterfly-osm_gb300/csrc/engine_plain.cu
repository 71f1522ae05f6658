// engine_plain.cu — the plain GPU sweep: one K = 32 batch at a time.
//
//   1. k_upward: one warp per source walks the source's elimination-tree
//      ancestor path in increasing rank order and relaxes UP edges into a
//      path-indexed distance array (replaces the per-lane BinaryHeap Dijkstra
//      of batched_phast.rs:156-189; ranks are a topological order of the UP
//      DAG, so a node's distance is final once every lower path node has
//      pushed). Settled (node, dist) pairs land in a seed slab.
//   2. k_sweep_level: one launch per level of the pull DAG; a warp per node,
//      lane = source. dist[v][lane] = min(seed, min over DOWN in-edges
//      (u -> v, w) of dist[u][lane] + w) — the pull form of the rank-
//      descending push scan of batched_phast.rs:205-250.
//   3. k_extract: gathers the target rows and writes the S x T row-major
//      matrix through a shared-memory transpose (batched_phast.rs:693-701).

#include <algorithm>
#include <cstdlib>

#include "engine.cuh"

namespace bf {

namespace {

template <bool GLOBAL_PATH>
__device__ __forceinline__ uint32_t pd_load(const uint32_t* p) {
  if (GLOBAL_PATH) return __ldcg(p);
  return *(const volatile uint32_t*)p;
}

}  // namespace

// Upward pass: warp w walks source (or seed unit) w's ancestor path in
// increasing rank order (replaces the per-lane BinaryHeap Dijkstra of
// batched_phast.rs:156-189; ranks are a topological order of the UP DAG, so a
// node's distance is final once every lower path node has pushed). Each warp
// keeps its path (nodes and distances) in dcap-entry arrays: shared memory
// (GLOBAL = false), or for elimination trees too deep for it a per-warp slot
// of global scratch (warps w0 .. w0 + launch size). The UP-edge ranges of 32
// path nodes are fetched in one parallel load and broadcast by shuffle, and
// the first edge record of the next path node is loaded while the current one
// is relaxed, so a path step costs about one memory round trip instead of two
// dependent ones.
template <bool GLOBAL>
__global__ void __launch_bounds__(UPWARD_WARPS * 32, 4)
    k_upward_fast(const uint32_t* __restrict__ src, uint32_t k, uint32_t threshold,
                  const uint32_t* __restrict__ parent, const uint32_t* __restrict__ run_end,
                  const uint32_t* __restrict__ depth, const uint64_t* __restrict__ up_off,
                  const uint2* __restrict__ up_rec, const uint32_t* __restrict__ pos_of,
                  uint32_t n, uint32_t* __restrict__ seed, uint32_t seed_stride,
                  uint32_t* __restrict__ flag, uint32_t dcap, uint32_t* __restrict__ err,
                  const uint32_t* __restrict__ lane_thr, const uint32_t* __restrict__ unit_cost,
                  const uint32_t* __restrict__ unit_lane, uint32_t mode, uint32_t w0,
                  uint32_t* __restrict__ gscratch) {
  extern __shared__ uint32_t smem[];
  const uint32_t wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t slot = blockIdx.x * UPWARD_WARPS + wib;
  const uint32_t w = w0 + slot;
  if (w >= k) return;
  const uint32_t s = src[w];
  if (s >= n) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  const uint32_t D = depth[s] + 1;
  uint32_t* pd = GLOBAL ? gscratch + (size_t)slot * 2 * dcap : smem + wib * 2 * dcap;
  uint32_t* pn = pd + dcap;
#define PN(x) (GLOBAL ? __ldcg(&pn[(x)]) : pn[(x)])
  if (D > dcap || walk_path(s, D, parent, run_end, pn, lane) != D) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  // a seeded unit starts at its seed cost and writes (min) into its source's lane
  const uint32_t c0 = unit_cost ? unit_cost[w] : 0u;
  const uint32_t out_lane = unit_lane ? unit_lane[w] : w;
  // a per-lane threshold also bounds the relaxations: values above it can
  // never lead to a distance within it
  if (lane_thr) threshold = min(threshold, lane_thr[out_lane]);
  for (uint32_t l = lane; l < D; l += 32) pd[l] = (l == 0) ? c0 : INF;
  if (GLOBAL) __threadfence_block();
  __syncwarp();
  const unsigned FULL = 0xFFFFFFFFu;
  uint64_t cb = 0, ce = 0;  // edge range of path node (chunk base + lane)
  if (lane < D) {
    const uint32_t x = PN(lane);
    cb = up_off[x];
    ce = up_off[x + 1];
  }
  uint64_t b_cur = __shfl_sync(FULL, cb, 0), e_cur = __shfl_sync(FULL, ce, 0);
  uint2 rec = (b_cur + lane < e_cur) ? up_rec[b_cur + lane] : make_uint2(0, 0);
  for (uint32_t i = 0; i < D; ++i) {
    const uint32_t j = i + 1;
    if ((j & 31) == 0 && j < D) {
      cb = ce = 0;
      if (j + lane < D) {
        const uint32_t x = PN(j + lane);
        cb = up_off[x];
        ce = up_off[x + 1];
      }
    }
    const uint64_t b_nx = __shfl_sync(FULL, cb, j & 31), e_nx = __shfl_sync(FULL, ce, j & 31);
    const uint2 nrec =
        (j < D && b_nx + lane < e_nx) ? up_rec[b_nx + lane] : make_uint2(0, 0);
    const uint32_t d = pd_load<GLOBAL>(&pd[i]);
    if (d != INF && d <= threshold) {
      if (b_cur + lane < e_cur) {
        const uint32_t t = i + rec.x;
        if (t < D) atomicMin(&pd[t], sat_add(d, rec.y));
        else atomicOr(err, DEVERR_EDGE);
      }
      // high-degree path nodes (the dense top separators): issue 8 record
      // loads before the first atomic so their latencies overlap
      for (uint64_t e0 = b_cur + 32; e0 < e_cur; e0 += 256) {
        uint2 r[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const uint64_t e = e0 + q * 32 + lane;
          r[q] = e < e_cur ? up_rec[e] : make_uint2(0xFFFFFFFFu, 0);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (r[q].x == 0xFFFFFFFFu) continue;
          const uint32_t t = i + r[q].x;
          if (t < D) atomicMin(&pd[t], sat_add(d, r[q].y));
          else atomicOr(err, DEVERR_EDGE);
        }
      }
    }
    if (GLOBAL) __threadfence_block();
    __syncwarp();
    rec = nrec;
    b_cur = b_nx;
    e_cur = e_nx;
  }
  // with lane_thr, a seed above this lane's own threshold can never reach a
  // node within it: it is written but does not mark its row active
  const uint32_t lt = lane_thr ? lane_thr[out_lane] : threshold;
  if (mode == UPWARD_OUT_COMPACT) {
    // entry (D-1-l) * seed_stride + w: indexed from the root, so entries of
    // different sources at one index mostly name the same top-of-tree row
    uint2* out = reinterpret_cast<uint2*>(seed);
    for (uint32_t l = lane; l < D; l += 32) {
      const uint32_t d = pd_load<GLOBAL>(&pd[l]);
      const uint32_t x = PN(l);
      const uint32_t p = (d == INF || d > threshold) ? NONE : (pos_of ? pos_of[x] : x);
      out[(size_t)(D - 1 - l) * seed_stride + w] = make_uint2(p, d);
    }
    return;
  }
  for (uint32_t l = lane; l < D; l += 32) {
    const uint32_t d = pd_load<GLOBAL>(&pd[l]);
    if (d == INF || d > threshold) continue;
    const uint32_t p = pos_of[PN(l)];
    if (p == NONE) continue;
    if (unit_lane) atomicMin(&seed[(size_t)p * seed_stride + out_lane], d);
    else if (mode == UPWARD_OUT_SLAB16)  // every stored d is within its lane threshold (< 0xFFFF)
      reinterpret_cast<uint16_t*>(seed)[(size_t)p * seed_stride + w] = (uint16_t)d;
    else seed[(size_t)p * seed_stride + w] = d;
    if (flag && d <= lt) atomicOr(&flag[p >> 5], 1u << (p & 31));
  }
}
#undef PN

// Path node at path index idx of a warp's ancestor path held as runs of
// consecutive ranks: lane r holds run r's first node (r_node) and first path
// index (r_idx; ~0 on lanes past the last run). Called by all lanes.
__device__ __forceinline__ uint32_t path_node(uint32_t idx, uint32_t r_node, uint32_t r_idx) {
  uint32_t lo = 0;
#pragma unroll
  for (uint32_t b = 16; b; b >>= 1) {
    const uint32_t c = __shfl_sync(0xFFFFFFFFu, r_idx, lo + b);
    if (c <= idx) lo += b;
  }
  return __shfl_sync(0xFFFFFFFFu, r_node, lo) + (idx - __shfl_sync(0xFFFFFFFFu, r_idx, lo));
}

// Upward pass for ancestor paths of at most 32 runs (the common case: paths
// are chains of separator runs; the country graph's have 12 on average and 21
// at most). The same walk as k_upward_fast, with three changes that cut its
// instructions per relaxation and raise occupancy:
//   - the path's nodes are not stored: lane r keeps run r, and the node at a
//     path index is found by a 5-step shuffle search (once per 32 steps for
//     the UP-edge ranges, and in the output), so shared memory holds only the
//     path distances (dcap words per warp: 10 blocks per SM instead of 5);
//   - a node's UP edges are walked in exact 32-edge chunks (four loads issued
//     before their relaxations) with 32-bit offsets, instead of groups of
//     eight chunks with sentinel records;
//   - the UP-edge ranges of the next 32 path nodes are loaded 32 steps
//     ahead, so the range loads never stall a step.
// Every UP edge u -> v has v on u's root path (elimination-tree ancestors),
// so t = i + rec.x < D; the bound is still checked before each atomic.
__global__ void __launch_bounds__(UPWARD_WARPS * 32, 10)
    k_upward_runs(const uint32_t* __restrict__ src, uint32_t k, uint32_t threshold,
                  const uint32_t* __restrict__ parent, const uint32_t* __restrict__ run_end,
                  const uint32_t* __restrict__ depth, const uint64_t* __restrict__ up_off,
                  const uint2* __restrict__ up_rec, const uint32_t* __restrict__ pos_of,
                  uint32_t n, uint32_t* __restrict__ seed, uint32_t seed_stride,
                  uint32_t* __restrict__ flag, uint32_t dcap, uint32_t* __restrict__ err,
                  const uint32_t* __restrict__ lane_thr, const uint32_t* __restrict__ unit_cost,
                  const uint32_t* __restrict__ unit_lane, uint32_t mode) {
  extern __shared__ uint32_t smem[];
  constexpr unsigned FULL = 0xFFFFFFFFu;
  const uint32_t wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t w = blockIdx.x * UPWARD_WARPS + wib;
  if (w >= k) return;
  const uint32_t s = src[w];
  if (s >= n) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  const uint32_t D = depth[s] + 1;
  uint32_t* pd = smem + wib * dcap;
  // the path as runs [x, run_end[x]], each continuing at the parent of its end
  uint32_t r_node = 0, r_idx = 0xFFFFFFFFu;
  {
    uint32_t x = s, i = 0, r = 0;
    for (; x != NONE && r < 32 && i < D; ++r) {
      const uint32_t e = run_end[x];
      if (e < x || e >= n) break;
      if (lane == r) {
        r_node = x;
        r_idx = i;
      }
      i += e - x + 1;
      x = parent[e];
    }
    if (x != NONE || i != D || D > dcap) {
      if (lane == 0) atomicOr(err, DEVERR_PATH);
      return;
    }
  }
  const uint32_t c0 = unit_cost ? unit_cost[w] : 0u;
  const uint32_t out_lane = unit_lane ? unit_lane[w] : w;
  if (lane_thr) threshold = min(threshold, lane_thr[out_lane]);
  const uint32_t thr1 = min(threshold, INF - 1);  // d must also be finite
  for (uint32_t l = lane; l < D; l += 32) pd[l] = (l == 0) ? c0 : INF;
  __syncwarp();
  // UP-edge ranges of path nodes [j0, j0 + 32): lane l holds node j0 + l's
  uint64_t cb, nb;
  uint32_t cn, nn;
  {
    const uint32_t x = path_node(min(lane, D - 1), r_node, r_idx);
    cb = up_off[x];
    cn = lane < D ? (uint32_t)(up_off[x + 1] - cb) : 0u;
    const uint32_t x2 = path_node(min(32 + lane, D - 1), r_node, r_idx);
    nb = up_off[x2];
    nn = 32 + lane < D ? (uint32_t)(up_off[x2 + 1] - nb) : 0u;
  }
  uint64_t b_cur = __shfl_sync(FULL, cb, 0);
  uint32_t n_cur = __shfl_sync(FULL, cn, 0);
  uint2 rec = lane < n_cur ? up_rec[b_cur + lane] : make_uint2(0, 0);
  for (uint32_t i = 0; i < D; ++i) {
    const uint32_t j = i + 1;
    if ((j & 31) == 0) {
      cb = nb;
      cn = nn;
      const uint32_t jn = j + 32 + lane;
      const uint32_t x = path_node(min(jn, D - 1), r_node, r_idx);
      if (j + 32 < D) {
        nb = up_off[x];
        nn = jn < D ? (uint32_t)(up_off[x + 1] - nb) : 0u;
      } else {
        nb = 0;
        nn = 0;
      }
    }
    const uint64_t b_nx = __shfl_sync(FULL, cb, j & 31);
    const uint32_t n_nx = __shfl_sync(FULL, cn, j & 31);
    const uint2 nrec = lane < n_nx ? up_rec[b_nx + lane] : make_uint2(0, 0);
    const uint32_t d = *(volatile const uint32_t*)&pd[i];
    if (d <= thr1) {
      if (lane < n_cur) {
        const uint32_t t = i + rec.x;
        if (t < D) atomicMin(&pd[t], sat_add(d, rec.y));
      }
      const uint2* rp = up_rec + b_cur;
      for (uint32_t c = 32 + lane; c < n_cur + lane; c += 128) {
        uint2 r[4];
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q)
          r[q] = c + q * 32 < n_cur ? rp[c + q * 32] : make_uint2(D, 0);
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
          const uint32_t t = i + r[q].x;
          if (t < D) atomicMin(&pd[t], sat_add(d, r[q].y));
        }
      }
    }
    __syncwarp();
    rec = nrec;
    b_cur = b_nx;
    n_cur = n_nx;
  }
  const uint32_t lt = lane_thr ? lane_thr[out_lane] : threshold;
  if (mode == UPWARD_OUT_COMPACT) {
    uint2* out = reinterpret_cast<uint2*>(seed);
    for (uint32_t l0 = 0; l0 < D; l0 += 32) {
      const uint32_t l = l0 + lane;
      const uint32_t x = path_node(min(l, D - 1), r_node, r_idx);
      if (l >= D) continue;
      const uint32_t d = pd[l];
      const uint32_t p = (d == INF || d > threshold) ? NONE : (pos_of ? pos_of[x] : x);
      out[(size_t)(D - 1 - l) * seed_stride + w] = make_uint2(p, d);
    }
    return;
  }
  for (uint32_t l0 = 0; l0 < D; l0 += 32) {
    const uint32_t l = l0 + lane;
    const uint32_t x = path_node(min(l, D - 1), r_node, r_idx);
    if (l >= D) continue;
    const uint32_t d = pd[l];
    if (d == INF || d > threshold) continue;
    const uint32_t p = pos_of[x];
    if (p == NONE) continue;
    if (unit_lane) atomicMin(&seed[(size_t)p * seed_stride + out_lane], d);
    else if (mode == UPWARD_OUT_SLAB16)  // every stored d is within its lane threshold (< 0xFFFF)
      reinterpret_cast<uint16_t*>(seed)[(size_t)p * seed_stride + w] = (uint16_t)d;
    else seed[(size_t)p * seed_stride + w] = d;
    if (flag && d <= lt) atomicOr(&flag[p >> 5], 1u << (p & 31));
  }
}

// Compact upward output -> slab: thread (w, i) writes entry i (counted from
// the root) of source w's ancestor path into lane w of its row. Consecutive
// threads are consecutive lanes, and near the root their rows coincide, so
// those writes are whole lines. Entries are read at column col0 + w of rows
// `stride` wide; with `cidx` they name ranks, mapped to rows here (NONE: a
// rank outside the restricted schedule).
__global__ void __launch_bounds__(256)
    k_scatter_seeds(const uint2* __restrict__ cseed, uint32_t k, const uint32_t* __restrict__ src,
                    const uint32_t* __restrict__ depth, uint32_t* __restrict__ slab, uint32_t Kp,
                    uint32_t stride, uint32_t col0, const uint32_t* __restrict__ cidx) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (w >= k || i > depth[src[w]]) return;
  const uint2 e = cseed[(size_t)i * stride + col0 + w];
  if (e.x == NONE) return;
  const uint32_t row = cidx ? cidx[e.x] : e.x;
  if (row != NONE) slab[(size_t)row * Kp + w] = e.y;
}

// One level of the pull sweep: positions [p0, p1), a warp per node.
__global__ void __launch_bounds__(256)
    k_sweep_level(uint32_t p0, uint32_t p1, const uint64_t* __restrict__ in_off,
                  const uint2* __restrict__ in_rec, uint32_t* __restrict__ dist,
                  uint32_t* __restrict__ seed, uint32_t* __restrict__ flag, uint32_t threshold) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t p = p0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (p >= p1) return;
  uint32_t best = INF;
  const uint32_t bit = 1u << (p & 31);
  if (flag[p >> 5] & bit) {
    best = seed[(size_t)p * PLAIN_K + lane];
    seed[(size_t)p * PLAIN_K + lane] = INF;
    __syncwarp();
    if (lane == 0) atomicAnd(&flag[p >> 5], ~bit);
  }
  uint64_t e = in_off[p];
  const uint64_t e1 = in_off[p + 1];
  for (; e + 4 <= e1; e += 4) {
    uint2 r0 = in_rec[e], r1 = in_rec[e + 1], r2 = in_rec[e + 2], r3 = in_rec[e + 3];
    uint32_t a0 = dist[(size_t)r0.x * PLAIN_K + lane];
    uint32_t a1 = dist[(size_t)r1.x * PLAIN_K + lane];
    uint32_t a2 = dist[(size_t)r2.x * PLAIN_K + lane];
    uint32_t a3 = dist[(size_t)r3.x * PLAIN_K + lane];
    best = min(best, min(min(sat_add(a0, r0.y), sat_add(a1, r1.y)),
                         min(sat_add(a2, r2.y), sat_add(a3, r3.y))));
  }
  for (; e < e1; ++e) {
    uint2 r = in_rec[e];
    best = min(best, sat_add(dist[(size_t)r.x * PLAIN_K + lane], r.y));
  }
  if (best > threshold) best = INF;
  dist[(size_t)p * PLAIN_K + lane] = best;
}

// The node step of the plain sweep for slab position p (a warp, lane =
// source): the seed, then the min-plus pull over the DOWN in-edges. Rows of
// earlier levels are read through L2 (other blocks of a persistent launch
// wrote them).
__device__ __forceinline__ void plain_node(uint32_t p, uint32_t lane,
                                           const uint64_t* __restrict__ in_off,
                                           const uint2* __restrict__ in_rec,
                                           uint32_t* __restrict__ dist, uint32_t* __restrict__ seed,
                                           uint32_t* __restrict__ flag, uint32_t threshold) {
  uint32_t best = INF;
  const uint32_t bit = 1u << (p & 31);
  if (flag[p >> 5] & bit) {
    best = seed[(size_t)p * PLAIN_K + lane];
    seed[(size_t)p * PLAIN_K + lane] = INF;
    __syncwarp();
    if (lane == 0) atomicAnd(&flag[p >> 5], ~bit);
  }
  uint64_t e = in_off[p];
  const uint64_t e1 = in_off[p + 1];
  for (; e + 4 <= e1; e += 4) {
    const uint2 r0 = in_rec[e], r1 = in_rec[e + 1], r2 = in_rec[e + 2], r3 = in_rec[e + 3];
    const uint32_t a0 = __ldcg(&dist[(size_t)r0.x * PLAIN_K + lane]);
    const uint32_t a1 = __ldcg(&dist[(size_t)r1.x * PLAIN_K + lane]);
    const uint32_t a2 = __ldcg(&dist[(size_t)r2.x * PLAIN_K + lane]);
    const uint32_t a3 = __ldcg(&dist[(size_t)r3.x * PLAIN_K + lane]);
    best = min(best, min(min(sat_add(a0, r0.y), sat_add(a1, r1.y)),
                         min(sat_add(a2, r2.y), sat_add(a3, r3.y))));
  }
  for (; e < e1; ++e) {
    const uint2 r = in_rec[e];
    best = min(best, sat_add(__ldcg(&dist[(size_t)r.x * PLAIN_K + lane]), r.y));
  }
  if (best > threshold) best = INF;
  dist[(size_t)p * PLAIN_K + lane] = best;
}

// The whole plain sweep of one K = 32 batch in one cooperative launch over
// the full-graph schedule (rows = slab positions; nodes of high in-degree are
// split into work items of at most 16 in-edges, combined with atomicMin). A
// warp owns an item, lane = source. Phase 0 sets the rows that are read
// before they are fully written (no in-edges, or split) to their seed or INF;
// then the blocks walk the level program (a level spread over every warp of
// the grid, or a run of small levels swept by block 0 alone) with a grid
// barrier between segments. Values above the threshold become INF in every
// item (a split row's minimum is then still the clamped minimum). `withhold`
// (a test hook, NONE otherwise) names a block that leaves before its first
// barrier arrival.
__global__ void __launch_bounds__(512)
    k_plain_persist(const uint2* __restrict__ prog, uint32_t P, const uint32_t* __restrict__ lvl,
                    const uint4* __restrict__ item, const uint2* __restrict__ erec,
                    const uint32_t* __restrict__ reset_bits, uint32_t words,
                    uint32_t* __restrict__ dist, uint32_t* __restrict__ seed,
                    uint32_t* __restrict__ flag, uint32_t threshold, uint32_t* __restrict__ bar,
                    long long timeout, uint32_t withhold, uint32_t* __restrict__ err) {
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const uint32_t gw = blockIdx.x * wpb + wib, tw = gridDim.x * wpb;
  for (uint32_t w = gw; w < words; w += tw) {
    const uint32_t m = reset_bits[w];
    if (!m) continue;
    const uint32_t f = flag[w];
    for (uint32_t mm = m; mm;) {
      const uint32_t b = __ffs(mm) - 1;
      mm &= mm - 1;
      const size_t at = (size_t)(w * 32 + b) * PLAIN_K + lane;
      uint32_t v = INF;
      if ((f >> b) & 1u) {
        v = seed[at];
        seed[at] = INF;
      }
      dist[at] = v > threshold ? INF : v;
    }
    __syncwarp();
    if (lane == 0 && (f & m)) atomicAnd(&flag[w], ~(f & m));
  }
  if (blockIdx.x == withhold) return;
  if (!grid_barrier(bar, 0, timeout, err)) return;
  for (uint32_t s = 0; s < P; ++s) {
    const uint2 sg = prog[s];
    const bool run = (sg.y & PROG_RUN) != 0;
    const uint32_t l0 = sg.x, l1 = run ? (blockIdx.x == 0 ? sg.y & ~PROG_RUN : l0) : l0 + 1;
    const uint32_t first = run ? wib : gw, stride = run ? wpb : tw;
    for (uint32_t l = l0; l < l1; ++l) {
      const uint32_t i1 = lvl[l + 1];
      for (uint32_t ii = lvl[l] + first; ii < i1; ii += stride) {
        const uint4 it = item[ii];
        uint32_t acc = INF;
        uint32_t e = it.y;
        for (; e + 4 <= it.z; e += 4) {
          const uint2 r0 = erec[e], r1 = erec[e + 1], r2 = erec[e + 2], r3 = erec[e + 3];
          const uint32_t a0 = __ldcg(&dist[(size_t)r0.x * PLAIN_K + lane]);
          const uint32_t a1 = __ldcg(&dist[(size_t)r1.x * PLAIN_K + lane]);
          const uint32_t a2 = __ldcg(&dist[(size_t)r2.x * PLAIN_K + lane]);
          const uint32_t a3 = __ldcg(&dist[(size_t)r3.x * PLAIN_K + lane]);
          acc = min(acc, min(min(sat_add(a0, r0.y), sat_add(a1, r1.y)),
                             min(sat_add(a2, r2.y), sat_add(a3, r3.y))));
        }
        for (; e < it.z; ++e) {
          const uint2 r = erec[e];
          acc = min(acc, sat_add(__ldcg(&dist[(size_t)r.x * PLAIN_K + lane]), r.y));
        }
        const size_t at = (size_t)it.x * PLAIN_K + lane;
        if (it.w) {  // a slice of a split row, initialised in phase 0
          if (acc <= threshold) atomicMin(&dist[at], acc);
        } else {
          const uint32_t bit = 1u << (it.x & 31);
          uint32_t best = acc;
          if (flag[it.x >> 5] & bit) {
            best = min(best, seed[at]);
            seed[at] = INF;
            __syncwarp();
            if (lane == 0) atomicAnd(&flag[it.x >> 5], ~bit);
          }
          dist[at] = best > threshold ? INF : best;
        }
      }
      if (run) __syncthreads();
    }
    if (s + 1 == P) break;
    if (!grid_barrier(bar, s + 1, timeout, err)) return;
  }
}

// out[(row0 + l) * T + t] = slab[tpos[t]][l] for l < k; tiles of 32 targets.
__global__ void __launch_bounds__(256)
    k_extract(const uint32_t* __restrict__ slab, uint32_t slab_stride,
              const uint32_t* __restrict__ tpos, uint64_t T, uint32_t k,
              uint32_t* __restrict__ out) {
  __shared__ uint32_t tile[32][33];
  const uint64_t t0 = (uint64_t)blockIdx.x * 32;
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    uint64_t t = t0 + r;
    tile[r][threadIdx.x] = (t < T) ? slab[(size_t)tpos[t] * slab_stride + threadIdx.x] : INF;
  }
  __syncthreads();
  for (uint32_t l = threadIdx.y; l < k; l += 8) {
    uint64_t t = t0 + threadIdx.x;
    if (t < T) out[(uint64_t)l * T + t] = tile[threadIdx.x][l];
  }
}

__global__ void k_to_positions(const uint32_t* __restrict__ ranks, uint64_t m,
                               const uint32_t* __restrict__ pos_of, uint32_t n,
                               uint32_t* __restrict__ pos, uint32_t* __restrict__ err) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  uint32_t r = ranks[i];
  if (r >= n) {
    atomicOr(err, DEVERR_PATH);
    pos[i] = 0;
  } else {
    pos[i] = pos_of[r];
  }
}

bf_status to_positions(Graph* g, const uint32_t* d_rank, uint64_t m, uint32_t* d_pos,
                       cudaStream_t st) {
  if (!m) return BF_OK;
  k_to_positions<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(d_rank, m, g->d_pos_of, g->n, d_pos,
                                                              g->d_err);
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

bf_status check_device_error(Graph* g, cudaStream_t st) {
  uint32_t h = 0;
  BF_CUDA(cudaMemcpyAsync(&h, g->d_err, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  if (h) {
    BF_CUDA(cudaMemsetAsync(g->d_err, 0, 4, st));
    BF_CUDA(cudaStreamSynchronize(st));
    if (h & DEVERR_TIMEOUT) {
      // a sweep that gave up may have left seeds in the plain engine's
      // buffers, which must be all INF / clear between calls
      if (g->d_seed) {
        BF_CUDA(cudaMemsetAsync(g->d_seed, 0xFF, (size_t)g->n * PLAIN_K * 4, st));
        BF_CUDA(cudaMemsetAsync(g->d_flag, 0, ((g->n + 31) / 32) * 4, st));
        BF_CUDA(cudaStreamSynchronize(st));
      }
      set_error("a bounded device wait ran out (error bits 0x" + std::to_string(h) + ")");
      return BF_ERR_TIMEOUT;
    }
    set_error("device reported error bits 0x" + std::to_string(h) +
              " (invalid node id or CCH inconsistent with its elimination tree)");
    return BF_ERR_INVALID;
  }
  return BF_OK;
}

bool test_withhold_arrival() { return std::getenv("BF_TEST_WITHHOLD_ARRIVAL") != nullptr; }

static bf_status plain_buffers(Graph* g) {
  if (g->d_dist) return BF_OK;
  const size_t slab = (size_t)g->n * PLAIN_K * sizeof(uint32_t);
  if (cudaMalloc(&g->d_dist, slab) != cudaSuccess || cudaMalloc(&g->d_seed, slab) != cudaSuccess ||
      cudaMalloc(&g->d_flag, ((g->n + 31) / 32) * 4) != cudaSuccess) {
    cudaGetLastError();
    set_error("cannot allocate the plain engine's distance slabs");
    return BF_ERR_OOM;
  }
  g->device_bytes += 2 * slab + ((g->n + 31) / 32) * 4;
  BF_CUDA(cudaMemset(g->d_seed, 0xFF, slab));
  BF_CUDA(cudaMemset(g->d_flag, 0, ((g->n + 31) / 32) * 4));
  return BF_OK;
}

bf_status launch_scatter_seeds(Graph* g, const void* cseed, uint64_t k, const uint32_t* d_src,
                               uint32_t* slab, uint32_t Kp, cudaStream_t st, uint64_t stride,
                               uint64_t col0, const uint32_t* cidx) {
  if (!k) return BF_OK;
  dim3 grid((unsigned)((k + 255) / 256), g->max_depth + 1);
  k_scatter_seeds<<<grid, 256, 0, st>>>(reinterpret_cast<const uint2*>(cseed), (uint32_t)k, d_src,
                                       g->d_depth, slab, Kp, (uint32_t)(stride ? stride : k),
                                       (uint32_t)col0, cidx);
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

// Upward pass for k sources: source i writes lane i of row pos_map[x] of
// `seed` (stride lanes per row) for every settled ancestor x; rows mapped to
// NONE are skipped. `flag` (optional) receives the seeded-row bits.
bf_status launch_upward(Graph* g, const uint32_t* d_src, uint64_t k, uint32_t threshold,
                        const uint32_t* pos_map, uint32_t* seed, uint32_t stride, uint32_t* flag,
                        cudaStream_t st, const uint32_t* lane_thr, const uint32_t* unit_cost,
                        const uint32_t* unit_lane, uint32_t mode) {
  if (mode == UPWARD_OUT_SLAB16 && (!lane_thr || unit_lane)) {
    set_error("16-bit seed lanes need per-lane thresholds below 0xFFFF");
    return BF_ERR_UNSUPPORTED;
  }
  const uint32_t dcap = ((g->max_depth + 1) + 31) & ~31u;
  const size_t runs_smem = (size_t)UPWARD_WARPS * dcap * 4;
  if (g->max_runs <= 32 && runs_smem <= 100 * 1024) {
    BF_CUDA(cudaFuncSetAttribute(k_upward_runs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)runs_smem));
    k_upward_runs<<<(unsigned)((k + UPWARD_WARPS - 1) / UPWARD_WARPS), UPWARD_WARPS * 32,
                    runs_smem, st>>>(d_src, (uint32_t)k, threshold, g->d_parent, g->d_run_end,
                                     g->d_depth, g->d_up_off, g->d_up_rec, pos_map, g->n, seed,
                                     stride, flag, dcap, g->d_err, lane_thr, unit_cost,
                                     unit_lane, mode);
    BF_CUDA(cudaGetLastError());
    return BF_OK;
  }
  const size_t fast_smem = (size_t)UPWARD_WARPS * 2 * dcap * 4;
  if (fast_smem <= 200 * 1024) {
    BF_CUDA(cudaFuncSetAttribute(k_upward_fast<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)fast_smem));
    k_upward_fast<false><<<(unsigned)((k + UPWARD_WARPS - 1) / UPWARD_WARPS), UPWARD_WARPS * 32,
                           fast_smem, st>>>(d_src, (uint32_t)k, threshold, g->d_parent,
                                            g->d_run_end, g->d_depth, g->d_up_off, g->d_up_rec,
                                            pos_map, g->n, seed, stride, flag, dcap, g->d_err,
                                            lane_thr, unit_cost, unit_lane, mode, 0u, nullptr);
    BF_CUDA(cudaGetLastError());
    return BF_OK;
  }
  // deep trees: ancestor paths in a per-call global scratch, a bounded
  // number of warps per launch
  const size_t per = (size_t)dcap * 2 * 4;
  uint64_t chunk = std::max<uint64_t>(UPWARD_WARPS, ((256ull << 20) / per) & ~(uint64_t)(UPWARD_WARPS - 1));
  chunk = std::min<uint64_t>(chunk, (k + UPWARD_WARPS - 1) & ~(uint64_t)(UPWARD_WARPS - 1));
  void* scratch = nullptr;
  if (cudaMalloc(&scratch, chunk * per) != cudaSuccess) {
    cudaGetLastError();
    set_error("cannot allocate the ancestor-path scratch");
    return BF_ERR_OOM;
  }
  cudaError_t le = cudaSuccess;
  for (uint64_t w0 = 0; w0 < k && le == cudaSuccess; w0 += chunk) {
    const uint64_t m = std::min<uint64_t>(chunk, k - w0);
    k_upward_fast<true><<<(unsigned)((m + UPWARD_WARPS - 1) / UPWARD_WARPS), UPWARD_WARPS * 32, 0,
                          st>>>(d_src, (uint32_t)k, threshold, g->d_parent, g->d_run_end,
                                g->d_depth, g->d_up_off, g->d_up_rec, pos_map, g->n, seed, stride,
                                flag, dcap, g->d_err, lane_thr, unit_cost, unit_lane, mode,
                                (uint32_t)w0, static_cast<uint32_t*>(scratch));
    le = cudaGetLastError();
  }
  // the scratch is freed once the launches that use it have finished
  const cudaError_t se = cudaStreamSynchronize(st);
  cudaFree(scratch);
  if (le != cudaSuccess) return cuda_status(le, "deep-tree upward launch");
  if (se != cudaSuccess) return cuda_status(se, "cudaStreamSynchronize");
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

static bf_status plain_upward(Graph* g, const uint32_t* d_src, uint32_t k, uint32_t threshold,
                              cudaStream_t st) {
  return launch_upward(g, d_src, k, threshold, g->d_pos_of, g->d_seed, PLAIN_K, g->d_flag, st);
}

// Blocks of a persistent launch: as many as are co-resident (the cooperative
// launch guarantees they run together), at most `cap`; two under the test hook.
unsigned persistent_blocks(Graph* g, const void* kern, unsigned tpb, unsigned cap) {
  if (test_withhold_arrival()) return 2;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)tpb, 0) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  return std::max(1u, std::min(cap, (unsigned)std::max(per_sm, 1) * g->sm_count));
}

bf_status ensure_barrier(Graph* g) {
  if (g->d_bar) return BF_OK;
  BF_CUDA(cudaMalloc(&g->d_bar, 64));
  g->device_bytes += 64;
  return BF_OK;
}

static bf_status plain_sweep_persistent(Graph* g, uint32_t threshold, cudaStream_t st,
                                        uint64_t* launches) {
  constexpr unsigned TPB = 512;
  bf_status s;
  if ((s = ensure_barrier(g))) return s;
  Ctx& c = g->ctx;
  if ((s = build_schedule(g, c, c.full, nullptr, 0, true, st))) return s;
  Sched& sc = c.full;
  if (g->plain_prog.empty() || g->plain_prog_levels != sc.lvl_item.size()) {
    // runs: levels of at most two rounds of one block's warps
    g->plain_prog = level_program(sc.lvl_item, g->n_levels, 2 * (TPB / 32));
    if (g->d_plain_prog) {
      cudaFree(g->d_plain_prog);
      g->device_bytes -= g->plain_prog_bytes;
      g->d_plain_prog = nullptr;
    }
    g->plain_prog_bytes = std::max<size_t>(g->plain_prog.size(), 1) * sizeof(uint2);
    BF_CUDA(cudaMalloc(&g->d_plain_prog, g->plain_prog_bytes));
    g->device_bytes += g->plain_prog_bytes;
    BF_CUDA(cudaMemcpyAsync(g->d_plain_prog, g->plain_prog.data(),
                            g->plain_prog.size() * sizeof(uint2), cudaMemcpyHostToDevice, st));
    g->plain_prog_levels = sc.lvl_item.size();
  }
  const bool hook = test_withhold_arrival();
  const unsigned blocks = persistent_blocks(g, (const void*)k_plain_persist, TPB, 4 * g->sm_count);
  BF_CUDA(cudaMemsetAsync(g->d_bar, 0, 8, st));
  BF_CUDA(launch_persistent(k_plain_persist, blocks, TPB, st, (const uint2*)g->d_plain_prog,
                            (uint32_t)g->plain_prog.size(), (const uint32_t*)sc.d_lvl,
                            (const uint4*)sc.d_item, (const uint2*)sc.d_erec,
                            (const uint32_t*)sc.d_split, (uint32_t)((g->n + 31) / 32), g->d_dist,
                            g->d_seed, g->d_flag, threshold, g->d_bar,
                            hook ? 2000000ll : BARRIER_TIMEOUT_CYCLES, hook ? 1u : NONE,
                            g->d_err));
  ++*launches;
  return BF_OK;
}

static bf_status plain_sweep(Graph* g, uint32_t threshold, cudaStream_t st, uint64_t* launches) {
  if (g->tune.persist & 1u) return plain_sweep_persistent(g, threshold, st, launches);
  for (uint32_t l = 0; l < g->n_levels; ++l) {
    uint32_t p0 = g->lvl_start[l], p1 = g->lvl_start[l + 1];
    if (p1 == p0) continue;
    unsigned blocks = (unsigned)(((uint64_t)(p1 - p0) * 32 + 255) / 256);
    k_sweep_level<<<blocks, 256, 0, st>>>(p0, p1, g->d_in_off, g->d_in_rec, g->d_dist, g->d_seed,
                                          g->d_flag, threshold);
    ++*launches;
  }
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

bf_status plain_matrix(Graph* g, const uint32_t* d_src, uint64_t S, const uint32_t* d_tpos,
                       uint64_t T, uint32_t threshold, uint32_t* d_out, cudaStream_t st,
                       bf_stats* stats) {
  bf_status s;
  if ((s = plain_buffers(g))) return s;
  const uint64_t nb = (S + PLAIN_K - 1) / PLAIN_K;
  uint64_t launches = 0;
  float t_up = 0, t_dn = 0, t_ex = 0;
  for (uint64_t b = 0; b < nb; ++b) {
    const uint64_t s0 = b * PLAIN_K;
    const uint32_t k = (uint32_t)std::min<uint64_t>(PLAIN_K, S - s0);
    if (stats) BF_CUDA(cudaEventRecord(g->ev[0], st));
    if ((s = plain_upward(g, d_src + s0, k, threshold, st))) return s;
    ++launches;
    if (stats) BF_CUDA(cudaEventRecord(g->ev[1], st));
    if ((s = plain_sweep(g, threshold, st, &launches))) return s;
    if (stats) BF_CUDA(cudaEventRecord(g->ev[2], st));
    if (T) {
      dim3 blk(32, 8);
      k_extract<<<(unsigned)((T + 31) / 32), blk, 0, st>>>(g->d_dist, PLAIN_K, d_tpos, T, k,
                                                          d_out + s0 * T);
      BF_CUDA(cudaGetLastError());
      ++launches;
    }
    if (stats) {
      BF_CUDA(cudaEventRecord(g->ev[3], st));
      BF_CUDA(cudaEventSynchronize(g->ev[3]));
      float a, c, d;
      BF_CUDA(cudaEventElapsedTime(&a, g->ev[0], g->ev[1]));
      BF_CUDA(cudaEventElapsedTime(&c, g->ev[1], g->ev[2]));
      BF_CUDA(cudaEventElapsedTime(&d, g->ev[2], g->ev[3]));
      t_up += a;
      t_dn += c;
      t_ex += d;
    }
  }
  if (stats) {
    stats->n_batches += nb;
    stats->waves += nb;
    stats->swept_nodes = g->n;
    stats->swept_edges = g->n_down;
    stats->lanes = PLAIN_K;
    stats->kernel_launches += launches;
    stats->upward_ms += t_up;
    stats->downward_ms += t_dn;
    stats->extract_ms += t_ex;
  }
  return BF_OK;
}

}  // namespace bf
