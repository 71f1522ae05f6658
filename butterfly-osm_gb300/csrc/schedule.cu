// schedule.cu — target-restricted sweep schedules built on the device.
//
// A restricted schedule (RPHAST: only the rows that reach a requested target
// along DOWN edges, route/src/range/tree_phast.rs:320-417 selects the same
// set) used to be built by host threads: ~35 ms for 10 000 targets on the
// country graph, more than the sweep itself. Here every step runs on the GPU:
//
//   1. ancestors   every DOWN edge u -> v joins v to one of its elimination-
//                  tree ancestors, so the rows reaching a target all lie on
//                  the targets' ancestor paths. One warp per target marks its
//                  path (whole runs of consecutive ranks at once) and stops
//                  where another warp has been: the candidate set C.
//   2. peeling     a row of C that is no target and none of whose DOWN
//                  out-edges lead to a live row of C reaches no target. Each
//                  row counts its out-edges into C (one atomic per in-edge of
//                  a C row); rows with count 0 start a frontier, and every
//                  dead row decrements its in-edge sources, which die at 0.
//                  All rounds run in one cooperative launch, separated by a
//                  grid barrier, until the frontier is empty (38 rounds for
//                  10 000 targets on the country graph); a row still alive
//                  when the round limit ends it would only be swept in vain.
//                  A row's in-edges are spread over a warp's lanes, 32 edges
//                  a step (counting, peeling and the fill alike), so rows
//                  with thousands of in-edges do not hold one thread.
//   3. compaction  rows are the live positions in slab-position order, so
//                  they come grouped by level; row(p) = popcount prefix of
//                  the live bitmap. A scan gives each row its edge and work-
//                  item offsets, a per-(level, item size) histogram orders
//                  each level's items heaviest first.
//   4. fill        edge records {source row, w}, work items, target rows, the
//                  rank -> row map (every rank rewritten) and per-row gather
//                  counts for the L2 hub choice.
//
// The host reads back only the counts and the level -> first item table
// (it launches one kernel per level). Results are those of the host-built
// schedule: the same rows and edges, items of one level in another order.

#include <algorithm>
#include <cstring>

#include "engine.cuh"
#include "scan.cuh"

namespace bf {

namespace {

// Peeling rounds at most (10 000 targets on the country graph take 38).
constexpr uint32_t PEEL_ROUNDS = 4096;
// meta words: three rotating frontier sizes, the row count, the candidate
// count, peeling rounds run and frontier left, the grid-barrier words
constexpr uint32_t META_NR = 3, META_NC = 4, META_ROUNDS = 5, META_LEFT = 6, META_BAR = 8,
                   META_WORDS = 16;
constexpr uint32_t HUB_BINS = 65536;

// Grow a device array to `need` elements (1/8 more with `slack`: arrays
// sized by a schedule's rows, items or edges, which vary a little between
// target sets, so most new sets reuse them instead of reallocating).
template <class T>
bf_status ensure_dev(T** p, size_t& cap, size_t need, Graph* g, bool slack = false) {
  if (need <= cap && *p) return BF_OK;
  if (*p) {
    cudaFree(*p);
    g->device_bytes -= cap * sizeof(T);
  }
  *p = nullptr;
  cap = 0;
  const size_t m = std::max<size_t>(slack ? need + need / 8 : need, 1);
  if (cudaMalloc((void**)p, m * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_error("cudaMalloc for the device schedule builder failed");
    return BF_ERR_OOM;
  }
  cap = m;
  g->device_bytes += m * sizeof(T);
  return BF_OK;
}

__device__ __forceinline__ uint32_t bit_of(const uint32_t* bm, uint32_t p) {
  return (bm[p >> 5] >> (p & 31)) & 1u;
}

// Row index of slab position p: live positions below p.
__device__ __forceinline__ uint32_t row_of(const uint32_t* __restrict__ alive,
                                           const uint32_t* __restrict__ wpre, uint32_t p) {
  return wpre[p >> 5] + __popc(alive[p >> 5] & ((1u << (p & 31)) - 1u));
}

// 1. Mark the ancestor paths of the targets (positions) and the targets.
// Every newly marked position is appended to the candidate list `clist`
// (count in *nc), which the counting and the first frontier walk.
__global__ void __launch_bounds__(128)
    k_sd_mark(const uint32_t* __restrict__ tgt, uint32_t T, const uint32_t* __restrict__ parent,
              const uint32_t* __restrict__ run_end, const uint32_t* __restrict__ pos_of, uint32_t n,
              uint32_t* __restrict__ alive, uint32_t* __restrict__ ist, uint32_t* __restrict__ cnt,
              uint32_t* __restrict__ clist, uint32_t* __restrict__ nc,
              uint32_t* __restrict__ err) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= T) return;
  uint32_t x = tgt[w];
  if (x >= n) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  if (lane == 0) {
    const uint32_t p = pos_of[x];
    atomicOr(&ist[p >> 5], 1u << (p & 31));
  }
  for (uint32_t guard = 0; x != NONE && guard < n; ++guard) {
    // a run whose first node is marked is marked up to the root by the warp
    // that marked it (it marks whole runs and then continues at the parent)
    const uint32_t p0 = pos_of[x];
    if ((*(volatile const uint32_t*)&alive[p0 >> 5] >> (p0 & 31)) & 1u) break;
    const uint32_t e = run_end[x];
    if (e < x || e >= n) {
      if (lane == 0) atomicOr(err, DEVERR_PATH);
      return;
    }
    for (uint32_t r0 = x; r0 <= e; r0 += 32) {
      const uint32_t r = r0 + lane;
      uint32_t p = 0;
      bool fresh = false;
      if (r <= e) {
        p = pos_of[r];
        const uint32_t b = 1u << (p & 31);
        fresh = !(atomicOr(&alive[p >> 5], b) & b);
        if (fresh) cnt[p] = 0;
      }
      const uint32_t f = __ballot_sync(0xFFFFFFFFu, fresh);
      uint32_t base = 0;
      if (lane == 0 && f) base = atomicAdd(nc, (uint32_t)__popc(f));
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (fresh) clist[base + __popc(f & ((1u << lane) - 1u))] = p;
    }
    __syncwarp();
    x = parent[e];
  }
}

// Edges of 32 rows, one row per lane (k0: first in-edge, deg: in-degree, 0
// for no row), spread over the warp's lanes, 32 edges per step whatever the
// degrees, so a row with thousands of in-edges does not hold one thread for
// thousands of steps. Every lane calls f(on, k, owner lane) once per step
// (f may use warp collectives); `on` is false past the last edge.
template <class F>
__device__ __forceinline__ void warp_edges(uint64_t k0, uint32_t deg, uint32_t lane, F& f) {
  constexpr unsigned FULL = 0xFFFFFFFFu;
  uint32_t inc = deg;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, inc, o);
    if (lane >= o) inc += t;
  }
  const uint32_t total = __shfl_sync(FULL, inc, 31), exc = inc - deg;
  for (uint32_t e0 = 0; e0 < total; e0 += 32) {
    const uint32_t e = e0 + lane;
    // owner: the last lane whose first edge is at or below e
    uint32_t lo = 0;
#pragma unroll
    for (uint32_t b = 16; b; b >>= 1) {
      const uint32_t ex = __shfl_sync(FULL, exc, lo + b);
      if (ex <= e) lo += b;
    }
    const uint64_t kb = __shfl_sync(FULL, k0, lo);
    const uint32_t xo = __shfl_sync(FULL, exc, lo);
    f(e < total, kb + (e - xo), lo);
  }
}

// 2a. cnt[u] = DOWN out-edges of u into C (every in-edge source of a C row is
// an ancestor of it, hence in C): one atomic per in-edge of a candidate.
struct CountEdge {
  const uint2* in_rec;
  uint32_t* cnt;
  __device__ __forceinline__ void operator()(bool on, uint64_t k, uint32_t) {
    if (on) atomicAdd(&cnt[in_rec[k].x], 1u);
  }
};

__global__ void __launch_bounds__(256)
    k_sd_count(const uint32_t* __restrict__ clist, const uint32_t* __restrict__ nc_p,
               const uint64_t* __restrict__ in_off, const uint2* __restrict__ in_rec,
               uint32_t* __restrict__ cnt) {
  const uint32_t nc = *nc_p, lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * blockDim.x / 32;
  CountEdge f{in_rec, cnt};
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < nc;
       base += warps * 32) {
    uint64_t k0 = 0;
    uint32_t deg = 0;
    if (base + lane < nc) {
      const uint32_t p = clist[base + lane];
      k0 = in_off[p];
      deg = (uint32_t)(in_off[p + 1] - k0);
    }
    warp_edges(k0, deg, lane, f);
  }
}

// 2b. First frontier: candidates that are no target and have no out-edge
// into C.
__global__ void __launch_bounds__(256)
    k_sd_front0(const uint32_t* __restrict__ clist, const uint32_t* __restrict__ nc_p,
                uint32_t* __restrict__ alive, const uint32_t* __restrict__ ist,
                const uint32_t* __restrict__ cnt, uint32_t* __restrict__ front,
                uint32_t* __restrict__ fcount) {
  const uint32_t nc = *nc_p, lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * blockDim.x / 32;
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < nc;
       base += warps * 32) {
    uint32_t p = 0;
    bool dead = false;
    if (base + lane < nc) {
      p = clist[base + lane];
      dead = !bit_of(ist, p) && cnt[p] == 0;
      if (dead) atomicAnd(&alive[p >> 5], ~(1u << (p & 31)));
    }
    const uint32_t d = __ballot_sync(0xFFFFFFFFu, dead);
    uint32_t slot = 0;
    if (lane == 0 && d) slot = atomicAdd(fcount, (uint32_t)__popc(d));
    slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
    if (dead) front[slot + __popc(d & ((1u << lane) - 1u))] = p;
  }
}

// 2c. Peeling rounds, one cooperative launch: in round r every dead row of
// frontier r releases its in-edge sources; a source whose count reaches 0
// (and is no target) dies and joins frontier r + 1. Frontiers alternate
// between the two halves of `front`; their sizes rotate through meta[0..2]
// (round r reads meta[r % 3], counts into meta[(r + 1) % 3], and block 0
// clears meta[(r + 2) % 3], which no block touches in round r). Rounds are
// separated by the bounded grid barrier; all blocks leave together once a
// frontier is empty or after `rounds` rounds (meta[META_LEFT] then holds
// the frontier left, whose rows stay live: a superset is still closed under
// in-edge sources, so it is swept correctly, only in vain).
struct PeelEdge {
  const uint2* in_rec;
  uint32_t* cnt;
  uint32_t* alive;
  const uint32_t* ist;
  uint32_t* fout;
  uint32_t* nout;
  uint32_t lane;
  __device__ __forceinline__ void operator()(bool on, uint64_t k, uint32_t) {
    uint32_t u = 0;
    bool dead = false;
    if (on) {
      u = in_rec[k].x;
      dead = atomicSub(&cnt[u], 1u) == 1u && !bit_of(ist, u);
      if (dead) atomicAnd(&alive[u >> 5], ~(1u << (u & 31)));
    }
    const uint32_t d = __ballot_sync(0xFFFFFFFFu, dead);
    uint32_t slot = 0;
    if (lane == 0 && d) slot = atomicAdd(nout, (uint32_t)__popc(d));
    slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
    if (dead) fout[slot + __popc(d & ((1u << lane) - 1u))] = u;
  }
};

__global__ void __launch_bounds__(256)
    k_sd_peel(uint32_t* __restrict__ front, uint32_t n, uint32_t* __restrict__ meta,
              uint32_t rounds, const uint64_t* __restrict__ in_off,
              const uint2* __restrict__ in_rec, uint32_t* __restrict__ cnt,
              uint32_t* __restrict__ alive, const uint32_t* __restrict__ ist,
              long long timeout, uint32_t withhold, uint32_t* __restrict__ err) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * blockDim.x / 32;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t r = 0, m = 0;
  for (; r < rounds; ++r) {
    // frontier r was completed before the barrier: read it through L2
    m = __ldcg(&meta[r % 3]);
    if (m == 0) break;
    const uint32_t* fin = front + (size_t)(r & 1) * n;
    PeelEdge f{in_rec, cnt, alive, ist, front + (size_t)((r + 1) & 1) * n,
               meta + (r + 1) % 3, lane};
    if (blockIdx.x == 0 && threadIdx.x == 0) meta[(r + 2) % 3] = 0;
    for (uint32_t base = wid * 32; base < m; base += warps * 32) {
      uint64_t k0 = 0;
      uint32_t deg = 0;
      if (base + lane < m) {
        const uint32_t v = __ldcg(&fin[base + lane]);
        k0 = in_off[v];
        deg = (uint32_t)(in_off[v + 1] - k0);
      }
      warp_edges(k0, deg, lane, f);
    }
    // (test hook: block `withhold` leaves before its first arrival)
    if (blockIdx.x == withhold || !grid_barrier(meta + META_BAR, r, timeout, err)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    meta[META_ROUNDS] = r;
    meta[META_LEFT] = r < rounds ? 0u : __ldcg(&meta[r % 3]);
  }
}

// 3a. Row positions, first row of each level, and the live-row count.
__global__ void __launch_bounds__(256)
    k_sd_rows(const uint32_t* __restrict__ alive, const uint32_t* __restrict__ wpre, uint32_t W,
              uint32_t* __restrict__ rowpos) {
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < W; w += gridDim.x * blockDim.x) {
    uint32_t m = alive[w], r = wpre[w];
    while (m) {
      rowpos[r++] = w * 32 + (__ffs(m) - 1);
      m &= m - 1;
    }
  }
}

__global__ void k_sd_lvlrow(const uint32_t* __restrict__ lvl_start, uint32_t L,
                            const uint32_t* __restrict__ alive, const uint32_t* __restrict__ wpre,
                            uint32_t* __restrict__ lvlrow, uint32_t* __restrict__ meta_nr,
                            uint32_t W) {
  const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l <= L) lvlrow[l] = row_of(alive, wpre, lvl_start[l]);
  if (l == 0) *meta_nr = wpre[W];
}

__device__ __forceinline__ uint32_t level_of_row(const uint32_t* __restrict__ lvlrow, uint32_t L,
                                                 uint32_t i) {
  uint32_t lo = 0, hi = L;  // largest l with lvlrow[l] <= i (lvlrow[0] = 0)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (lvlrow[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

struct SplitCfg {
  uint32_t split, small_split, small_rows, s1;
};

__device__ __forceinline__ uint32_t split_of_level(const uint32_t* __restrict__ lvlrow, uint32_t l,
                                                   const SplitCfg& c) {
  return lvlrow[l + 1] - lvlrow[l] < c.small_rows ? c.small_split : c.split;
}

// 3b. Per row: in-degree and work items (edges | items << 32), items per
// (level, size), and the rows reset every wave (no in-edges, or split).
__global__ void __launch_bounds__(256)
    k_sd_deg(const uint32_t* __restrict__ rowpos, const uint32_t* __restrict__ n_r_p,
             const uint64_t* __restrict__ in_off, const uint32_t* __restrict__ lvlrow, uint32_t L,
             SplitCfg c, uint64_t* __restrict__ rdeg, uint32_t* __restrict__ hist,
             uint32_t* __restrict__ split_bits) {
  const uint32_t n_r = *n_r_p;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * blockDim.x / 32;
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < n_r;
       base += warps * 32) {
    const uint32_t i = base + lane;
    bool flag = false;
    if (i < n_r) {
      const uint32_t p = rowpos[i];
      const uint32_t deg = (uint32_t)(in_off[p + 1] - in_off[p]);
      const uint32_t l = level_of_row(lvlrow, L, i);
      const uint32_t sp = split_of_level(lvlrow, l, c);
      const uint32_t items = (deg + sp - 1) / sp;
      rdeg[i] = (uint64_t)deg | ((uint64_t)items << 32);
      flag = deg == 0 || deg > sp;
      if (deg >= sp) atomicAdd(&hist[(size_t)l * c.s1 + sp], deg / sp);
      if (deg % sp) atomicAdd(&hist[(size_t)l * c.s1 + deg % sp], 1u);
    }
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, flag);
    if (lane == 0) split_bits[base >> 5] = m;
  }
}

// 3c. Item cursors: level l's items start at lvl_item[l], sizes descending.
__global__ void __launch_bounds__(SCAN_TPB)
    k_sd_cursor(uint32_t* __restrict__ hist, uint32_t L, uint32_t s1,
                uint32_t* __restrict__ lvl_item) {
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t l0 = 0; l0 < L; l0 += SCAN_TPB) {
    const uint32_t l = l0 + threadIdx.x;
    uint32_t tot = 0;
    if (l < L)
      for (uint32_t s = 1; s < s1; ++s) tot += hist[(size_t)l * s1 + s];
    uint32_t all;
    const uint32_t ex = block_exscan<uint32_t>(tot, &all);
    const uint32_t c0 = carry;
    if (l < L) {
      uint32_t cur = c0 + ex;
      lvl_item[l] = cur;
      for (uint32_t s = s1; s-- > 1;) {
        const uint32_t k = hist[(size_t)l * s1 + s];
        hist[(size_t)l * s1 + s] = cur;
        cur += k;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) carry = c0 + all;
    __syncthreads();
  }
  if (threadIdx.x == 0) lvl_item[L] = carry;
}

// Per level: first row and first edge record (for the per-level table).
__global__ void k_sd_lvledge(const uint32_t* __restrict__ lvlrow, const uint64_t* __restrict__ rpre,
                             uint32_t L, uint32_t* __restrict__ lvl_edge) {
  const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l <= L) lvl_edge[l] = (uint32_t)rpre[lvlrow[l]];
}

// 4a. Edge records, work items and gather counts: 32 rows per warp step,
// their edges spread over the lanes; each lane then cuts its own row into
// work items (one cursor atomic for all full-size items of the row).
struct FillEdge {
  const uint2* in_rec;
  const uint32_t* in_len;
  const uint32_t* alive;
  const uint32_t* wpre;
  uint2* erec;
  uint32_t* elen;
  uint32_t* uses;
  uint64_t kbase;  // this lane's row: first in-edge and first edge record
  uint32_t ebase;
  __device__ __forceinline__ void operator()(bool on, uint64_t k, uint32_t owner) {
    const uint64_t kb = __shfl_sync(0xFFFFFFFFu, kbase, owner);
    const uint32_t eb = __shfl_sync(0xFFFFFFFFu, ebase, owner);
    if (!on) return;
    const uint2 r = in_rec[k];
    const uint32_t src = row_of(alive, wpre, r.x);
    const uint32_t e = eb + (uint32_t)(k - kb);
    erec[e] = make_uint2(src, r.y);
    if (elen) elen[e] = in_len[k];
    atomicAdd(&uses[src], 1u);
  }
};

__global__ void __launch_bounds__(256)
    k_sd_fill(const uint32_t* __restrict__ rowpos, const uint32_t* __restrict__ n_r_p,
              const uint64_t* __restrict__ rpre, const uint64_t* __restrict__ in_off,
              const uint2* __restrict__ in_rec, const uint32_t* __restrict__ in_len,
              const uint32_t* __restrict__ alive, const uint32_t* __restrict__ wpre,
              const uint32_t* __restrict__ lvlrow, uint32_t L, SplitCfg c,
              uint32_t* __restrict__ cursor, uint4* __restrict__ item, uint2* __restrict__ erec,
              uint32_t* __restrict__ elen, uint32_t* __restrict__ uses) {
  const uint32_t n_r = *n_r_p, lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * blockDim.x / 32;
  FillEdge f{in_rec, in_len, alive, wpre, erec, elen, uses, 0, 0};
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < n_r;
       base += warps * 32) {
    const uint32_t i = base + lane;
    uint64_t k0 = 0;
    uint32_t deg = 0, e0 = 0;
    if (i < n_r) {
      const uint32_t p = rowpos[i];
      e0 = (uint32_t)rpre[i];  // edges never reach 2^32 (checked by the host)
      k0 = in_off[p];
      deg = (uint32_t)(in_off[p + 1] - k0);
    }
    f.kbase = k0;
    f.ebase = e0;
    warp_edges(k0, deg, lane, f);
    if (!deg) continue;
    const uint32_t l = level_of_row(lvlrow, L, i);
    const uint32_t sp = split_of_level(lvlrow, l, c);
    const uint32_t split = deg > sp ? 1u : 0u;
    const uint32_t full = deg / sp, rest = deg % sp;
    if (full) {
      const uint32_t slot = atomicAdd(&cursor[(size_t)l * c.s1 + sp], full);
      for (uint32_t q = 0; q < full; ++q)
        item[slot + q] = make_uint4(i, e0 + q * sp, e0 + (q + 1) * sp, split);
    }
    if (rest) {
      const uint32_t slot = atomicAdd(&cursor[(size_t)l * c.s1 + rest], 1u);
      item[slot] = make_uint4(i, e0 + full * sp, e0 + deg, split);
    }
  }
}

// 4b. Target rows and the full rank -> row map.
__global__ void k_sd_trow(const uint32_t* __restrict__ tgt, uint64_t T,
                          const uint32_t* __restrict__ pos_of, const uint32_t* __restrict__ alive,
                          const uint32_t* __restrict__ wpre, uint32_t* __restrict__ trow) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < T) trow[i] = row_of(alive, wpre, pos_of[tgt[i]]);
}

__global__ void __launch_bounds__(256)
    k_sd_cidx(const uint32_t* __restrict__ pos_of, uint32_t n, const uint32_t* __restrict__ alive,
              const uint32_t* __restrict__ wpre, uint32_t* __restrict__ cidx) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const uint32_t p = pos_of[r];
    cidx[r] = bit_of(alive, p) ? row_of(alive, wpre, p) : NONE;
  }
}

// Hub rows: the H most-gathered rows (by a 65536-bin histogram of gather
// counts, rows with counts from the threshold up).
__global__ void __launch_bounds__(256)
    k_hub_hist(const uint32_t* __restrict__ uses, uint32_t n_r, uint32_t* __restrict__ h) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_r; i += gridDim.x * blockDim.x)
    atomicAdd(&h[min(uses[i], HUB_BINS - 1)], 1u);
}

__global__ void __launch_bounds__(SCAN_TPB)
    k_hub_thresh(const uint32_t* __restrict__ h, uint32_t H, uint32_t* __restrict__ thr) {
  // thread t owns bins [t * B, (t + 1) * B); suffix sums from the top bin
  constexpr uint32_t B = HUB_BINS / SCAN_TPB;
  const uint32_t t = threadIdx.x;
  uint32_t s = 0;
  for (uint32_t b = 0; b < B; ++b) s += h[t * B + b];
  // exclusive scan in reversed thread order = rows in bins above my chunk
  __shared__ uint32_t rev[SCAN_TPB];
  rev[SCAN_TPB - 1 - t] = s;
  __syncthreads();
  const uint32_t mine = rev[t];
  uint32_t tot;
  const uint32_t above_rev = block_exscan<uint32_t>(mine, &tot);
  __syncthreads();
  rev[t] = above_rev;  // for reversed index t: rows in chunks above chunk (SCAN_TPB-1-t)
  __syncthreads();
  const uint32_t above = rev[SCAN_TPB - 1 - t];
  if (t == 0) *thr = 0xFFFFFFFFu;
  __syncthreads();
  // the chunk where the running count from the top first exceeds H
  if (above <= H && above + s > H) {
    uint32_t acc = above;
    for (uint32_t b = B; b-- > 0;) {
      acc += h[t * B + b];
      if (acc > H) {
        *thr = t * B + b + 1;  // rows with counts >= thr: at most H
        break;
      }
    }
  }
  __syncthreads();
  if (t == 0 && *thr == 0xFFFFFFFFu) *thr = 1;  // fewer than H rows in all: every used row
}

__global__ void __launch_bounds__(256)
    k_hub_bits(const uint32_t* __restrict__ uses, uint32_t n_r, const uint32_t* __restrict__ thr,
               uint32_t* __restrict__ bits) {
  const uint32_t t = *thr;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * blockDim.x / 32;
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < n_r;
       base += warps * 32) {
    const uint32_t i = base + lane;
    const uint32_t u = i < n_r ? uses[i] : 0;
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, u >= t && u > 0);
    if (lane == 0) bits[base >> 5] = m;
  }
}

unsigned grid_for(uint64_t items, unsigned tpb, unsigned cap = 152 * 16) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((items + tpb - 1) / tpb, cap));
}

}  // namespace

// Scratch of the device schedule builder (per context; sized by the graph).
struct SchedScratch {
  uint32_t* alive = nullptr;  // [W + 1] bitmap by position
  uint32_t* ist = nullptr;    // [W + 1] target positions
  uint32_t* cnt = nullptr;    // [n]
  uint32_t* front = nullptr;  // [2n] peeling frontiers
  uint32_t* wpre = nullptr;   // [W + 1]
  uint32_t* rowpos = nullptr;  // [n]
  uint64_t* rdeg = nullptr;   // [n]
  uint64_t* rpre = nullptr;   // [n + 1]
  uint64_t* bsum64 = nullptr;  // block sums
  uint32_t* bsum32 = nullptr;
  uint32_t* lvlrow = nullptr;  // [L + 1]
  uint32_t* lvl_item = nullptr;  // [L + 1]
  uint32_t* hist = nullptr;   // [L * s1]
  uint32_t* clist = nullptr;  // [n] candidate positions (ancestors of the targets)
  uint32_t* meta = nullptr;   // [META_WORDS]: frontier sizes, n_r, candidates, barrier
  uint32_t* tgt = nullptr;    // uploaded targets
  uint32_t* h_back = nullptr;  // page-locked read-back: meta words, totals, lvl_item
  size_t cap_alive = 0, cap_ist = 0, cap_cnt = 0, cap_front = 0, cap_wpre = 0, cap_rowpos = 0,
         cap_rdeg = 0, cap_rpre = 0, cap_b64 = 0, cap_b32 = 0, cap_lvlrow = 0, cap_lvli = 0,
         cap_hist = 0, cap_meta = 0, cap_tgt = 0, cap_clist = 0;
  unsigned peel_blocks = 0;  // co-resident blocks of the peeling launch
  size_t back_words = 0;
};

void free_sched_scratch(SchedScratch* s) {
  if (!s) return;
  void* p[] = {s->alive, s->ist, s->cnt, s->front, s->wpre, s->rowpos, s->rdeg, s->rpre,
               s->bsum64, s->bsum32, s->lvlrow, s->lvl_item, s->hist, s->meta, s->tgt, s->clist};
  for (void* q : p)
    if (q) cudaFree(q);
  if (s->h_back) cudaFreeHost(s->h_back);
  delete s;
}

bf_status build_schedule_device(Graph* g, Ctx& c, Sched& sc, const uint32_t* h_tgt,
                                const uint32_t* d_tgt, uint64_t T, uint64_t key,
                                cudaStream_t st) {
  const uint32_t n = g->n, L = g->n_levels;
  const uint32_t W = (n + 31) / 32;
  const uint32_t SPLIT = std::max<uint32_t>(1, g->tune.split);
  const uint32_t SMALL_SPLIT = std::max<uint32_t>(1, std::min(SPLIT, g->tune.small_split));
  SplitCfg cfg{SPLIT, SMALL_SPLIT, g->tune.small_rows, SPLIT + 1};
  if (!c.sd) {
    c.sd = new (std::nothrow) SchedScratch();
    if (!c.sd) {
      set_error("out of host memory");
      return BF_ERR_OOM;
    }
  }
  SchedScratch& s = *c.sd;
  const uint64_t nb_rows = (n + SCAN_BLOCK - 1) / SCAN_BLOCK + 1;
  const uint64_t nb_words = (W + 1 + SCAN_BLOCK - 1) / SCAN_BLOCK + 1;
  bf_status rc;
  if ((rc = ensure_dev(&s.alive, s.cap_alive, W + 1, g)) ||
      (rc = ensure_dev(&s.clist, s.cap_clist, n, g)) ||
      (rc = ensure_dev(&s.ist, s.cap_ist, W + 1, g)) ||
      (rc = ensure_dev(&s.cnt, s.cap_cnt, n, g)) ||
      (rc = ensure_dev(&s.front, s.cap_front, 2 * (size_t)n, g)) ||
      (rc = ensure_dev(&s.wpre, s.cap_wpre, W + 2, g)) ||
      (rc = ensure_dev(&s.rowpos, s.cap_rowpos, n, g)) ||
      (rc = ensure_dev(&s.rdeg, s.cap_rdeg, n, g)) ||
      (rc = ensure_dev(&s.rpre, s.cap_rpre, (size_t)n + 1, g)) ||
      (rc = ensure_dev(&s.bsum64, s.cap_b64, nb_rows + 1, g)) ||
      (rc = ensure_dev(&s.bsum32, s.cap_b32, nb_words + 1, g)) ||
      (rc = ensure_dev(&s.lvlrow, s.cap_lvlrow, (size_t)L + 1, g)) ||
      (rc = ensure_dev(&s.lvl_item, s.cap_lvli, (size_t)L + 1, g)) ||
      (rc = ensure_dev(&s.hist, s.cap_hist, (size_t)L * cfg.s1, g)) ||
      (rc = ensure_dev(&s.meta, s.cap_meta, META_WORDS, g)) ||
      (rc = ensure_dev(&sc.d_split, sc.cap_split, (size_t)W + 1, g)) ||
      (rc = ensure_dev(&sc.d_cidx, sc.cap_cidx, n, g)))
    return rc;
  if (!g->d_lvl_start) {
    set_error("device schedule: level table missing");
    return BF_ERR_DEVICE;
  }
  const size_t back = 4 + 3 * ((size_t)L + 1);
  if (back > s.back_words) {
    if (s.h_back) cudaFreeHost(s.h_back);
    s.h_back = nullptr;
    s.back_words = 0;
    if (cudaHostAlloc((void**)&s.h_back, back * 4, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      set_error("cannot allocate the schedule read-back buffer");
      return BF_ERR_OOM;
    }
    s.back_words = back;
  }
  if (!d_tgt) {
    if ((rc = ensure_dev(&s.tgt, s.cap_tgt, T, g))) return rc;
    if (T) BF_CUDA(cudaMemcpyAsync(s.tgt, h_tgt, T * 4, cudaMemcpyHostToDevice, st));
    d_tgt = s.tgt;
  }
  BF_CUDA(cudaMemsetAsync(s.alive, 0, (size_t)(W + 1) * 4, st));
  BF_CUDA(cudaMemsetAsync(s.ist, 0, (size_t)(W + 1) * 4, st));
  BF_CUDA(cudaMemsetAsync(s.meta, 0, META_WORDS * 4, st));
  BF_CUDA(cudaMemsetAsync(s.hist, 0, (size_t)L * cfg.s1 * 4, st));
  // 1. ancestors of the targets
  uint32_t* d_nc = s.meta + META_NC;
  if (T)
    k_sd_mark<<<(unsigned)((T + 3) / 4), 128, 0, st>>>(d_tgt, (uint32_t)T, g->d_parent,
                                                        g->d_run_end, g->d_pos_of, n, s.alive,
                                                        s.ist, s.cnt, s.clist, d_nc, g->d_err);
  // 2. peeling
  k_sd_count<<<152 * 8, 256, 0, st>>>(s.clist, d_nc, g->d_in_off, g->d_in_rec, s.cnt);
  k_sd_front0<<<152 * 8, 256, 0, st>>>(s.clist, d_nc, s.alive, s.ist, s.cnt, s.front, s.meta);
  if (!s.peel_blocks) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sd_peel, 256, 0) !=
        cudaSuccess) {
      cudaGetLastError();
      per_sm = 1;
    }
    s.peel_blocks = std::max(1u, std::min(4u, (unsigned)std::max(per_sm, 1)) * g->sm_count);
  }
  const bool hook = test_withhold_arrival();
  BF_CUDA(launch_persistent(k_sd_peel, hook ? 2u : s.peel_blocks, 256, st, s.front, n, s.meta,
                            PEEL_ROUNDS, (const uint64_t*)g->d_in_off,
                            (const uint2*)g->d_in_rec, s.cnt, s.alive, (const uint32_t*)s.ist,
                            hook ? 2000000ll : BARRIER_TIMEOUT_CYCLES, hook ? 1u : NONE,
                            g->d_err));
  // 3. compaction
  const unsigned nbw = (unsigned)((W + 1 + SCAN_BLOCK - 1) / SCAN_BLOCK);
  PopVal pv{s.alive};
  k_scan_sums<uint32_t><<<nbw, SCAN_TPB, 0, st>>>(pv, W, nullptr, s.bsum32);
  k_scan_top<uint32_t><<<1, SCAN_TPB, 0, st>>>(s.bsum32, nbw);
  k_scan_out<uint32_t><<<nbw, SCAN_TPB, 0, st>>>(pv, W, nullptr, s.bsum32, nbw, s.wpre);
  uint32_t* d_nr = s.meta + META_NR;
  k_sd_rows<<<grid_for(W, 256), 256, 0, st>>>(s.alive, s.wpre, W, s.rowpos);
  k_sd_lvlrow<<<(L + 1 + 255) / 256, 256, 0, st>>>(g->d_lvl_start, L, s.alive, s.wpre, s.lvlrow,
                                                    d_nr, W);
  k_sd_deg<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(s.rowpos, d_nr, g->d_in_off, s.lvlrow, L,
                                                      cfg, s.rdeg, s.hist, sc.d_split);
  const unsigned nbr = (unsigned)((n + SCAN_BLOCK - 1) / SCAN_BLOCK);
  U64Val uv{s.rdeg};
  k_scan_sums<uint64_t><<<nbr, SCAN_TPB, 0, st>>>(uv, 0, d_nr, s.bsum64);
  k_scan_top<uint64_t><<<1, SCAN_TPB, 0, st>>>(s.bsum64, nbr);
  k_scan_out<uint64_t><<<nbr, SCAN_TPB, 0, st>>>(uv, 0, d_nr, s.bsum64, nbr, s.rpre);
  k_sd_cursor<<<1, SCAN_TPB, 0, st>>>(s.hist, L, cfg.s1, s.lvl_item);
  // level -> first edge record, into the peeling frontier (free by now)
  k_sd_lvledge<<<(L + 1 + 255) / 256, 256, 0, st>>>(s.lvlrow, s.rpre, L, s.front);
  BF_CUDA(cudaGetLastError());
  // read back: n_r, total (edges | items << 32), peel rounds used, level items
  BF_CUDA(cudaMemcpyAsync(s.h_back, d_nr, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaMemcpyAsync(s.h_back + 1, s.bsum64 + nbr, 8, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaMemcpyAsync(s.h_back + 3, s.meta + META_LEFT, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaMemcpyAsync(s.h_back + 4 + (L + 1), s.lvlrow, ((size_t)L + 1) * 4,
                          cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaMemcpyAsync(s.h_back + 4 + 2 * (L + 1), s.front, ((size_t)L + 1) * 4,
                          cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaMemcpyAsync(s.h_back + 4, s.lvl_item, ((size_t)L + 1) * 4, cudaMemcpyDeviceToHost,
                          st));
  BF_CUDA(cudaStreamSynchronize(st));
  const uint32_t n_r = s.h_back[0];
  uint64_t tot;
  std::memcpy(&tot, s.h_back + 1, 8);
  const uint64_t n_e = tot & 0xFFFFFFFFull, n_i = tot >> 32;
  if (n_i != s.h_back[4 + L] || n_r > n) {
    set_error("device schedule: inconsistent counts");
    return BF_ERR_DEVICE;
  }
  sc.valid = false;
  const bool two = g->has_len;
  if ((rc = ensure_dev(&sc.d_item, sc.cap_items, n_i, g, true)) ||
      (rc = ensure_dev(&sc.d_erec, sc.cap_edges, n_e + 2, g, true)) ||
      (two && (rc = ensure_dev(&sc.d_elen, sc.cap_elen, n_e, g, true))) ||
      (rc = ensure_dev(&sc.d_trow, sc.cap_t, T, g, true)) ||
      (rc = ensure_dev(&sc.d_lvl, sc.cap_lvl, (size_t)L + 1, g)) ||
      (rc = ensure_dev(&sc.d_uses, sc.cap_uses, (size_t)n_r + 1, g, true)))
    return rc;
  BF_CUDA(cudaMemsetAsync(sc.d_uses, 0, (size_t)std::max<uint32_t>(n_r, 1) * 4, st));
  // 4. fill
  k_sd_fill<<<grid_for(n_r, 256, 152 * 8), 256, 0, st>>>(
      s.rowpos, d_nr, s.rpre, g->d_in_off, g->d_in_rec, two ? g->d_in_len : nullptr, s.alive,
      s.wpre, s.lvlrow, L, cfg, s.hist, sc.d_item, sc.d_erec, two ? sc.d_elen : nullptr,
      sc.d_uses);
  if (T)
    k_sd_trow<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(d_tgt, T, g->d_pos_of, s.alive,
                                                            s.wpre, sc.d_trow);
  k_sd_cidx<<<grid_for(n, 256), 256, 0, st>>>(g->d_pos_of, n, s.alive, s.wpre, sc.d_cidx);
  BF_CUDA(cudaMemcpyAsync(sc.d_lvl, s.lvl_item, ((size_t)L + 1) * 4, cudaMemcpyDeviceToDevice,
                          st));
  BF_CUDA(cudaGetLastError());
  sc.lvl_item.assign(s.h_back + 4, s.h_back + 4 + L + 1);
  sc.lvl_row.assign(s.h_back + 4 + (L + 1), s.h_back + 4 + 2 * (L + 1));
  sc.lvl_edge.assign(s.h_back + 4 + 2 * (L + 1), s.h_back + 4 + 3 * (L + 1));
  sc.n_r = n_r;
  sc.n_items = n_i;
  sc.n_edges = n_e;
  sc.T = T;
  sc.key = key;
  sc.tgt.assign(h_tgt, h_tgt + T);
  sc.uses = 0;
  sc.dev_built = true;
  sc.lvl_erec_ready = false;
  sc.peel_left = s.h_back[3];
  sc.ranks.clear();
  sc.cidx_ready = true;
  sc.cidx_dirty = true;  // every rank was written: a host build must reset the map whole
  sc.hub_order.clear();
  sc.hub_rows = NONE;
  sc.valid = true;
  return BF_OK;
}

// Hub rows of a device-built schedule: the H most-gathered rows as the
// schedule's device bitmap (the host-built form is in engine_batched.cu).
bf_status hub_rows_device(Graph* g, Sched& sc, uint32_t H, cudaStream_t st) {
  bf_status rc;
  const uint32_t words = (std::max<uint32_t>(sc.n_r, 1) + 31) / 32;
  if ((rc = ensure_dev(&sc.d_hub, sc.cap_hub, (size_t)words + 1, g)) ||
      (rc = ensure_dev(&sc.d_hub_h, sc.cap_hub_h, HUB_BINS + 1, g)))
    return rc;
  BF_CUDA(cudaMemsetAsync(sc.d_hub_h, 0, HUB_BINS * 4, st));
  k_hub_hist<<<grid_for(sc.n_r, 256), 256, 0, st>>>(sc.d_uses, sc.n_r, sc.d_hub_h);
  uint32_t* thr = sc.d_hub_h + HUB_BINS;
  k_hub_thresh<<<1, SCAN_TPB, 0, st>>>(sc.d_hub_h, H, thr);
  k_hub_bits<<<grid_for(sc.n_r, 256, 152 * 8), 256, 0, st>>>(sc.d_uses, sc.n_r, thr, sc.d_hub);
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

}  // namespace bf
