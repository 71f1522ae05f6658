// seeded.cu — phantom-seeded queries.
//
//   matrix_seeded   table_phast_lopsided (route/src/matrix/bucket_ch.rs:6717-6852):
//                   one seeded PHAST field per source, evaluated at the target
//                   seeds as min over (rank, part) of F[rank] - part.
//   bounded_seeded  run_phast_bounded_fast_seeded (route/src/server/
//                   isochrone_handler.rs:338-491): settled (rank, dist <= T)
//                   pairs of one multi-seed query, ascending rank.
//
// A multi-seed source is a super-source with non-negative arcs
// (isochrone_handler.rs:366-373): each seed runs its own upward path walk
// starting at its cost and writes into the source's lane with atomicMin, so
// the lane holds min over seeds of cost + upward distance, exactly the
// multi-source upward Dijkstra.

#include <algorithm>
#include <unordered_map>

#include "engine.cuh"

namespace bf {

namespace {

// out[(s0 + s) * T + t] = min over t's seeds (r, part) of F[row(r)][s] - part,
// INF above the threshold. Tile: 32 targets x 32 lanes, transposed through
// shared memory so both the slab reads and the matrix writes are coalesced.
__global__ void __launch_bounds__(256)
    k_seeded_extract(const uint32_t* __restrict__ slab, uint32_t Kp,
                     const uint32_t* __restrict__ cidx, const uint64_t* __restrict__ toff,
                     const uint2* __restrict__ tseed, uint64_t T, uint32_t kw, uint32_t threshold,
                     uint32_t* __restrict__ out) {
  __shared__ uint32_t tile[32][33];
  const uint64_t t0 = (uint64_t)blockIdx.x * 32;
  const uint32_t l0 = blockIdx.y * 32;
  const uint32_t lane = threadIdx.x;
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint64_t t = t0 + r;
    uint32_t best = INF;
    if (t < T && l0 + lane < kw) {
      for (uint64_t k = toff[t]; k < toff[t + 1]; ++k) {
        const uint2 sd = tseed[k];  // {rank, part}
        const uint32_t f = slab[(size_t)cidx[sd.x] * Kp + l0 + lane];
        if (f == INF) continue;
        best = min(best, f > sd.y ? f - sd.y : 0u);
      }
    }
    tile[r][lane] = best;
  }
  __syncthreads();
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint32_t l = l0 + r;
    const uint64_t t = t0 + lane;
    if (l < kw && t < T) {
      const uint32_t v = tile[lane][r];
      out[(uint64_t)l * T + t] = v > threshold ? INF : v;
    }
  }
}

// One level of the gated single-lane sweep (one bounded query): a thread per
// work item. A source row takes part only when its bit in `active` is set (a
// distance within the threshold); a row whose new distance is within the
// threshold sets its own bit. The slab is one INF-initialised u32 per row.
__global__ void __launch_bounds__(128)
    k_sweep_one(const uint4* __restrict__ item, uint32_t i0, uint32_t i1,
                const uint2* __restrict__ erec, uint32_t* __restrict__ slab,
                uint32_t* __restrict__ active, const uint32_t* __restrict__ thr) {
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (i >= i1) return;
  const uint32_t threshold = *thr;
  const uint4 it = item[i];
  uint32_t acc = INF;
  for (uint32_t e = it.y; e < it.z; ++e) {
    const uint2 r = erec[e];
    if (!((active[r.x >> 5] >> (r.x & 31)) & 1u)) continue;
    acc = min(acc, sat_add(slab[r.x], r.y));
  }
  if (acc > threshold) return;  // cannot lead to a distance within the threshold
  if (it.w) atomicMin(&slab[it.x], acc);
  else if (acc < slab[it.x]) slab[it.x] = acc;
  atomicOr(&active[it.x >> 5], 1u << (it.x & 31));
}

// Settled-set compaction for one lane (lane 0): ranks in blocks of 1024.
__device__ __forceinline__ bool settled(const uint32_t* slab, uint32_t Kp, const uint32_t* cidx,
                                        const uint32_t* active, uint32_t rank, uint32_t n,
                                        uint32_t thr, uint32_t* d) {
  if (rank >= n) return false;
  const uint32_t row = cidx[rank];
  if (!((active[row >> 5] >> (row & 31)) & 1u)) return false;
  *d = slab[(size_t)row * Kp];
  return *d != INF && *d <= thr;
}

__global__ void __launch_bounds__(1024)
    k_rank_count(const uint32_t* __restrict__ slab, uint32_t Kp, const uint32_t* __restrict__ cidx,
                 const uint32_t* __restrict__ active, uint32_t n, uint32_t thr,
                 uint32_t* __restrict__ counts) {
  __shared__ uint32_t wc[32];
  uint32_t d;
  const bool ok = settled(slab, Kp, cidx, active, blockIdx.x * 1024 + threadIdx.x, n, thr, &d);
  const uint32_t b = __ballot_sync(0xFFFFFFFFu, ok);
  if ((threadIdx.x & 31) == 0) wc[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t c = 0;
    for (int i = 0; i < 32; ++i) c += wc[i];
    counts[blockIdx.x] = c;
  }
}

__global__ void __launch_bounds__(1024)
    k_rank_scatter(const uint32_t* __restrict__ slab, uint32_t Kp, const uint32_t* __restrict__ cidx,
                   const uint32_t* __restrict__ active, uint32_t n, uint32_t thr,
                   const uint64_t* __restrict__ offs, uint64_t cap, uint32_t* __restrict__ o_rank,
                   uint32_t* __restrict__ o_dist) {
  __shared__ uint32_t wc[32];
  const uint32_t rank = blockIdx.x * 1024 + threadIdx.x, w = threadIdx.x >> 5,
                 lane = threadIdx.x & 31;
  uint32_t d = INF;
  const bool ok = settled(slab, Kp, cidx, active, rank, n, thr, &d);
  const uint32_t b = __ballot_sync(0xFFFFFFFFu, ok);
  if (lane == 0) wc[w] = __popc(b);
  __syncthreads();
  if (!ok) return;
  uint64_t pos = offs[blockIdx.x];
  for (uint32_t i = 0; i < w; ++i) pos += wc[i];
  pos += __popc(b & ((1u << lane) - 1u));
  if (pos < cap) {
    o_rank[pos] = rank;
    o_dist[pos] = d;
  }
}

struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t b) {
    if (cudaMalloc(&p, std::max<size_t>(b, 16)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      set_error("cudaMalloc of " + std::to_string(b) + " bytes failed");
      return false;
    }
    return true;
  }
  template <class T>
  T* as() {
    return (T*)p;
  }
};

}  // namespace

bf_status matrix_seeded(Graph* g, Ctx& c, const bf_seed* src_seeds, const uint64_t* src_off, uint64_t S,
                        const bf_seed* tgt_seeds, const uint64_t* tgt_off, uint64_t T,
                        uint32_t threshold, uint32_t* out, uint64_t* conflicts,
                        uint64_t conflict_cap, uint64_t* n_conflicts, bf_stats* st) {
  cudaStream_t s = g->stream;
  bf_status rc;
  const uint64_t ns = src_off[S], nt = tgt_off[T];
  // target seed ranks -> restricted schedule
  std::vector<uint32_t> tr(nt);
  for (uint64_t k = 0; k < nt; ++k) tr[k] = tgt_seeds[k].rank;
  std::sort(tr.begin(), tr.end());
  tr.erase(std::unique(tr.begin(), tr.end()), tr.end());
  if ((rc = build_schedule(g, c, c.sc, tr.data(), tr.size(), false, s))) return rc;
  Sched& sc = c.sc;
  const uint64_t rows = std::max<uint32_t>(sc.n_r, 1);
  uint64_t max_lanes = ctx_budget(g, c) / (rows * 4 + (uint64_t)T * 4 * 2);
  max_lanes = max_lanes >= 32 ? max_lanes & ~31ull : 0;
  if (!max_lanes) {
    set_error("HBM budget too small for a 32-lane seeded wave");
    return BF_ERR_OOM;
  }
  const uint64_t wave = std::min<uint64_t>(max_lanes, (S + 3) & ~3ull);
  const uint32_t Kp = (uint32_t)((wave + 3) & ~3ull);
  if ((rc = ensure_slab(g, c, (size_t)rows * Kp * 4))) return rc;
  // device copies: target seeds {rank, part}, target offsets, units, output
  Dev d_ts, d_to, d_units, d_out;
  if (!d_ts.alloc(nt * 8) || !d_to.alloc((T + 1) * 8) || !d_units.alloc(ns * 12) ||
      !d_out.alloc(std::min<uint64_t>(wave, S) * T * 4))
    return BF_ERR_OOM;
  static_assert(sizeof(bf_seed) == 8, "bf_seed is two u32");
  BF_CUDA(cudaMemcpyAsync(d_ts.p, tgt_seeds, nt * 8, cudaMemcpyHostToDevice, s));
  BF_CUDA(cudaMemcpyAsync(d_to.p, tgt_off, (T + 1) * 8, cudaMemcpyHostToDevice, s));
  const unsigned tpb = std::min<uint32_t>(128, ((Kp / 4 + 31) / 32) * 32);
  const unsigned lane_blocks = (Kp / 4 + tpb - 1) / tpb;
  uint64_t launches = 0;
  std::vector<uint32_t> units;
  for (uint64_t s0 = 0; s0 < S; s0 += wave) {
    const uint64_t kw = std::min<uint64_t>(wave, S - s0);
    const uint64_t u0 = src_off[s0], u1 = src_off[s0 + kw], nu = u1 - u0;
    units.assign(3 * nu, 0);
    for (uint64_t si = s0; si < s0 + kw; ++si)
      for (uint64_t k = src_off[si]; k < src_off[si + 1]; ++k) {
        units[k - u0] = src_seeds[k].rank;
        units[nu + k - u0] = src_seeds[k].cost;
        units[2 * nu + k - u0] = (uint32_t)(si - s0);
      }
    uint32_t* du = d_units.as<uint32_t>();
    if (nu) BF_CUDA(cudaMemcpyAsync(du, units.data(), units.size() * 4, cudaMemcpyHostToDevice, s));
    if ((rc = prepare_rows(g, c, sc, du, nu, Kp, s, &launches))) return rc;
    if (nu) {
      if ((rc = launch_upward(g, du, nu, INF, sc.d_cidx, c.d_slab, Kp, nullptr, s, nullptr,
                              du + nu, du + 2 * nu)))
        return rc;
      ++launches;
    }
    if ((rc = sweep_levels(g, sc, c.d_slab, Kp, lane_blocks, tpb, s, &launches, c.d_seeded)))
      return rc;
    dim3 eg((unsigned)((T + 31) / 32), (unsigned)((kw + 31) / 32)), eb(32, 8);
    k_seeded_extract<<<eg, eb, 0, s>>>(c.d_slab, Kp, sc.d_cidx, d_to.as<uint64_t>(),
                                       d_ts.as<uint2>(), T, (uint32_t)kw, threshold,
                                       d_out.as<uint32_t>());
    BF_CUDA(cudaGetLastError());
    ++launches;
    BF_CUDA(cudaMemcpyAsync(out + s0 * T, d_out.p, kw * T * 4, cudaMemcpyDeviceToHost, s));
    BF_CUDA(cudaStreamSynchronize(s));  // units is rebuilt for the next wave
  }
  if ((rc = check_device_error(g, s))) return rc;
  // same-rank pairs belong to the caller's bucket engine (bucket_ch.rs:6786-6845)
  std::unordered_map<uint32_t, std::vector<uint32_t>> src_at;
  for (uint64_t si = 0; si < S; ++si)
    for (uint64_t k = src_off[si]; k < src_off[si + 1]; ++k)
      src_at[src_seeds[k].rank].push_back((uint32_t)si);
  std::vector<uint64_t> cells;
  for (uint64_t t = 0; t < T; ++t)
    for (uint64_t k = tgt_off[t]; k < tgt_off[t + 1]; ++k) {
      auto it = src_at.find(tgt_seeds[k].rank);
      if (it == src_at.end()) continue;
      for (uint32_t si : it->second) cells.push_back(si * T + t);
    }
  std::sort(cells.begin(), cells.end());
  cells.erase(std::unique(cells.begin(), cells.end()), cells.end());
  for (uint64_t c : cells) out[c] = INF;
  if (n_conflicts) *n_conflicts = cells.size();
  for (uint64_t i = 0; i < cells.size() && i < conflict_cap; ++i) conflicts[i] = cells[i];
  if (st) {
    st->n_batches += (S + wave - 1) / wave;
    st->waves += (S + wave - 1) / wave;
    st->kernel_launches += launches;
    st->swept_nodes = sc.n_r;
    st->swept_edges = sc.n_edges;
    st->lanes = Kp;
  }
  return BF_OK;
}

bf_status bounded_seeded(Graph* g, Ctx& c, const bf_seed* seeds, uint32_t n_seeds, uint32_t threshold,
                         uint32_t* out_rank, uint32_t* out_dist, uint64_t cap, uint64_t* n_out) {
  cudaStream_t s = g->stream;
  bf_status rc;
  if ((rc = build_schedule(g, c, c.full, nullptr, 0, true, s))) return rc;
  Sched& sc = c.full;
  const uint32_t Kp = 1, n = g->n;
  const uint64_t aw = (n + 31) / 32, nb = (n + 1023) / 1024;
  if ((rc = ensure_slab(g, c, (size_t)n * Kp * 4))) return rc;
  // persistent query state (active bitmap + threshold word) so that the level
  // launches can be replayed from a captured graph
  if (c.cap_one < aw + 4) {
    if (c.d_one) {
      cudaFree(c.d_one);
      g->device_bytes -= c.cap_one * 4;
      c.d_one = nullptr;
      c.cap_one = 0;
    }
    if (cudaMalloc(&c.d_one, (aw + 4) * 4) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc for the bounded-query state failed");
      return BF_ERR_OOM;
    }
    c.cap_one = aw + 4;
    g->device_bytes += c.cap_one * 4;
  }
  uint32_t* act = c.d_one;
  uint32_t* d_thr = c.d_one + aw;
  Dev d_u, d_cnt, d_off, d_res;
  if (!d_u.alloc((size_t)n_seeds * 12 + 16) || !d_cnt.alloc(nb * 4) || !d_off.alloc(nb * 8))
    return BF_ERR_OOM;
  std::vector<uint32_t> units(3 * (size_t)n_seeds + 4, 0);
  for (uint32_t i = 0; i < n_seeds; ++i) {
    units[i] = seeds[i].rank;
    units[n_seeds + i] = seeds[i].cost;
    units[2 * (size_t)n_seeds + i] = 0;
  }
  uint32_t* du = d_u.as<uint32_t>();
  BF_CUDA(cudaMemcpyAsync(du, units.data(), units.size() * 4, cudaMemcpyHostToDevice, s));
  BF_CUDA(cudaMemcpyAsync(d_thr, &threshold, 4, cudaMemcpyHostToDevice, s));  // lane 0's threshold
  BF_CUDA(cudaMemsetAsync(c.d_slab, 0xFF, (size_t)n * Kp * 4, s));
  BF_CUDA(cudaMemsetAsync(act, 0, aw * 4, s));
  uint64_t launches = 0;
  if (n_seeds && (rc = launch_upward(g, du, n_seeds, threshold, sc.d_cidx, c.d_slab, Kp, act, s,
                                     d_thr, du + n_seeds, du + 2 * (size_t)n_seeds)))
    return rc;
  const bool pdl = g->tune.pdl != 0;
  auto issue = [&](cudaStream_t st) -> cudaError_t {
    for (uint32_t l = 0; l < g->n_levels; ++l) {
      const uint32_t i0 = sc.lvl_item[l], i1 = sc.lvl_item[l + 1];
      if (i1 == i0) continue;
      cudaError_t e = launch_level(k_sweep_one, dim3((i1 - i0 + 127) / 128), 128, pdl, st,
                                   (const uint4*)sc.d_item, i0, i1, (const uint2*)sc.d_erec,
                                   c.d_slab, act, (const uint32_t*)d_thr);
      if (e != cudaSuccess) return e;
      ++launches;
    }
    return cudaSuccess;
  };
  // the schedule is static: from its second use the level launches are
  // captured once and replayed (geometry: slab, state, launch mode)
  if (sc.one_exec && (sc.one_slab != c.d_slab || sc.one_state != c.d_one || sc.one_pdl != pdl)) {
    cudaGraphExecDestroy(sc.one_exec);
    sc.one_exec = nullptr;
  }
  if (!sc.one_exec && sc.uses >= 1 && g->tune.graphs) {
    cudaGraph_t graph;
    uint64_t before = launches;
    BF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const cudaError_t le = issue(s);
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    launches = before;
    if (le != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      return cuda_status(le, "level launch during capture");
    }
    if (ce != cudaSuccess) return cuda_status(ce, "cudaStreamEndCapture");
    const cudaError_t ie = cudaGraphInstantiate(&sc.one_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return cuda_status(ie, "cudaGraphInstantiate");
    sc.one_slab = c.d_slab;
    sc.one_state = c.d_one;
    sc.one_pdl = pdl;
  }
  if (sc.one_exec && g->tune.graphs) {
    BF_CUDA(cudaGraphLaunch(sc.one_exec, s));
  } else {
    BF_CUDA(issue(s));
  }
  BF_CUDA(cudaGetLastError());
  k_rank_count<<<(unsigned)nb, 1024, 0, s>>>(c.d_slab, Kp, sc.d_cidx, act, n,
                                            threshold, d_cnt.as<uint32_t>());
  BF_CUDA(cudaGetLastError());
  std::vector<uint32_t> cnt(nb);
  BF_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt.p, nb * 4, cudaMemcpyDeviceToHost, s));
  BF_CUDA(cudaStreamSynchronize(s));
  std::vector<uint64_t> off(nb);
  uint64_t tot = 0;
  for (uint64_t b = 0; b < nb; ++b) {
    off[b] = tot;
    tot += cnt[b];
  }
  if (n_out) *n_out = tot;
  const uint64_t keep = std::min<uint64_t>(tot, cap);
  if (!d_res.alloc(keep * 8 + 16)) return BF_ERR_OOM;
  BF_CUDA(cudaMemcpyAsync(d_off.p, off.data(), nb * 8, cudaMemcpyHostToDevice, s));
  k_rank_scatter<<<(unsigned)nb, 1024, 0, s>>>(c.d_slab, Kp, sc.d_cidx, act, n,
                                              threshold, d_off.as<uint64_t>(), keep,
                                              d_res.as<uint32_t>(), d_res.as<uint32_t>() + keep);
  BF_CUDA(cudaGetLastError());
  if (keep) {
    BF_CUDA(cudaMemcpyAsync(out_rank, d_res.p, keep * 4, cudaMemcpyDeviceToHost, s));
    BF_CUDA(cudaMemcpyAsync(out_dist, d_res.as<uint32_t>() + keep, keep * 4,
                            cudaMemcpyDeviceToHost, s));
  }
  BF_CUDA(cudaStreamSynchronize(s));
  return check_device_error(g, s);
}

}  // namespace bf
