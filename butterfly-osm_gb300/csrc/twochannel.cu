// twochannel.cu — two-channel (time, length along the time path) seeded PHAST.
//
//   bounded_seeded_2ch  run_phast_bounded_fast_seeded_2ch
//                       (route/src/server/isochrone_handler.rs:500-625)
//   matrix_seeded_2ch   table_phast_lopsided_2ch (route/src/matrix/bucket_ch.rs:6381-6521)
//
// A label is one u64: time in the high word, length in the low word. The
// reference relaxes with "new time smaller, or equal (finite) time and
// shorter length" (isochrone_handler.rs:543-571 upward, :599-611 downward),
// which is the lexicographic order of (time, length) — the u64 order of the
// packed label. Both channels add with u32 saturation. So every min-plus step
// of the one-channel engine carries over with a u64 min: the upward path walk
// (atomicMin on u64 path labels), the pull sweep and the split-item combine.
// A label whose time is INF never becomes visible (the reference never
// stores a time of INF), so the one place where the packed order differs —
// two INF times with different lengths — does not matter.
//
// Seeds: the reference enters seed (r, t, l) only when t is below r's current
// time (isochrone_handler.rs:527-531), so among seeds on one rank the first
// with the smallest time wins, length included. The host applies that rule
// before the seeds become upward units (one unit per remaining rank).

#include <algorithm>
#include <unordered_map>

#include "engine.cuh"

namespace bf {

namespace {

constexpr uint64_t LINF = ~0ull;

__device__ __forceinline__ uint64_t lab_add(uint64_t a, uint32_t wt, uint32_t wl) {
  const uint32_t t = sat_add((uint32_t)(a >> 32), wt), l = sat_add((uint32_t)a, wl);
  return ((uint64_t)t << 32) | l;
}

template <bool GLOBAL>
__device__ __forceinline__ uint64_t lab_load(const uint64_t* p) {
  if (GLOBAL) return __ldcg((const unsigned long long*)p);
  return *(const volatile uint64_t*)p;
}

// Upward pass: warp w walks unit w's ancestor path with u64 labels, starting
// at the unit's seed label, and min-writes every label with time <= threshold
// into lane unit_lane[w] of row cidx[x] of the slab (stride u64 lanes per
// row). flag (optional) receives the row bits of those labels. Path storage
// is shared memory (GLOBAL = false, dcap entries per warp) or a per-warp
// global scratch slot of dcap labels + dcap node ids.
template <bool GLOBAL>
__global__ void __launch_bounds__(UPWARD_WARPS * 32)
    k_upward_2ch(uint32_t w0, uint32_t k, const uint32_t* __restrict__ u_rank,
                 const uint32_t* __restrict__ u_cost, const uint32_t* __restrict__ u_len,
                 const uint32_t* __restrict__ u_lane, uint32_t threshold,
                 const uint32_t* __restrict__ parent, const uint32_t* __restrict__ run_end,
                 const uint32_t* __restrict__ depth, const uint64_t* __restrict__ up_off,
                 const uint2* __restrict__ up_rec, const uint32_t* __restrict__ up_len,
                 const uint32_t* __restrict__ cidx, uint32_t n, uint64_t* __restrict__ slab,
                 uint32_t stride, uint32_t* __restrict__ flag, uint32_t dcap,
                 uint8_t* __restrict__ gscratch, uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint8_t smem2[];
  const uint32_t wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t slot = blockIdx.x * UPWARD_WARPS + wib;
  const uint32_t w = w0 + slot;
  if (w >= k) return;
  const uint32_t s = u_rank[w];
  if (s >= n) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  const uint32_t D = depth[s] + 1;
  uint64_t* pd;
  uint32_t* pn;
  if (GLOBAL) {
    pd = reinterpret_cast<uint64_t*>(gscratch + (size_t)slot * dcap * 12);
    pn = reinterpret_cast<uint32_t*>(pd + dcap);
  } else {
    pd = reinterpret_cast<uint64_t*>(smem2) + (size_t)wib * dcap;
    pn = reinterpret_cast<uint32_t*>(reinterpret_cast<uint64_t*>(smem2) + UPWARD_WARPS * dcap) +
         (size_t)wib * dcap;
  }
  if (D > dcap || walk_path(s, D, parent, run_end, pn, lane) != D) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  const uint64_t seed = ((uint64_t)u_cost[w] << 32) | u_len[w];
  for (uint32_t l = lane; l < D; l += 32) pd[l] = (l == 0) ? seed : LINF;
  if (GLOBAL) __threadfence_block();
  __syncwarp();
  const unsigned FULL = 0xFFFFFFFFu;
  uint64_t cb = 0, ce = 0;  // UP-edge range of path node (chunk base + lane)
  for (uint32_t i = 0; i < D; ++i) {
    if ((i & 31) == 0) {
      cb = ce = 0;
      if (i + lane < D) {
        const uint32_t x = GLOBAL ? __ldcg(&pn[i + lane]) : pn[i + lane];
        cb = up_off[x];
        ce = up_off[x + 1];
      }
    }
    const uint64_t b = __shfl_sync(FULL, cb, i & 31), e1 = __shfl_sync(FULL, ce, i & 31);
    const uint64_t lab = lab_load<GLOBAL>(&pd[i]);
    const uint32_t t = (uint32_t)(lab >> 32);
    if (t != INF && t <= threshold) {
      for (uint64_t e = b + lane; e < e1; e += 32) {
        const uint2 r = up_rec[e];
        const uint32_t j = i + r.x;
        if (j < D)
          atomicMin((unsigned long long*)&pd[j], (unsigned long long)lab_add(lab, r.y, up_len[e]));
        else
          atomicOr(err, DEVERR_EDGE);
      }
    }
    if (GLOBAL) __threadfence_block();
    __syncwarp();
  }
  const uint32_t out_lane = u_lane[w];
  for (uint32_t l = lane; l < D; l += 32) {
    const uint64_t lab = lab_load<GLOBAL>(&pd[l]);
    const uint32_t t = (uint32_t)(lab >> 32);
    if (t == INF || t > threshold) continue;
    const uint32_t row = cidx[GLOBAL ? __ldcg(&pn[l]) : pn[l]];
    if (row == NONE) continue;
    atomicMin((unsigned long long*)&slab[(size_t)row * stride + out_lane], (unsigned long long)lab);
    if (flag) atomicOr(&flag[row >> 5], 1u << (row & 31));
  }
}

// One level of the two-channel pull sweep: blockIdx.x = work item, a thread
// owns 2 consecutive u64 lanes (one 16-byte load per gathered row). Rows are
// Kp2 lanes wide (Kp2 even). Rows without a seed this wave read as INF.
__global__ void __launch_bounds__(256)
    k_sweep_items_2ch(const uint4* __restrict__ item, uint32_t i0, const uint2* __restrict__ erec,
                      const uint32_t* __restrict__ elen, uint64_t* __restrict__ slab, uint32_t Kp2,
                      const uint32_t* __restrict__ seeded) {
  const uint4 it = item[i0 + blockIdx.x];
  const uint32_t lane = (blockIdx.y * blockDim.x + threadIdx.x) * 2;
  if (lane >= Kp2) return;
  uint64_t a0 = LINF, a1 = LINF;
  uint32_t e = it.y;
  for (; e + 2 <= it.z; e += 2) {
    const uint2 r0 = erec[e], r1 = erec[e + 1];
    const uint32_t l0 = elen[e], l1 = elen[e + 1];
    const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(slab + (size_t)r0.x * Kp2 + lane);
    const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(slab + (size_t)r1.x * Kp2 + lane);
    a0 = min(a0, min(lab_add(a.x, r0.y, l0), lab_add(b.x, r1.y, l1)));
    a1 = min(a1, min(lab_add(a.y, r0.y, l0), lab_add(b.y, r1.y, l1)));
  }
  if (e < it.z) {
    const uint2 r0 = erec[e];
    const uint32_t l0 = elen[e];
    const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(slab + (size_t)r0.x * Kp2 + lane);
    a0 = min(a0, lab_add(a.x, r0.y, l0));
    a1 = min(a1, lab_add(a.y, r0.y, l0));
  }
  uint64_t* dst = slab + (size_t)it.x * Kp2 + lane;
  if (it.w) {
    if (a0 != LINF) atomicMin((unsigned long long*)dst, (unsigned long long)a0);
    if (a1 != LINF) atomicMin((unsigned long long*)dst + 1, (unsigned long long)a1);
  } else {
    ulonglong2 c = ((seeded[it.x >> 5] >> (it.x & 31)) & 1u)
                       ? *reinterpret_cast<const ulonglong2*>(dst)
                       : make_ulonglong2(LINF, LINF);
    c.x = min((uint64_t)c.x, a0);
    c.y = min((uint64_t)c.y, a1);
    *reinterpret_cast<ulonglong2*>(dst) = c;
  }
}

// One level of the gated single-lane sweep (one bounded query): a thread per
// work item. A source row takes part only when its bit in `active` is set (a
// time within the threshold); a row whose new label is within the threshold
// sets its own bit. The slab is INF-initialised, one u64 per row.
__global__ void __launch_bounds__(128)
    k_sweep_one_2ch(const uint4* __restrict__ item, uint32_t i0, uint32_t i1,
                    const uint2* __restrict__ erec, const uint32_t* __restrict__ elen,
                    uint64_t* __restrict__ slab, uint32_t* __restrict__ active,
                    uint32_t threshold) {
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (i >= i1) return;
  const uint4 it = item[i];
  uint64_t acc = LINF;
  for (uint32_t e = it.y; e < it.z; ++e) {
    const uint2 r = erec[e];
    if (!((active[r.x >> 5] >> (r.x & 31)) & 1u)) continue;
    acc = min(acc, lab_add(slab[r.x], r.y, elen[e]));
  }
  if (acc == LINF) return;
  if (it.w) {
    atomicMin((unsigned long long*)&slab[it.x], (unsigned long long)acc);
  } else if (acc < slab[it.x]) {
    slab[it.x] = acc;
  }
  if ((uint32_t)(acc >> 32) <= threshold) atomicOr(&active[it.x >> 5], 1u << (it.x & 31));
}

// out_t/out_l[(s0 + s) * T + t]: over t's seeds {rank, part_t, part_l} in
// order, the first one with the smallest F_t[rank] - part_t (saturating;
// INF field values skipped) gives both cells (bucket_ch.rs:6452-6472); cells
// whose time exceeds the threshold become INF in both channels. Tiles of 32
// targets x 32 lanes transposed through shared memory.
__global__ void __launch_bounds__(256)
    k_extract_2ch(const uint64_t* __restrict__ slab, uint32_t Kp2,
                  const uint32_t* __restrict__ cidx, const uint64_t* __restrict__ toff,
                  const uint32_t* __restrict__ tseed, uint64_t T, uint32_t kw, uint32_t threshold,
                  uint32_t* __restrict__ out_t, uint32_t* __restrict__ out_l) {
  __shared__ uint32_t tt[32][33], tl[32][33];
  const uint64_t t0 = (uint64_t)blockIdx.x * 32;
  const uint32_t l0 = blockIdx.y * 32;
  const uint32_t lane = threadIdx.x;
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint64_t t = t0 + r;
    uint32_t bt = INF, bl = INF;
    if (t < T && l0 + lane < kw) {
      for (uint64_t k = toff[t]; k < toff[t + 1]; ++k) {
        const uint32_t rank = tseed[3 * k], pt = tseed[3 * k + 1], pl = tseed[3 * k + 2];
        const uint64_t lab = slab[(size_t)cidx[rank] * Kp2 + l0 + lane];
        const uint32_t ft = (uint32_t)(lab >> 32);
        if (ft == INF) continue;
        const uint32_t at = ft > pt ? ft - pt : 0u;
        if (at < bt) {
          const uint32_t fl = (uint32_t)lab;
          bt = at;
          bl = fl > pl ? fl - pl : 0u;
        }
      }
    }
    if (bt > threshold) {
      bt = INF;
      bl = INF;
    }
    tt[r][lane] = bt;
    tl[r][lane] = bl;
  }
  __syncthreads();
  for (uint32_t r = threadIdx.y; r < 32; r += 8) {
    const uint32_t l = l0 + r;
    const uint64_t t = t0 + lane;
    if (l < kw && t < T) {
      out_t[(uint64_t)l * T + t] = tt[lane][r];
      out_l[(uint64_t)l * T + t] = tl[lane][r];
    }
  }
}

// Settled rows of a bounded single-lane field, ranks in blocks of 1024:
// count per block, then scatter (rank, time, length) in ascending rank.
__device__ __forceinline__ bool settled_2ch(const uint64_t* slab, const uint32_t* cidx,
                                            const uint32_t* active, uint32_t rank, uint32_t n,
                                            uint32_t thr, uint64_t* lab) {
  if (rank >= n) return false;
  const uint32_t row = cidx[rank];
  if (!((active[row >> 5] >> (row & 31)) & 1u)) return false;
  *lab = slab[row];
  const uint32_t t = (uint32_t)(*lab >> 32);
  return t != INF && t <= thr;
}

__global__ void __launch_bounds__(1024)
    k_count_2ch(const uint64_t* __restrict__ slab, const uint32_t* __restrict__ cidx,
                const uint32_t* __restrict__ active, uint32_t n, uint32_t thr,
                uint32_t* __restrict__ counts) {
  __shared__ uint32_t wc[32];
  uint64_t lab;
  const bool ok = settled_2ch(slab, cidx, active, blockIdx.x * 1024 + threadIdx.x, n, thr, &lab);
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
    k_scatter_2ch(const uint64_t* __restrict__ slab, const uint32_t* __restrict__ cidx,
                  const uint32_t* __restrict__ active, uint32_t n, uint32_t thr,
                  const uint64_t* __restrict__ offs, uint64_t cap, uint32_t* __restrict__ o_rank,
                  uint32_t* __restrict__ o_time, uint32_t* __restrict__ o_len) {
  __shared__ uint32_t wc[32];
  const uint32_t rank = blockIdx.x * 1024 + threadIdx.x, w = threadIdx.x >> 5,
                 lane = threadIdx.x & 31;
  uint64_t lab = LINF;
  const bool ok = settled_2ch(slab, cidx, active, rank, n, thr, &lab);
  const uint32_t b = __ballot_sync(0xFFFFFFFFu, ok);
  if (lane == 0) wc[w] = __popc(b);
  __syncthreads();
  if (!ok) return;
  uint64_t pos = offs[blockIdx.x];
  for (uint32_t i = 0; i < w; ++i) pos += wc[i];
  pos += __popc(b & ((1u << lane) - 1u));
  if (pos < cap) {
    o_rank[pos] = rank;
    o_time[pos] = (uint32_t)(lab >> 32);
    o_len[pos] = (uint32_t)lab;
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

// Seeds of one seed set -> upward units {rank, cost, len} appended to u:
// per rank the first seed with the smallest cost (isochrone_handler.rs:527-531).
void dedupe_seeds(const bf_seed2* s, uint64_t b, uint64_t e, std::vector<bf_seed2>& u) {
  const size_t base = u.size();
  if (e - b <= 16) {
    for (uint64_t k = b; k < e; ++k) {
      size_t j = base;
      while (j < u.size() && u[j].rank != s[k].rank) ++j;
      if (j == u.size()) u.push_back(s[k]);
      else if (s[k].cost < u[j].cost) u[j] = s[k];
    }
    return;
  }
  std::unordered_map<uint32_t, size_t> at;
  for (uint64_t k = b; k < e; ++k) {
    auto it = at.find(s[k].rank);
    if (it == at.end()) {
      at.emplace(s[k].rank, u.size());
      u.push_back(s[k]);
    } else if (s[k].cost < u[it->second].cost) {
      u[it->second] = s[k];
    }
  }
}

}  // namespace

// Upward pass of nu two-channel units: d_units holds rank[nu], cost[nu],
// len[nu], lane[nu]. Shared-memory path storage when the elimination tree is
// shallow enough, else global per-warp scratch in chunks.
static bf_status launch_upward_2ch(Graph* g, const uint32_t* d_units, uint64_t nu,
                                   uint32_t threshold, const uint32_t* cidx, uint64_t* slab,
                                   uint32_t stride, uint32_t* flag, cudaStream_t st) {
  if (!nu) return BF_OK;
  const uint32_t dcap = ((g->max_depth + 1) + 31) & ~31u;
  const uint32_t *ur = d_units, *uc = d_units + nu, *ul = d_units + 2 * nu,
                 *ua = d_units + 3 * nu;
  const size_t smem = (size_t)UPWARD_WARPS * dcap * 12;
  if (smem <= 200 * 1024) {
    BF_CUDA(cudaFuncSetAttribute(k_upward_2ch<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    k_upward_2ch<false><<<(unsigned)((nu + UPWARD_WARPS - 1) / UPWARD_WARPS), UPWARD_WARPS * 32,
                          smem, st>>>(0, (uint32_t)nu, ur, uc, ul, ua, threshold, g->d_parent,
                                      g->d_run_end, g->d_depth, g->d_up_off, g->d_up_rec,
                                      g->d_up_len, cidx, g->n, slab, stride, flag, dcap, nullptr,
                                      g->d_err);
    BF_CUDA(cudaGetLastError());
    return BF_OK;
  }
  // deep trees: a bounded number of warps per launch, each with a global slot
  const size_t per = (size_t)dcap * 12;
  uint64_t chunk = std::max<uint64_t>(UPWARD_WARPS, ((256ull << 20) / per) & ~(uint64_t)(UPWARD_WARPS - 1));
  chunk = std::min<uint64_t>(chunk, (nu + UPWARD_WARPS - 1) & ~(uint64_t)(UPWARD_WARPS - 1));
  Dev scratch;
  if (!scratch.alloc(chunk * per)) return BF_ERR_OOM;
  for (uint64_t w0 = 0; w0 < nu; w0 += chunk) {
    const uint64_t m = std::min<uint64_t>(chunk, nu - w0);
    k_upward_2ch<true><<<(unsigned)((m + UPWARD_WARPS - 1) / UPWARD_WARPS), UPWARD_WARPS * 32, 0,
                         st>>>((uint32_t)w0, (uint32_t)nu, ur, uc, ul, ua, threshold, g->d_parent,
                               g->d_run_end, g->d_depth, g->d_up_off, g->d_up_rec, g->d_up_len,
                               cidx, g->n, slab, stride, flag, dcap, scratch.as<uint8_t>(),
                               g->d_err);
    BF_CUDA(cudaGetLastError());
  }
  BF_CUDA(cudaStreamSynchronize(st));  // the scratch is freed on return
  return BF_OK;
}


bf_status matrix_seeded_2ch(Graph* g, Ctx& c, const bf_seed2* src_seeds, const uint64_t* src_off,
                            uint64_t S, const bf_seed2* tgt_seeds, const uint64_t* tgt_off,
                            uint64_t T, uint32_t threshold, uint32_t* out_time, uint32_t* out_len,
                            uint64_t* conflicts, uint64_t conflict_cap, uint64_t* n_conflicts,
                            bf_stats* st) {
  cudaStream_t s = g->stream;
  bf_status rc;
  const uint64_t nt = tgt_off[T];
  std::vector<uint32_t> tr(nt);
  for (uint64_t k = 0; k < nt; ++k) tr[k] = tgt_seeds[k].rank;
  std::sort(tr.begin(), tr.end());
  tr.erase(std::unique(tr.begin(), tr.end()), tr.end());
  if ((rc = build_schedule(g, c, c.sc, tr.data(), tr.size(), false, s))) return rc;
  Sched& sc = c.sc;
  const uint64_t rows = std::max<uint32_t>(sc.n_r, 1);
  uint64_t max_lanes = ctx_budget(g, c) / (rows * 8 + (uint64_t)T * 4 * 2 * 2);
  max_lanes = max_lanes >= 32 ? max_lanes & ~31ull : 0;
  if (!max_lanes) {
    set_error("HBM budget too small for a 32-lane two-channel wave");
    return BF_ERR_OOM;
  }
  if (g->tune.max_lanes) max_lanes = std::min<uint64_t>(max_lanes, std::max(32u, g->tune.max_lanes));
  const uint64_t wave = std::min<uint64_t>(max_lanes, (S + 1) & ~1ull);
  const uint32_t Kp2 = (uint32_t)((wave + 1) & ~1ull);
  if ((rc = ensure_slab(g, c, (size_t)rows * Kp2 * 8))) return rc;
  uint64_t* slab = reinterpret_cast<uint64_t*>(c.d_slab);
  static_assert(sizeof(bf_seed2) == 12, "bf_seed2 is three u32");
  Dev d_ts, d_to, d_units, d_out;
  const uint64_t out_cells = std::min<uint64_t>(wave, S) * T;
  if (!d_ts.alloc(nt * 12) || !d_to.alloc((T + 1) * 8) || !d_units.alloc(src_off[S] * 16) ||
      !d_out.alloc(out_cells * 8))
    return BF_ERR_OOM;
  BF_CUDA(cudaMemcpyAsync(d_ts.p, tgt_seeds, nt * 12, cudaMemcpyHostToDevice, s));
  BF_CUDA(cudaMemcpyAsync(d_to.p, tgt_off, (T + 1) * 8, cudaMemcpyHostToDevice, s));
  uint32_t* d_ot = d_out.as<uint32_t>();
  uint32_t* d_ol = d_ot + out_cells;
  const unsigned tpb = std::min<uint32_t>(128, ((Kp2 / 2 + 31) / 32) * 32);
  const unsigned lane_blocks = (Kp2 / 2 + tpb - 1) / tpb;
  uint64_t launches = 0;
  std::vector<bf_seed2> kept;
  std::vector<uint32_t> units;
  for (uint64_t s0 = 0; s0 < S; s0 += wave) {
    const uint64_t kw = std::min<uint64_t>(wave, S - s0);
    kept.clear();
    std::vector<uint32_t> lane_of;
    for (uint64_t si = s0; si < s0 + kw; ++si) {
      dedupe_seeds(src_seeds, src_off[si], src_off[si + 1], kept);
      lane_of.resize(kept.size(), (uint32_t)(si - s0));
    }
    const uint64_t nu = kept.size();
    units.assign(4 * nu, 0);
    for (uint64_t i = 0; i < nu; ++i) {
      units[i] = kept[i].rank;
      units[nu + i] = kept[i].cost;
      units[2 * nu + i] = kept[i].len;
      units[3 * nu + i] = lane_of[i];
    }
    uint32_t* du = d_units.as<uint32_t>();
    if (nu) BF_CUDA(cudaMemcpyAsync(du, units.data(), units.size() * 4, cudaMemcpyHostToDevice, s));
    // rows hold Kp2 u64 lanes = 2 * Kp2 u32 words
    if ((rc = prepare_rows(g, c, sc, du, nu, 2 * Kp2, s, &launches))) return rc;
    if ((rc = launch_upward_2ch(g, du, nu, INF, sc.d_cidx, slab, Kp2, nullptr, s))) return rc;
    if (nu) ++launches;
    for (uint32_t l = 0; l < g->n_levels; ++l) {
      const uint32_t i0 = sc.lvl_item[l], i1 = sc.lvl_item[l + 1];
      if (i1 == i0) continue;
      dim3 grid(i1 - i0, lane_blocks);
      k_sweep_items_2ch<<<grid, tpb, 0, s>>>(sc.d_item, i0, sc.d_erec, sc.d_elen, slab, Kp2,
                                            c.d_seeded);
      ++launches;
    }
    BF_CUDA(cudaGetLastError());
    dim3 eg((unsigned)((T + 31) / 32), (unsigned)((kw + 31) / 32)), eb(32, 8);
    k_extract_2ch<<<eg, eb, 0, s>>>(slab, Kp2, sc.d_cidx, d_to.as<uint64_t>(),
                                    d_ts.as<uint32_t>(), T, (uint32_t)kw, threshold, d_ot, d_ol);
    BF_CUDA(cudaGetLastError());
    ++launches;
    BF_CUDA(cudaMemcpyAsync(out_time + s0 * T, d_ot, kw * T * 4, cudaMemcpyDeviceToHost, s));
    BF_CUDA(cudaMemcpyAsync(out_len + s0 * T, d_ol, kw * T * 4, cudaMemcpyDeviceToHost, s));
    BF_CUDA(cudaStreamSynchronize(s));  // units is rebuilt for the next wave
  }
  if ((rc = check_device_error(g, s))) return rc;
  // same-rank pairs belong to the caller's two-channel bucket engine
  // (bucket_ch.rs:6460-6463, :6497-6516)
  std::unordered_map<uint32_t, std::vector<uint32_t>> src_at;
  for (uint64_t si = 0; si < S; ++si)
    for (uint64_t k = src_off[si]; k < src_off[si + 1]; ++k) {
      auto& v = src_at[src_seeds[k].rank];
      if (v.empty() || v.back() != (uint32_t)si) v.push_back((uint32_t)si);
    }
  std::vector<uint64_t> cells;
  for (uint64_t t = 0; t < T; ++t)
    for (uint64_t k = tgt_off[t]; k < tgt_off[t + 1]; ++k) {
      auto it = src_at.find(tgt_seeds[k].rank);
      if (it == src_at.end()) continue;
      for (uint32_t si : it->second) cells.push_back(si * T + t);
    }
  std::sort(cells.begin(), cells.end());
  cells.erase(std::unique(cells.begin(), cells.end()), cells.end());
  for (uint64_t x : cells) out_time[x] = out_len[x] = INF;
  if (n_conflicts) *n_conflicts = cells.size();
  for (uint64_t i = 0; i < cells.size() && i < conflict_cap; ++i) conflicts[i] = cells[i];
  if (st) {
    st->n_batches += (S + wave - 1) / wave;
    st->waves += (S + wave - 1) / wave;
    st->kernel_launches += launches;
    st->swept_nodes = sc.n_r;
    st->swept_edges = sc.n_edges;
    st->lanes = Kp2;
  }
  return BF_OK;
}

bf_status bounded_seeded_2ch(Graph* g, Ctx& c, const bf_seed2* seeds, uint32_t n_seeds,
                             uint32_t threshold, uint32_t* out_rank, uint32_t* out_time,
                             uint32_t* out_len, uint64_t cap, uint64_t* n_out) {
  cudaStream_t s = g->stream;
  bf_status rc;
  if ((rc = build_schedule(g, c, c.full, nullptr, 0, true, s))) return rc;
  Sched& sc = c.full;
  const uint32_t n = g->n;
  const uint64_t aw = (n + 31) / 32, nb = (n + 1023) / 1024;
  if ((rc = ensure_slab(g, c, (size_t)n * 8))) return rc;
  uint64_t* slab = reinterpret_cast<uint64_t*>(c.d_slab);
  std::vector<bf_seed2> kept;
  dedupe_seeds(seeds, 0, n_seeds, kept);
  const uint64_t nu = kept.size();
  Dev d_u, d_act, d_cnt, d_off, d_res;
  if (!d_u.alloc(nu * 16) || !d_act.alloc(aw * 4) || !d_cnt.alloc(nb * 4) || !d_off.alloc(nb * 8))
    return BF_ERR_OOM;
  std::vector<uint32_t> units(4 * nu, 0);
  for (uint64_t i = 0; i < nu; ++i) {
    units[i] = kept[i].rank;
    units[nu + i] = kept[i].cost;
    units[2 * nu + i] = kept[i].len;
  }
  uint32_t* du = d_u.as<uint32_t>();
  if (nu) BF_CUDA(cudaMemcpyAsync(du, units.data(), units.size() * 4, cudaMemcpyHostToDevice, s));
  BF_CUDA(cudaMemsetAsync(slab, 0xFF, (size_t)n * 8, s));
  BF_CUDA(cudaMemsetAsync(d_act.p, 0, aw * 4, s));
  uint32_t* act = d_act.as<uint32_t>();
  if ((rc = launch_upward_2ch(g, du, nu, threshold, sc.d_cidx, slab, 1, act, s))) return rc;
  for (uint32_t l = 0; l < g->n_levels; ++l) {
    const uint32_t i0 = sc.lvl_item[l], i1 = sc.lvl_item[l + 1];
    if (i1 == i0) continue;
    BF_CUDA(launch_level(k_sweep_one_2ch, dim3((i1 - i0 + 127) / 128), 128, g->tune.pdl != 0, s,
                         (const uint4*)sc.d_item, i0, i1, (const uint2*)sc.d_erec,
                         (const uint32_t*)sc.d_elen, slab, act, threshold));
  }
  BF_CUDA(cudaGetLastError());
  k_count_2ch<<<(unsigned)nb, 1024, 0, s>>>(slab, sc.d_cidx, act, n, threshold,
                                           d_cnt.as<uint32_t>());
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
  if (!d_res.alloc(keep * 12 + 16)) return BF_ERR_OOM;
  BF_CUDA(cudaMemcpyAsync(d_off.p, off.data(), nb * 8, cudaMemcpyHostToDevice, s));
  uint32_t* res = d_res.as<uint32_t>();
  k_scatter_2ch<<<(unsigned)nb, 1024, 0, s>>>(slab, sc.d_cidx, act, n, threshold,
                                             d_off.as<uint64_t>(), keep, res, res + keep,
                                             res + 2 * keep);
  BF_CUDA(cudaGetLastError());
  if (keep) {
    BF_CUDA(cudaMemcpyAsync(out_rank, res, keep * 4, cudaMemcpyDeviceToHost, s));
    BF_CUDA(cudaMemcpyAsync(out_time, res + keep, keep * 4, cudaMemcpyDeviceToHost, s));
    BF_CUDA(cudaMemcpyAsync(out_len, res + 2 * keep, keep * 4, cudaMemcpyDeviceToHost, s));
  }
  BF_CUDA(cudaStreamSynchronize(s));
  return check_device_error(g, s);
}

}  // namespace bf
