// noalloc.cu — bf_query_batch_noalloc: distances from up to 32 sources to
// every node, computed without allocating any memory.
//
// Some callers cannot call cudaMalloc: a host process whose device memory is
// fully reserved up front by its own pool allocator (it hands the library
// exactly the buffers it may touch), or code on a latency-critical path where
// cudaMalloc's implicit device synchronisation would stall the other streams
// of the process. For them this entry point takes device input and output
// buffers from the caller and keeps its only scratch — the per-source
// ancestor-path arrays of the upward pass — in the file-scope device array
// below, of fixed size BF_NOALLOC_SCRATCH_BYTES. Every GPU that loads the
// library holds that array until the process exits.
//
// Host code never uses the array's name as an address (on the host it is only
// a stand-in symbol): the device address is resolved with
// cudaGetSymbolAddress, once per device with that device current, and cached;
// calls pass the cached pointer to the kernels. CUDA loads this file's module
// (and with it the array) lazily, at that first resolution, and the loading
// itself allocates device memory. So bf_graph_create resolves it on the
// graph's device, and a call with k = 0 does too (a warm-up): a caller that
// reserves all remaining device memory for its own pool after creating the
// graph, or that captures streams, has the array in place before either.
//
// All calls share the array and it keeps the last call's contents, so each
// call re-initialises every scratch entry it reads. Calls whose kernels
// overlap on the GPU (e.g. issued on different streams) race on the array;
// callers must serialise them.

#include <algorithm>
#include <mutex>

#include "engine.cuh"

namespace bf {

namespace {

constexpr uint32_t NA_WORDS = BF_NOALLOC_SCRATCH_BYTES / 4;
constexpr uint32_t NA_MAX_K = 32;
constexpr int NA_MAX_DEVICES = 64;

static __device__ __align__(256) uint32_t g_noalloc_scratch[NA_WORDS];

std::mutex na_mu;
uint32_t* na_ptr[NA_MAX_DEVICES] = {};

}  // namespace

// Resolve the scratch array's device address on `device` (current).
bf_status na_scratch(int device, uint32_t** out) {
  std::lock_guard<std::mutex> lk(na_mu);
  if (device < 0 || device >= NA_MAX_DEVICES) {
    set_error("bf_query_batch_noalloc: device ordinal out of range");
    return BF_ERR_INVALID;
  }
  if (!na_ptr[device]) {
    uint32_t* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    na_ptr[device] = p;
  }
  *out = na_ptr[device];
  return BF_OK;
}

namespace {

__global__ void k_na_fill(uint32_t* __restrict__ d, uint64_t m) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    d[i] = INF;
}

// One warp per source: ancestor path (nodes and distances) in the scratch,
// settled distances written to dist[w * n + rank].
__global__ void __launch_bounds__(128)
    k_na_upward(const uint32_t* __restrict__ src, uint32_t k, const uint32_t* __restrict__ parent,
                const uint32_t* __restrict__ run_end, const uint32_t* __restrict__ depth,
                const uint64_t* __restrict__ up_off, const uint2* __restrict__ up_rec, uint32_t n,
                uint32_t* __restrict__ scratch, uint32_t stride, uint32_t* __restrict__ dist,
                uint32_t* __restrict__ err) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= k) return;
  const uint32_t s = src[w];
  if (s >= n) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  const uint32_t D = depth[s] + 1;
  uint32_t* pd = scratch + (size_t)w * stride;
  uint32_t* pn = pd + stride / 2;
  if (D > stride / 2) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  uint32_t i = 0, x = s;
  bool ok = true;
  while (x != NONE) {
    uint32_t e = run_end[x], len = e - x + 1;
    if (i + len > D) {
      ok = false;
      break;
    }
    for (uint32_t l = lane; l < len; l += 32) pn[i + l] = x + l;
    i += len;
    x = parent[e];
  }
  if (!ok || i != D) {
    if (lane == 0) atomicOr(err, DEVERR_PATH);
    return;
  }
  for (uint32_t l = lane; l < D; l += 32) pd[l] = (l == 0) ? 0u : INF;
  __threadfence_block();
  __syncwarp();
  for (uint32_t a = 0; a < D; ++a) {
    const uint32_t d = __ldcg(&pd[a]);
    if (d == INF) continue;
    const uint32_t xa = __ldcg(&pn[a]);
    const uint64_t e1 = up_off[xa + 1];
    for (uint64_t e = up_off[xa] + lane; e < e1; e += 32) {
      const uint2 r = up_rec[e];
      const uint32_t j = a + r.x;
      if (j >= D) {
        atomicOr(err, DEVERR_EDGE);
        continue;
      }
      atomicMin(&pd[j], sat_add(d, r.y));
    }
    __threadfence_block();
    __syncwarp();
  }
  for (uint32_t l = lane; l < D; l += 32) {
    const uint32_t d = __ldcg(&pd[l]);
    if (d != INF) dist[(size_t)w * n + __ldcg(&pn[l])] = d;
  }
}

// One pull-sweep level in rank-indexed, lane-major layout: thread per
// (node, lane).
__global__ void __launch_bounds__(256)
    k_na_sweep(uint32_t p0, uint32_t p1, uint32_t k, const uint64_t* __restrict__ in_off,
               const uint2* __restrict__ in_rec, const uint32_t* __restrict__ rank_at, uint32_t n,
               uint32_t* __restrict__ dist) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t p = p0 + t / k;
  if (p >= p1) return;
  const uint32_t lane = (uint32_t)(t % k);
  uint32_t* row = dist + (size_t)lane * n;
  const uint32_t v = rank_at[p];
  uint32_t best = row[v];
  for (uint64_t e = in_off[p]; e < in_off[p + 1]; ++e) {
    const uint2 r = in_rec[e];
    best = min(best, sat_add(row[rank_at[r.x]], r.y));
  }
  row[v] = best;
}

__global__ void k_na_clamp(uint32_t* __restrict__ d, uint64_t m, uint32_t threshold) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (d[i] > threshold) d[i] = INF;
}

}  // namespace

bf_status query_batch_noalloc(Graph* g, const uint32_t* d_src, uint32_t k, uint32_t threshold,
                              uint32_t* d_out, cudaStream_t st) {
  if (k > NA_MAX_K) {
    set_error("bf_query_batch_noalloc: k = " + std::to_string(k) + " exceeds the maximum of " +
              std::to_string(NA_MAX_K) + " sources per call");
    return BF_ERR_INVALID;
  }
  const uint64_t stride = 2ull * (g->max_depth + 1);
  if ((uint64_t)k * stride > NA_WORDS) {
    set_error("bf_query_batch_noalloc: " + std::to_string(k) + " sources need " +
              std::to_string((uint64_t)k * stride * 4) + " bytes of path scratch; the static "
              "scratch holds " + std::to_string((uint64_t)BF_NOALLOC_SCRATCH_BYTES) + " bytes");
    return BF_ERR_INVALID;
  }
  // resolved before the k == 0 return, so that an empty call is a warm-up
  uint32_t* scratch = nullptr;
  bf_status s;
  if ((s = na_scratch(g->device, &scratch))) return s;
  if (k == 0) return BF_OK;
  const uint64_t m = (uint64_t)k * g->n;
  const unsigned fill_blocks = (unsigned)std::min<uint64_t>((m + 255) / 256, 152 * 32);
  k_na_fill<<<fill_blocks, 256, 0, st>>>(d_out, m);
  k_na_upward<<<(k + 3) / 4, 128, 0, st>>>(d_src, k, g->d_parent, g->d_run_end, g->d_depth,
                                          g->d_up_off, g->d_up_rec, g->n, scratch,
                                          (uint32_t)stride, d_out, g->d_err);
  for (uint32_t l = 0; l < g->n_levels; ++l) {
    const uint32_t p0 = g->lvl_start[l], p1 = g->lvl_start[l + 1];
    if (p1 == p0) continue;
    const uint64_t threads = (uint64_t)(p1 - p0) * k;
    k_na_sweep<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
        p0, p1, k, g->d_in_off, g->d_in_rec, g->d_rank_at, g->n, d_out);
  }
  if (threshold != INF) k_na_clamp<<<fill_blocks, 256, 0, st>>>(d_out, m, threshold);
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

}  // namespace bf
