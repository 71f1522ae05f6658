// engine.cuh — internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "../../include/bf_phast.h"

namespace bf {

constexpr uint32_t INF = 0xFFFFFFFFu;
constexpr uint32_t NONE = 0xFFFFFFFFu;

// Device error codes written into the per-graph error word by kernels that
// detect an inconsistency; the host turns them into BF_ERR_DEVICE.
enum : uint32_t {
  DEVERR_PATH = 1u,       // ancestor path inconsistent with the depth table
  DEVERR_EDGE = 2u,       // upward edge leaves the ancestor path
  DEVERR_TIMEOUT = 4u,    // a bounded spin-wait ran out
  DEVERR_SMEM = 8u        // a subtree does not fit its shared-memory tile
};

__host__ __device__ __forceinline__ uint32_t sat_add(uint32_t a, uint32_t b) {
  uint32_t s = a + b;
  return (s < a) ? INF : s;  // wraps only on overflow; INF + x also saturates
}

// Ancestor path of `s` written into pn[0 .. D): runs of consecutive ranks are
// emitted by the whole warp at once. Returns D (or 0 on inconsistency).
__device__ __forceinline__ uint32_t walk_path(uint32_t s, uint32_t D,
                                              const uint32_t* __restrict__ parent,
                                              const uint32_t* __restrict__ run_end, uint32_t* pn,
                                              uint32_t lane) {
  uint32_t i = 0, x = s;
  while (x != 0xFFFFFFFFu) {
    const uint32_t e = run_end[x];
    const uint32_t len = e - x + 1;
    if (i + len > D) return 0;
    for (uint32_t l = lane; l < len; l += 32) pn[i + l] = x + l;
    i += len;
    x = parent[e];
  }
  return i == D ? D : 0;
}

// L2 eviction-priority policies and cache-hinted 16-byte global loads/stores.
__device__ __forceinline__ uint64_t l2_policy_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_normal() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint4 ld_hint(const uint32_t* a, uint64_t pol) {
  uint4 v;
  asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_hint(uint32_t* a, uint4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(a), "r"(v.x),
               "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ bool is_hub(const uint32_t* hub, uint32_t r) {
  return hub && ((hub[r >> 5] >> (r & 31)) & 1u);
}

// ---- persistent level loops -------------------------------------------------
// A persistent sweep is one cooperative launch whose blocks walk the levels
// themselves, separated by a software grid barrier, instead of one launch per
// level. Its level program lists segments: one level for the whole grid
// (followed by a barrier), or a run of consecutive small levels that block 0
// sweeps alone with __syncthreads between them (one barrier after the run).
// A segment is {first level, last level + 1 | PROG_RUN}.
constexpr uint32_t PROG_RUN = 0x80000000u;
// Cycles a block waits at a grid barrier before it gives up (about 2 s).
constexpr long long BARRIER_TIMEOUT_CYCLES = 4000000000ll;

// Grid barrier number b of a cooperative launch: bar[0] counts arrivals
// (monotonic over the launch, zeroed before it), bar[1] is set by a block
// that gave up. Every wait is bounded: past `timeout` cycles the block sets
// DEVERR_TIMEOUT and the abort flag, and all blocks leave (returns false).
// The release/acquire pair orders each block's writes before the barrier
// against every block's reads after it; callers read data other blocks wrote
// through L2 (ld.cg), never through L1.
__device__ __forceinline__ bool grid_barrier(uint32_t* bar, uint32_t b, long long timeout,
                                             uint32_t* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t target = (b + 1) * gridDim.x;
    __threadfence();
    atomicAdd(bar, 1u);
    const long long t0 = clock64();
    int ok = 1;
    for (;;) {
      uint32_t v, ab;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
      if (v >= target) break;
      asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(ab) : "l"(bar + 1) : "memory");
      if (ab) {
        ok = 0;
        break;
      }
      if (clock64() - t0 > timeout) {
        atomicOr(err, DEVERR_TIMEOUT);
        atomicExch(bar + 1, 1u);
        ok = 0;
        break;
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Lanes per batch of the plain engine (one warp lane per source).
constexpr uint32_t PLAIN_K = 32;
// Ancestor-path entries a warp keeps in shared memory during the upward pass.
constexpr uint32_t UPWARD_SMEM_PATH = 2048;
constexpr uint32_t UPWARD_WARPS = 4;

// A sweep schedule (target-restricted or full graph) with its cached CUDA graph.
struct Sched {
  bool valid = false;
  uint64_t key = 0;              // hash of the targets and split settings (a pre-check)
  std::vector<uint32_t> tgt;     // the targets the schedule was built for (compared exactly)
  uint32_t n_r = 0;              // restricted nodes
  uint64_t n_items = 0;
  uint64_t n_edges = 0;
  std::vector<uint32_t> lvl_item;  // level -> first work item, n_levels + 1
  uint32_t* d_lvl = nullptr;     // device copy of lvl_item
  size_t cap_lvl = 0;
  uint32_t* d_cidx = nullptr;    // [n] rank -> compact row or NONE
  uint4* d_item = nullptr;       // {row, edge0, edge1, split flag}
  uint2* d_erec = nullptr;       // {source row, w}
  uint32_t* d_elen = nullptr;    // length weight per edge of d_erec (two-channel graphs)
  size_t cap_elen = 0;
  uint32_t* d_trow = nullptr;    // [T] target rows
  uint32_t* d_split = nullptr;   // [rows / 32] rows reset every wave: no in-edges, or
                                 // in-edges split over items (combined by atomicMin)
  size_t cap_split = 0;
  uint64_t T = 0;
  size_t cap_items = 0, cap_edges = 0, cap_t = 0;
  uint32_t uses = 0;             // calls that reused this schedule
  cudaGraphExec_t gexec = nullptr;  // captured level launches
  uint32_t g_kp = 0, g_lb = 0, g_tpb = 0;
  uint32_t* g_slab = nullptr;
  cudaStream_t g_stream = nullptr;
  const uint32_t* g_seeded = nullptr;
  bool g_pdl = false;
  const uint32_t* g_hub = nullptr;
  bool g_hinted = false;
  // captured single-lane bounded sweep (full schedule), with its geometry
  cudaGraphExec_t one_exec = nullptr;
  const void* one_slab = nullptr;
  const void* one_state = nullptr;
  bool one_pdl = false;
  std::vector<uint32_t> hub_order;  // rows by descending gather count (most-used first)
  uint32_t* d_hub = nullptr;     // [rows / 32] hub rows (kept in L2 by cache hints)
  size_t cap_hub = 0;
  uint32_t hub_rows = 0;         // rows set in d_hub
  std::vector<uint32_t> ranks;   // ranks whose d_cidx entry is set (reset on rebuild)
  bool cidx_ready = false;       // d_cidx holds NONE outside `ranks`
  size_t cap_cidx = 0;
  // built on the device (schedule.cu): d_cidx was rewritten whole, gather
  // counts per row in d_uses feed the hub choice on the device
  bool dev_built = false;
  bool cidx_dirty = false;       // d_cidx entries outside `ranks` may be set
  uint32_t peel_left = 0;        // frontier left when the peeling round limit ended (0 = exact)
  uint32_t* d_uses = nullptr;    // [rows] gathers per row
  size_t cap_uses = 0;
  uint32_t* d_hub_h = nullptr;   // hub histogram (65536 bins) and threshold
  size_t cap_hub_h = 0;
  std::vector<uint32_t> lvl_row;   // level -> first row, n_levels + 1
  std::vector<uint32_t> lvl_edge;  // level -> first edge record, n_levels + 1
  uint32_t* d_lvl_erec = nullptr;  // [levels + 1] level -> first edge record (host builds)
  size_t cap_lvl_erec = 0;
  bool lvl_erec_ready = false;
};

struct SchedScratch;  // device schedule builder scratch (schedule.cu)
void free_sched_scratch(SchedScratch* s);

// Execution context of the batched engine: schedules, the distance slab and
// scratch of one in-flight computation. The C-ABI calls use the graph's
// context; the serving loop runs two contexts on two streams.
struct Ctx {
  Sched sc;                        // last target-restricted schedule
  Sched full;                      // every node (isochrones, seeded fields)
  uint32_t* d_slab = nullptr;      // distance slab [rows][Kp]
  size_t slab_bytes = 0;
  uint32_t* d_iso_tmp = nullptr;   // isochrone permutation and active-row bitmap
  size_t iso_tmp_bytes = 0;
  cudaEvent_t ev[4] = {};
  uint64_t budget = 0;             // slab bytes this context may use (0 = graph budget)
  std::vector<uint32_t> rowmap;    // host scratch [n], all NONE between builds
  std::vector<uint64_t> markbits;  // host scratch [n bits], all 0 between builds
  uint32_t* d_pairs = nullptr;     // device scratch for (rank, row) updates
  size_t cap_pairs = 0;
  uint32_t* d_seeded = nullptr;    // [rows / 32] rows seeded by the current wave
  size_t cap_seeded = 0;
  cudaStream_t aux = nullptr;      // side stream: upward pass overlapping the slab reset
  cudaEvent_t fork = nullptr, join = nullptr;
  uint2* d_cseed = nullptr;        // compact upward output [depth from root][source]
  size_t cap_cseed = 0;
  uint32_t* d_one = nullptr;       // bounded-query state: active bitmap, then the threshold
  size_t cap_one = 0;
  void* h_stage = nullptr;         // page-locked staging arena for schedule uploads
  size_t stage_bytes = 0;
  SchedScratch* sd = nullptr;      // device schedule builder scratch
  // level program of the persistent isochrone sweep (full schedule)
  std::vector<uint2> iso_prog;
  uint2* d_iso_prog = nullptr;
  size_t iso_prog_bytes = 0;
  uint32_t iso_prog_slots = 0;
  size_t iso_prog_levels = 0;
  uint64_t* d_count = nullptr;     // [2] algorithmic-byte and row counters of isochrone sweeps
  Sched* shared_full = nullptr;    // a full-graph schedule owned elsewhere (serving slots)
};

// Tunables of the batched sweep (chosen by bf_autotune).
struct Tune {
  uint32_t tpb = 128;        // threads per sweep block (4 lanes each)
  uint32_t split = 16;       // max in-edges per work item
  uint32_t graphs = 1;       // replay the level schedule from a CUDA graph
  uint32_t max_lanes = 0;    // lanes per wave (0 = as many as the budget allows)
  uint32_t iso_lanes = 1024; // isochrone origins per wave (spatially compact waves)
  uint32_t small_rows = 64;  // levels with fewer rows use small_split edges per item
  uint32_t small_split = 8;
  uint32_t pdl = 1;          // level launches as programmatic dependents
  uint32_t iso_half = 1;     // 16-bit isochrone lanes when all thresholds fit
  uint32_t overlap_up = 1;   // upward pass on a side stream during the slab reset
  uint32_t hub_mb = 48;      // L2 megabytes the most-gathered rows may keep (0 = off)
  uint32_t mapped_out = 1;   // bf_matrix writes a page-locked output buffer directly
  uint32_t dev_sched = 1;    // build target-restricted schedules on the device
  uint32_t persist = 1;      // bit 0: the plain engine's sweep, bit 1: isochrone waves'
                             // sweeps as one persistent launch instead of one per level
  uint32_t staged = 0;       // runs of small isochrone levels stage each level's items and
                             // edge records in shared memory by bulk copies
};

struct Graph {
  Tune tune;
  int device = 0;
  uint32_t n = 0;
  uint64_t n_up = 0, n_down = 0;
  uint32_t n_levels = 0, max_depth = 0;
  uint32_t max_runs = 0;  // most runs of consecutive ranks on one root path
  uint32_t engine = BF_ENGINE_BATCHED;
  uint32_t k_lanes = 0;
  std::atomic<uint64_t> device_bytes{0};
  uint64_t hbm_budget = 0;
  uint64_t l2_bytes = 0;          // L2 size of the device (cache-hint decisions)
  uint32_t sm_count = 0;          // streaming multiprocessors (persistent grids)
  uint32_t* d_bar = nullptr;      // grid-barrier words of persistent launches (2 per stream use)
  std::vector<uint2> plain_prog;  // level program of the plain engine's persistent sweep
  uint2* d_plain_prog = nullptr;
  size_t plain_prog_bytes = 0;
  size_t plain_prog_levels = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  std::mutex mu;

  // host tables
  std::vector<uint32_t> pos_of;     // rank -> slab position (plain engine)
  std::vector<uint32_t> lvl_start;  // level -> first position, n_levels + 1
  std::vector<uint32_t> rank_at;    // slab position -> rank

  // device: elimination tree / upward
  uint32_t* d_parent = nullptr;   // [n] etree parent rank (NONE at roots)
  uint32_t* d_run_end = nullptr;  // [n] last rank of the consecutive-parent run from r
  uint32_t* d_depth = nullptr;    // [n] etree depth
  uint64_t* d_up_off = nullptr;   // [n+1] finite UP edges by source rank
  uint2* d_up_rec = nullptr;      // {depth(src) - depth(dst), w}
  uint32_t* d_up_len = nullptr;   // length weight per UP record (two-channel graphs)
  bool has_len = false;           // created with length-along-time weights
  uint32_t* d_pos_of = nullptr;   // [n] rank -> plain slab position
  uint32_t* d_rank_at = nullptr;  // [n] plain slab position -> rank
  // device: level-ordered pull CSR (plain engine)
  uint64_t* d_in_off = nullptr;   // [n+1] by slab position
  uint2* d_in_rec = nullptr;      // {source slab position, w}
  uint32_t* d_in_len = nullptr;   // length weight per d_in_rec entry (two-channel graphs)
  uint32_t* d_lvl_start = nullptr;  // [n_levels + 1] level -> first slab position
  // device: plain engine work buffers
  uint32_t* d_dist = nullptr;     // [n][32]
  uint32_t* d_seed = nullptr;     // [n][32], all INF between calls
  uint32_t* d_flag = nullptr;     // [ceil(n/32)] seeded-row bits, all 0 between calls
  uint32_t* d_err = nullptr;      // device error word

  // host copies of the pull CSR (target restriction is computed on the host)
  std::vector<uint64_t> h_in_off;  // [n+1] by slab position
  std::vector<uint2> h_in_rec;     // {source position, w}
  std::vector<uint32_t> h_in_len;  // length weight per h_in_rec entry (two-channel graphs)

  Ctx ctx;                         // execution context of the C-ABI calls
  uint32_t* d_io = nullptr;        // bf_matrix host-call I/O buffer
  size_t io_bytes = 0;
  uint8_t* d_iso = nullptr;        // isochrone I/O: origins, thresholds, counts, bits
  size_t iso_bytes = 0;
  // bulk settled sets: per-lane popcount prefixes, a wave's output and lane
  // offsets on the device, and the page-locked staging of a call's output
  uint32_t* d_set_pre = nullptr;
  size_t set_pre_bytes = 0;
  uint32_t* d_set_out = nullptr;
  size_t set_out_bytes = 0;
  uint64_t* d_set_off = nullptr;
  size_t set_off_bytes = 0;
  uint32_t* h_set_stage = nullptr;
  uint64_t set_stage_cap = 0;      // u32 entries
};

// Level program of a persistent sweep over levels whose sizes are
// first[l + 1] - first[l] (rows or work items): levels of at most `small`
// units form runs for block 0 when two or more are consecutive.
inline std::vector<uint2> level_program(const std::vector<uint32_t>& first, uint32_t n_levels,
                                        uint32_t small) {
  std::vector<uint2> prog;
  for (uint32_t l = 0; l < n_levels; ++l) {
    const uint32_t m = first[l + 1] - first[l];
    if (!m) continue;
    if (m <= small) {
      uint32_t l1 = l + 1;
      while (l1 < n_levels && first[l1 + 1] - first[l1] <= small) ++l1;
      if (l1 - l >= 2) {
        prog.push_back(make_uint2(l, l1 | PROG_RUN));
        l = l1 - 1;
        continue;
      }
    }
    prog.push_back(make_uint2(l, l + 1));
  }
  return prog;
}

// Test hook of the persistent sweeps: with BF_TEST_WITHHOLD_ARRIVAL set in
// the environment, a persistent sweep runs on two blocks, block 1 leaves
// before its first grid-barrier arrival and the waits end after about a
// millisecond, so the call must report BF_ERR_TIMEOUT.
bool test_withhold_arrival();

// f(i) for i in [0, n) on up to 64 host threads (dynamic assignment).
template <class F>
inline void parallel_for(uint64_t n, F&& f) {
  const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(),
                                                      (unsigned)std::min<uint64_t>(n, 64)));
  std::atomic<uint64_t> next{0};
  auto work = [&]() {
    for (uint64_t i; (i = next.fetch_add(1)) < n;) f(i);
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
}

// One level launch; with `pdl` it is a programmatic dependent of the
// previous launch on the stream (the kernels wait before reading rows).
template <class... P, class... A>
inline cudaError_t launch_level(void (*kern)(P...), dim3 grid, unsigned tpb, bool pdl,
                                cudaStream_t s, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(tpb);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

// Cooperative launch of a persistent sweep kernel on `blocks` blocks.
template <class... P, class... A>
inline cudaError_t launch_persistent(void (*kern)(P...), unsigned blocks, unsigned tpb,
                                     cudaStream_t s, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(tpb);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}
// engine_plain.cu: co-resident blocks of a persistent kernel (at most cap,
// two under the test hook) and the graph's grid-barrier words
unsigned persistent_blocks(Graph* g, const void* kern, unsigned tpb, unsigned cap);
bf_status ensure_barrier(Graph* g);

// graph.cu
bf_status build_graph(const bf_cch_csr* csr, const bf_config* cfg, Graph* g,
                      const uint32_t* up_len = nullptr, const uint32_t* down_len = nullptr);
void free_graph(Graph* g);

// engine_plain.cu
bf_status plain_matrix(Graph* g, const uint32_t* d_src, uint64_t S, const uint32_t* d_tpos,
                       uint64_t T, uint32_t threshold, uint32_t* d_out, cudaStream_t st,
                       bf_stats* stats);
bf_status plain_dist(Graph* g, const uint32_t* d_src, uint32_t k, uint32_t threshold,
                     uint32_t* d_out_rank_major, cudaStream_t st);
bf_status to_positions(Graph* g, const uint32_t* d_rank, uint64_t n, uint32_t* d_pos,
                       cudaStream_t st);
bf_status check_device_error(Graph* g, cudaStream_t st);
bf_status launch_upward(Graph* g, const uint32_t* d_src, uint64_t k, uint32_t threshold,
                        const uint32_t* pos_map, uint32_t* seed, uint32_t stride, uint32_t* flag,
                        cudaStream_t st, const uint32_t* lane_thr = nullptr,
                        const uint32_t* unit_cost = nullptr, const uint32_t* unit_lane = nullptr,
                        uint32_t mode = 0);
// Output of the upward pass: the u32 slab, a 16-bit slab (isochrone lanes), or
// a compact per-source buffer of k x (max_depth + 1) {row, dist} entries that
// launch_scatter_seeds writes into the slab later (so the pass can overlap
// the slab reset, or run before the restricted schedule exists: with a null
// pos_map the entries hold ranks, which the scatter maps through `cidx`).
enum : uint32_t { UPWARD_OUT_SLAB32 = 0, UPWARD_OUT_SLAB16 = 1, UPWARD_OUT_COMPACT = 2 };
// Entries of sources [0, k) read at columns col0 .. col0 + k - 1 of rows
// `stride` entries wide (stride 0: k).
bf_status launch_scatter_seeds(Graph* g, const void* cseed, uint64_t k, const uint32_t* d_src,
                               uint32_t* slab, uint32_t Kp, cudaStream_t st, uint64_t stride = 0,
                               uint64_t col0 = 0, const uint32_t* cidx = nullptr);
__global__ void k_extract(const uint32_t* __restrict__ slab, uint32_t slab_stride,
                          const uint32_t* __restrict__ tpos, uint64_t T, uint32_t k,
                          uint32_t* __restrict__ out);

// engine_batched.cu
bf_status batched_prepare(Graph* g, uint32_t split_edges);
bf_status build_schedule(Graph* g, Ctx& c, Sched& sc, const uint32_t* h_tgt, uint64_t T, bool all,
                         cudaStream_t st, const uint32_t* d_tgt = nullptr);
// schedule.cu: the target-restricted schedule of h_tgt (host) / d_tgt (the
// same targets on the device, or null) built on the device
bf_status build_schedule_device(Graph* g, Ctx& c, Sched& sc, const uint32_t* h_tgt,
                                const uint32_t* d_tgt, uint64_t T, uint64_t key, cudaStream_t st);
bf_status hub_rows_device(Graph* g, Sched& sc, uint32_t H, cudaStream_t st);
bf_status sweep_levels(Graph* g, Sched& sc, uint32_t* slab, uint32_t Kp, unsigned lane_blocks,
                       unsigned tpb, cudaStream_t st, uint64_t* launches,
                       const uint32_t* seeded);
// Reset the slab for a wave and mark its seeded rows (the ancestor paths of
// the wave's sources) so the sweep reads a row's old value only when seeded.
void launch_mark_paths(Graph* g, const uint32_t* d_src, uint64_t k, const uint32_t* cidx,
                       uint32_t* seeded, cudaStream_t st);
void launch_init_rows(const uint32_t* seeded, const uint32_t* split, uint32_t words,
                      uint32_t* slab, uint32_t Kp, cudaStream_t st);
bf_status prepare_rows(Graph* g, Ctx& c, Sched& sc, const uint32_t* d_src, uint64_t kw,
                       uint32_t Kp, cudaStream_t st, uint64_t* launches);
bf_status sweep_levels_gated(Graph* g, Sched& sc, uint32_t* slab, uint32_t Kp, unsigned lane_blocks,
                             unsigned tpb, uint32_t* active, const uint32_t* thr, uint32_t kw,
                             cudaStream_t st, uint64_t* launches,
                             const uint32_t* seeded = nullptr);
bf_status ensure_slab(Graph* g, Ctx& c, size_t bytes);
bf_status hub_rows(Graph* g, Sched& sc, uint64_t row_bytes, cudaStream_t st, const uint32_t** hub);
uint64_t ctx_budget(Graph* g, Ctx& c);
void free_ctx(Ctx& c);
bf_status init_ctx(Ctx& c);
// pre_stride != 0: the wave's upward pass already ran (compact entries at
// columns pre_col .. pre_col + kw - 1 of rows pre_stride wide, c.join marks
// its end on the side stream).
bf_status batched_wave(Graph* g, Ctx& c, const uint32_t* d_src, uint64_t kw, uint32_t Kp,
                       cudaStream_t st, uint64_t* launches, bool timed, uint64_t pre_stride = 0,
                       uint64_t pre_col = 0);
bf_status batched_matrix(Graph* g, Ctx& c, const uint32_t* d_src, uint64_t S, const uint32_t* d_tgt,
                         uint64_t T, uint32_t threshold, uint32_t* d_out, cudaStream_t st,
                         bf_stats* stats);

// isochrone.cu
// Settled (rank, distance) lists of bulk isochrones, filled wave by wave:
// per origin of the call (its index in the call), ranks ascending.
// Where the bulk settled sets land: the graph's page-locked staging buffer
// (appended wave by wave) and each origin's place in it, or, with `on_wave`,
// a consumer of each wave's sets while they are on the device: ranks and
// distances of lane l at [off[l], off[l + 1]) of d_ranks / d_dists (device
// lane offsets in d_off), lane l being origin rows[l] of the call.
struct SettledSink {
  uint64_t base = 0;                     // input index of the chunk's first origin
  uint64_t used = 0;                     // u32 entries of the staging buffer in use
  std::vector<uint64_t> r_at, d_at, cnt;  // per origin: ranks, distances, entries
  std::function<bf_status(const uint32_t* d_ranks, const uint32_t* d_dists, const uint64_t* d_off,
                          const std::vector<uint64_t>& off, const std::vector<uint32_t>& rows,
                          cudaStream_t st)>
      on_wave;
};
// The waves of bf_isochrone_settled for n origins (chunked by bitset memory)
// into `sink`; the caller holds the graph's lock.
bf_status settled_waves(Graph* g, const uint32_t* orig, const uint32_t* thr, uint64_t n,
                        SettledSink& sink, bf_stats* st);
bf_status isochrone_bitsets(Graph* g, Ctx& c, const uint32_t* d_orig, const uint32_t* d_thr, uint64_t n,
                            uint64_t* d_bits, uint64_t* d_counts, cudaStream_t st,
                            bf_stats* stats, SettledSink* sink = nullptr);

// seeded.cu
bf_status matrix_seeded(Graph* g, Ctx& c, const bf_seed* src_seeds, const uint64_t* src_off, uint64_t S,
                        const bf_seed* tgt_seeds, const uint64_t* tgt_off, uint64_t T,
                        uint32_t threshold, uint32_t* out, uint64_t* conflicts,
                        uint64_t conflict_cap, uint64_t* n_conflicts, bf_stats* st);
bf_status bounded_seeded(Graph* g, Ctx& c, const bf_seed* seeds, uint32_t n_seeds, uint32_t threshold,
                         uint32_t* out_rank, uint32_t* out_dist, uint64_t cap, uint64_t* n_out);

// twochannel.cu
bf_status matrix_seeded_2ch(Graph* g, Ctx& c, const bf_seed2* src_seeds, const uint64_t* src_off,
                            uint64_t S, const bf_seed2* tgt_seeds, const uint64_t* tgt_off,
                            uint64_t T, uint32_t threshold, uint32_t* out_time, uint32_t* out_len,
                            uint64_t* conflicts, uint64_t conflict_cap, uint64_t* n_conflicts,
                            bf_stats* st);
bf_status bounded_seeded_2ch(Graph* g, Ctx& c, const bf_seed2* seeds, uint32_t n_seeds,
                             uint32_t threshold, uint32_t* out_rank, uint32_t* out_time,
                             uint32_t* out_len, uint64_t cap, uint64_t* n_out);

// noalloc.cu
// Device address of the static scratch array on `device` (current), resolved
// (and the array's module loaded) on the first call per device.
bf_status na_scratch(int device, uint32_t** out);
bf_status query_batch_noalloc(Graph* g, const uint32_t* d_src, uint32_t k, uint32_t threshold,
                              uint32_t* d_out, cudaStream_t st);

// trace.cu: the chosen, back-projected and simplified ring of each of n_iso
// closed rasters whose words are on the current device (d_words, laid out as
// `ras`), as bf_contour_polygons returns them; runs on st.
bf_status trace_rings_device(const uint64_t* d_words, const bf_raster* ras, uint32_t n_iso,
                             const double* cell_m, const double* simplify_m,
                             const uint8_t* has_anchor, const double* anchor_xy, cudaStream_t st,
                             std::vector<uint64_t>& ring_off, std::vector<double>& lonlat);

// k_extract_lanes (engine_batched.cu): out[s * T + t] = slab[trow[t]][s]
void launch_extract_lanes(const uint32_t* slab, uint32_t Kp, const uint32_t* trow, uint64_t T,
                          uint32_t S, uint32_t threshold, uint32_t* out, cudaStream_t st);

// api.cu
Graph* graph_of(bf_graph* h);
void set_error(const std::string& msg);
bf_status cuda_status(cudaError_t e, const char* what);

}  // namespace bf

#define BF_CUDA(call)                                                    \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) return ::bf::cuda_status(_e, #call);          \
  } while (0)
