// customize.cu — CCH customization on the GPU: the bottom-up pass and the
// triangle relaxation that turn original arc weights into the UP / DOWN
// shortcut weights (and middles) the PHAST engine consumes
// (route/src/customization.rs:953-1436).
//
// Topology: the reference's rank-space CchTopo (formats/cch_topo.rs:250-290),
// directed: UP edges u -> v (v > u) and DOWN edges u -> v (v < u), two CSRs
// with targets ascending per node. A triangle is x -> m -> y with m the
// lowest rank (DOWN edge x -> m, UP edge m -> y); it offers
// w(x -> m) + w(m -> y) to edge x -> y.
//
// The reference runs apex-parallel passes of fetch_min until a pass changes
// nothing. The value it converges to is, for every edge,
//   p(e) = min(seed(e), min over triangles (w(x->m) + w(m->y), m))
// over the converged legs (a stalled pass certifies the right-hand side and
// every stored value is either the seed or a candidate of no smaller legs).
// Both legs of a triangle have the apex m as lower endpoint, and m is a lower
// neighbour of both x and y; so p is a recursion over lower endpoints and has
// exactly one solution. One pass in an order where every node comes after
// its lower neighbours computes it: nodes are grouped by elimination-tree
// height (kept when heights strictly increase along every edge, which the
// plan verifies; else longest-path levels), and a level pushes the
// candidates of all its apexes. Middles, tie-breaks and saturating sums
// therefore match the reference bit for bit, from any seeds.
//
// State layout for the relaxation: every node j has a row R(j) of its upper
// neighbours in either direction (ascending); the unordered pair {j, v},
// v in R(j), owns one 16-byte slot holding both directions, packed
// (weight << 32 | middle): .x = j -> v (an UP edge), .y = v -> j (a DOWN
// edge). A direction the topology lacks holds u32::MAX and is never written.
// An apex m relaxes each unordered pair {x < y} of R(m) once, both
// directions: x -> y from (x -> m) + (m -> y) and y -> x from
// (y -> m) + (m -> x), all four legs in m's own row and both targets in one
// slot of x's row.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "engine.cuh"

using namespace bf;

namespace {

constexpr int RT = 256;      // threads per relaxation block
constexpr int RI = 2;        // pair candidates per thread
constexpr int RC = RT * RI;  // pair candidates per block
constexpr uint32_t DIR_DOWN = 0x80000000u;  // bottom-up list entry: a DOWN edge
// Target of a pair candidate: the pair's slot index with the directions
// present in the topology; neither bit set = nothing to relax.
constexpr uint32_t T_UP = 1u << 31;
constexpr uint32_t T_DOWN = 1u << 30;
constexpr uint32_t T_PAIR = T_DOWN - 1;
// per-pair flag byte
constexpr uint8_t P_UP = 1, P_DOWN = 2, P_UP_SHORT = 4, P_DOWN_SHORT = 8;

// Device view of a plan.
struct PlanDev {
  uint32_t n;
  const uint64_t* uo;    // UP CSR offsets [n + 1] (reference layout)
  const uint32_t* ut;    // UP targets
  const uint64_t* dof;   // DOWN CSR offsets [n + 1]
  const uint32_t* dt;    // DOWN targets
  const uint64_t* qo;    // pair rows: offsets [n + 1]
  const uint32_t* qt;    //   upper neighbours in either direction, ascending
  const uint8_t* pf;     //   per pair: P_* flags
  const uint32_t* apex;  // apexes (row of >= 2) in level order
  const uint64_t* cpre;  // pair-candidate prefix over `apex` [napex + 1]
};

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Index of v in tgt[off[u], off[u + 1]) (ascending), or ~0 when absent
// (find_edge_index, customization.rs:1507-1521).
__device__ __forceinline__ uint64_t find_edge(const uint64_t* __restrict__ off,
                                              const uint32_t* __restrict__ tgt, uint32_t u,
                                              uint32_t v) {
  uint64_t lo = __ldg(off + u);
  const uint64_t end = __ldg(off + u + 1);
  uint64_t hi = end;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (__ldg(tgt + mid) < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < end && __ldg(tgt + lo) == v) ? lo : ~0ull;
}

// Candidate value of a triangle from its two packed legs; false when a leg
// has weight (time) u32::MAX, which the reference skips.
template <bool LEX>
__device__ __forceinline__ bool candidate(uint64_t leg1, uint64_t leg2, uint32_t m,
                                          uint64_t* out) {
  const uint32_t a = (uint32_t)(leg1 >> 32), b = (uint32_t)(leg2 >> 32);
  if (a == INF || b == INF) return false;
  const uint32_t lo = LEX ? sat_add((uint32_t)leg1, (uint32_t)leg2) : m;
  *out = ((uint64_t)sat_add(a, b) << 32) | lo;
  return true;
}

// One block of RC consecutive pair candidates of a level, computed when the
// plan is built: its first candidate, the apexes [k0, k0 + na) it touches and
// its candidate count.
struct Blk {
  uint64_t cb;
  uint32_t k0;
  uint16_t na;
  uint16_t cnt;
};

// Apexes of a block staged in shared memory: candidate prefix relative to
// the block's first apex, row offset, row length, rank.
struct Stage {
  uint32_t pre[RC + 1];
  uint32_t roff[RC];
  uint32_t d[RC];
  uint32_t m[RC];
};

// Stages block `b` (plan arrays only, so it may run before the previous
// level has finished); returns the block's descriptor.
__device__ __forceinline__ Blk stage_block(const PlanDev& p, const Blk* __restrict__ blk,
                                           uint64_t b, Stage& st) {
  const Blk d = blk[b];
  const uint64_t base = __ldg(p.cpre + d.k0);
  for (uint32_t i = threadIdx.x; i <= d.na; i += blockDim.x)
    st.pre[i] = (uint32_t)(__ldg(p.cpre + d.k0 + i) - base);
  for (uint32_t i = threadIdx.x; i < d.na; i += blockDim.x) {
    const uint32_t m = __ldg(p.apex + d.k0 + i);
    const uint64_t q0 = __ldg(p.qo + m);
    st.m[i] = m;
    st.roff[i] = (uint32_t)q0;
    st.d[i] = (uint32_t)(__ldg(p.qo + m + 1) - q0);
  }
  __syncthreads();
  return d;
}

// Row i of the strict upper triangle of a d x d matrix starts at
// i * (2d - i - 1) / 2.
__device__ __forceinline__ uint32_t tri_start(uint32_t d, uint32_t i) {
  return (uint32_t)(((uint64_t)i * (2ull * d - i - 1)) >> 1);
}

// Locates the pair candidate at offset q from the block's first apex: local
// apex index k and the positions i < j of the pair in the apex's row.
__device__ __forceinline__ void locate(const Stage& st, uint32_t na, uint32_t q, uint32_t* k,
                                       uint32_t* pi, uint32_t* pj) {
  uint32_t lo = 0, hi = na;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (st.pre[mid] <= q)
      lo = mid;
    else
      hi = mid;
  }
  const uint32_t r = q - st.pre[lo];
  const uint32_t d = st.d[lo];
  // estimate the row from the quadratic, then correct it exactly
  const float b = 2.f * (float)d - 1.f;
  const float disc = fmaxf(b * b - 8.f * (float)r, 0.f);
  int i = (int)((b - sqrtf(disc)) * 0.5f);
  i = max(0, min(i, (int)d - 2));
  while (i > 0 && tri_start(d, (uint32_t)i) > r) --i;
  while (i + 1 <= (int)d - 2 && tri_start(d, (uint32_t)i + 1) <= r) ++i;
  *k = lo;
  *pi = (uint32_t)i;
  *pj = r - tri_start(d, (uint32_t)i) + (uint32_t)i + 1;
}

// Target of the pair {x, y} (x < y): its slot in x's row with the present
// directions; read from the plan's index or searched in x's row.
template <bool TIDX>
__device__ __forceinline__ uint32_t target_of(const PlanDev& p, const uint32_t* __restrict__ tidx,
                                              uint64_t c, uint32_t si, uint32_t sj) {
  if (TIDX) return __ldcs(tidx + c);  // read once per call: streaming
  const uint32_t x = __ldg(p.qt + si);
  const uint32_t y = __ldg(p.qt + sj);
  const uint64_t e = find_edge(p.qo, p.qt, x, y);
  if (e == ~0ull) return 0;
  const uint8_t f = __ldg(p.pf + e);
  return (uint32_t)e | ((f & P_UP) ? T_UP : 0u) | ((f & P_DOWN) ? T_DOWN : 0u);
}

// The target of every pair candidate, once per plan.
__global__ void __launch_bounds__(RT) k_tidx(PlanDev p, const Blk* __restrict__ blk,
                                             uint32_t* __restrict__ tidx) {
  __shared__ Stage st;
  const Blk d = stage_block(p, blk, blockIdx.x, st);
  const uint32_t q0 = (uint32_t)(d.cb - __ldg(p.cpre + d.k0));
  for (uint32_t r = threadIdx.x; r < d.cnt; r += RT) {
    uint32_t k, i, j;
    locate(st, d.na, q0 + r, &k, &i, &j);
    tidx[d.cb + r] = target_of<false>(p, nullptr, 0, st.roff[k] + i, st.roff[k] + j);
  }
}

// Relaxation of one staged block. Everything that depends on the plan alone
// (pair positions, target) is fetched first; then, after the dependency on
// the previous level (PDL: the wait on the previous launch), each pair
// candidate issues its three 16-byte slot loads (two leg pairs, the target
// pair) at once, for all of the thread's candidates together, and lowers
// each present direction with a 64-bit atomicMin when the candidate beats the
// value just read (values only decrease, so the read is an upper bound).
template <bool LEX, bool TIDX, bool PDL>
__device__ __forceinline__ void relax_block(const PlanDev& p, const Blk& d, const Stage& st,
                                            const uint32_t* __restrict__ tidx,
                                            ulonglong2* __restrict__ sl) {
  const uint32_t q0 = (uint32_t)(d.cb - __ldg(p.cpre + d.k0));
  uint32_t tg[RI], si[RI], sj[RI], am[RI];
#pragma unroll
  for (int u = 0; u < RI; ++u) {
    const uint32_t r = threadIdx.x + u * RT;
    tg[u] = 0;
    if (r < d.cnt) {
      uint32_t k, i, j;
      locate(st, d.na, q0 + r, &k, &i, &j);
      si[u] = st.roff[k] + i;
      sj[u] = st.roff[k] + j;
      am[u] = st.m[k];
      tg[u] = target_of<TIDX>(p, tidx, d.cb + r, si[u], sj[u]);
    }
  }
  if (PDL) pdl_wait();
  ulonglong2 A[RI], B[RI], T[RI];
#pragma unroll
  for (int u = 0; u < RI; ++u) {
    if (!(tg[u] & (T_UP | T_DOWN))) continue;
    A[u] = __ldcg(sl + si[u]);  // {m -> x, x -> m}
    B[u] = __ldcg(sl + sj[u]);  // {m -> y, y -> m}
    T[u] = __ldcg(sl + (tg[u] & T_PAIR));
  }
#pragma unroll
  for (int u = 0; u < RI; ++u) {
    if (!(tg[u] & (T_UP | T_DOWN))) continue;
    ulonglong2* t = sl + (tg[u] & T_PAIR);
    uint64_t cand;
    if ((tg[u] & T_UP) && candidate<LEX>(A[u].y, B[u].x, am[u], &cand) && cand < T[u].x)
      atomicMin(&t->x, (unsigned long long)cand);  // x -> y
    if ((tg[u] & T_DOWN) && candidate<LEX>(B[u].y, A[u].x, am[u], &cand) && cand < T[u].y)
      atomicMin(&t->y, (unsigned long long)cand);  // y -> x
  }
}

// One level of the relaxation as its own launch, replayed from a CUDA graph
// with programmatic dependent launches (the staging overlaps the previous
// level).
template <bool LEX, bool TIDX>
__global__ void __launch_bounds__(RT) k_relax(PlanDev p, const Blk* __restrict__ blk, uint64_t b0,
                                              const uint32_t* __restrict__ tidx,
                                              ulonglong2* __restrict__ sl) {
  __shared__ Stage st;
  const Blk d = stage_block(p, blk, b0 + blockIdx.x, st);
  pdl_launch();
  relax_block<LEX, TIDX, true>(p, d, st, tidx, sl);
}

// Middle election of the lexicographic relaxation on converged values
// (customization.rs:1340-1400): the smallest apex whose candidate equals a
// SHORTCUT direction's packed value. mid[2 * pair + 0 / 1] = UP / DOWN.
template <bool TIDX>
__global__ void __launch_bounds__(RT) k_recover(PlanDev p, const Blk* __restrict__ blk,
                                                const uint32_t* __restrict__ tidx,
                                                const ulonglong2* __restrict__ sl,
                                                uint32_t* __restrict__ mid) {
  __shared__ Stage st;
  const Blk d = stage_block(p, blk, blockIdx.x, st);
  const uint32_t q0 = (uint32_t)(d.cb - __ldg(p.cpre + d.k0));
  for (uint32_t r = threadIdx.x; r < d.cnt; r += RT) {
    uint32_t k, i, j;
    locate(st, d.na, q0 + r, &k, &i, &j);
    const uint32_t a = st.roff[k] + i, b = st.roff[k] + j;
    const uint32_t tg = target_of<TIDX>(p, tidx, d.cb + r, a, b);
    if (!(tg & (T_UP | T_DOWN))) continue;
    const uint32_t pr = tg & T_PAIR;
    const uint8_t f = __ldg(p.pf + pr);
    if (!(f & (P_UP_SHORT | P_DOWN_SHORT))) continue;
    const ulonglong2 A = __ldg(sl + a), B = __ldg(sl + b), T = __ldg(sl + pr);
    uint64_t cand;
    if ((f & P_UP_SHORT) && candidate<true>(A.y, B.x, 0, &cand) && cand == T.x)
      atomicMin(mid + 2ull * pr, st.m[k]);
    if ((f & P_DOWN_SHORT) && candidate<true>(B.y, A.x, 0, &cand) && cand == T.y)
      atomicMin(mid + 2ull * pr + 1, st.m[k]);
  }
}

// Pair slots from reference-layout inputs, one whole 16-byte slot per pair
// (coalesced writes; a direction the topology lacks is u32::MAX):
// word = (hi[e] << 32 | lo[e]) for the pair's UP edge e and DOWN edge e.
// With `us` / `ds` (the seeds of a full customization) shortcuts get weight
// u32::MAX: a shortcut's bottom-up value is dominated by the triangle through
// its own contraction middle, so the fixed point is the same. lo NULL =
// u32::MAX.
__global__ void k_pack_pairs(uint64_t np, const uint32_t* __restrict__ up_edge,
                             const uint32_t* __restrict__ dn_edge, const uint32_t* __restrict__ hu,
                             const uint32_t* __restrict__ lu, const uint8_t* __restrict__ us,
                             const uint32_t* __restrict__ hd, const uint32_t* __restrict__ ld,
                             const uint8_t* __restrict__ ds, ulonglong2* __restrict__ sl) {
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < np;
       p += (uint64_t)gridDim.x * blockDim.x) {
    ulonglong2 v;
    v.x = v.y = ~0ull;
    const uint32_t eu = up_edge[p], ed = dn_edge[p];
    if (eu != INF) {
      const uint32_t w = (us && us[eu]) ? INF : hu[eu];
      v.x = ((uint64_t)w << 32) | (lu ? lu[eu] : INF);
    }
    if (ed != INF) {
      const uint32_t w = (ds && ds[ed]) ? INF : hd[ed];
      v.y = ((uint64_t)w << 32) | (ld ? ld[ed] : INF);
    }
    sl[p] = v;
  }
}

// Pair slots back to the reference layout: w[e] = weight; mid[e] = packed
// low word, or (lexicographic) the elected middle when there is one.
__global__ void k_gather(uint64_t n, const uint32_t* __restrict__ pair, int dir,
                         const ulonglong2* __restrict__ sl, uint32_t* __restrict__ w,
                         uint32_t* __restrict__ mid, const uint32_t* __restrict__ elected) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t pr = pair[e];
    const uint64_t v = reinterpret_cast<const unsigned long long*>(sl + pr)[dir];
    w[e] = (uint32_t)(v >> 32);
    if (!elected) {
      mid[e] = (uint32_t)v;
    } else {
      const uint32_t m = elected[2ull * pr + dir];
      if (m != INF) mid[e] = m;
    }
  }
}

// Bottom-up pass, originals: w = original on an original edge, u32::MAX on a
// shortcut (filled level by level next).
__global__ void k_bu_orig(uint64_t n, const uint32_t* __restrict__ orig,
                          const uint8_t* __restrict__ is_short, uint32_t* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (is_short && is_short[i]) ? INF : orig[i];
}

// Bottom-up pass, one level: every shortcut whose lower endpoint is in the
// level takes w(u -> m) + w(m -> v) through its middle m
// (customization.rs:953-1052). A middle at or above the lower endpoint reads
// legs the reference has not computed yet (u32::MAX); a middle that is not a
// rank sets the error word.
__global__ void __launch_bounds__(256) k_bu_level(PlanDev p, uint64_t b0, uint64_t b1,
                                                  const uint32_t* __restrict__ tail,
                                                  const uint32_t* __restrict__ edge,
                                                  const uint32_t* __restrict__ mu,
                                                  const uint32_t* __restrict__ md,
                                                  uint32_t* __restrict__ wu,
                                                  uint32_t* __restrict__ wd,
                                                  uint32_t* __restrict__ err) {
  pdl_launch();
  pdl_wait();
  const uint64_t i = b0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= b1) return;
  const uint32_t u = __ldg(tail + i), ed = __ldg(edge + i);
  const bool down = ed & DIR_DOWN;
  const uint32_t e = ed & ~DIR_DOWN;
  const uint32_t v = down ? __ldg(p.dt + e) : __ldg(p.ut + e);
  const uint32_t m = down ? __ldg(md + e) : __ldg(mu + e);
  uint32_t w = INF;
  if (m >= p.n) {
    atomicOr(err, 1u);
  } else if (m < min(u, v)) {
    const uint64_t e1 = find_edge(p.dof, p.dt, u, m);
    const uint64_t e2 = find_edge(p.uo, p.ut, m, v);
    const uint32_t w1 = e1 == ~0ull ? INF : __ldcg(wd + e1);
    const uint32_t w2 = e2 == ~0ull ? INF : __ldcg(wu + e2);
    w = sat_add(w1, w2);
  }
  if (down)
    wd[e] = w;
  else
    wu[e] = w;
}

unsigned grid_for(uint64_t n, unsigned tpb) {
  const uint64_t b = (n + tpb - 1) / tpb;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, 152ull * 32));
}

}  // namespace

// ---------------------------------------------------------------------------

struct bf_cch {
  std::mutex mu;
  int device = 0;
  uint32_t n = 0;
  uint64_t nu = 0, nd = 0, npair = 0;
  cudaStream_t s = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // reference layout (bottom-up pass, seeds)
  uint64_t *d_uo = nullptr, *d_do = nullptr;
  uint32_t *d_ut = nullptr, *d_dt = nullptr;
  uint8_t *d_us = nullptr, *d_ds = nullptr;         // shortcut flags (null: none given)
  uint32_t *d_mu0 = nullptr, *d_md0 = nullptr;      // topology middles (null: all u32::MAX)
  uint32_t *d_btail = nullptr, *d_bedge = nullptr;  // bottom-up lists by level
  std::vector<uint64_t> lv_bu;                      // [levels + 1]
  // pair layout (relaxation)
  uint64_t* d_qo = nullptr;
  uint32_t* d_qt = nullptr;
  uint8_t* d_pf = nullptr;
  uint32_t *d_up_pair = nullptr, *d_dn_pair = nullptr;  // reference edge -> pair slot
  uint32_t *d_pair_up = nullptr, *d_pair_dn = nullptr;  // pair slot -> edge (u32::MAX: none)
  uint32_t* d_apex = nullptr;
  uint64_t* d_cpre = nullptr;
  Blk* d_blk = nullptr;                             // relaxation blocks, level after level
  uint32_t* d_tidx = nullptr;                       // target per pair candidate (or null)
  std::vector<uint64_t> lv_blk;                     // [levels + 1] first block per level
  uint32_t napex = 0;
  uint64_t ncand = 0;                               // pair candidates
  // working state
  ulonglong2* d_sl = nullptr;                       // one slot per pair
  uint32_t* d_elect = nullptr;                      // lexicographic election, 2 per pair
  uint32_t* d_w[4] = {nullptr, nullptr, nullptr, nullptr};  // up/down weight, up/down middle
  uint32_t* d_l[2] = {nullptr, nullptr};                    // up/down length or original
  uint32_t* d_err = nullptr;
  cudaGraphExec_t g_relax[2] = {nullptr, nullptr};  // plain, lexicographic
  cudaGraphExec_t g_bu = nullptr;
  double plan_ms = 0;
  uint32_t levels = 0;
  bool etree_levels = true;
  float last_device_ms = 0, last_total_ms = 0;

  PlanDev dev() const {
    return PlanDev{n, d_uo, d_ut, d_do, d_dt, d_qo, d_qt, d_pf, d_apex, d_cpre};
  }
};

namespace {

void free_plan(bf_cch* c) {
  for (auto& g : c->g_relax)
    if (g) cudaGraphExecDestroy(g);
  if (c->g_bu) cudaGraphExecDestroy(c->g_bu);
  void* ptrs[] = {c->d_uo, c->d_do, c->d_ut, c->d_dt, c->d_us, c->d_ds, c->d_mu0, c->d_md0,
                  c->d_btail, c->d_bedge, c->d_qo, c->d_qt, c->d_pf, c->d_up_pair, c->d_dn_pair,
                  c->d_pair_up, c->d_pair_dn,
                  c->d_apex, c->d_cpre, c->d_blk, c->d_tidx, c->d_sl, c->d_elect, c->d_w[0],
                  c->d_w[1], c->d_w[2], c->d_w[3], c->d_l[0], c->d_l[1], c->d_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->s) cudaStreamDestroy(c->s);
}

template <class T>
cudaError_t upload(T** d, const T* h, uint64_t count) {
  if (!count) return cudaSuccess;
  cudaError_t e = cudaMalloc((void**)d, count * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*d, h, count * sizeof(T), cudaMemcpyHostToDevice);
}

bool valid_csr(uint32_t n, const uint64_t* off, const uint32_t* tgt, bool up) {
  if (off[0] != 0) return false;
  for (uint32_t u = 0; u < n; ++u) {
    if (off[u + 1] < off[u]) return false;
    for (uint64_t i = off[u]; i < off[u + 1]; ++i) {
      const uint32_t v = tgt[i];
      if (v >= n || (up ? v <= u : v >= u)) return false;
      if (i > off[u] && tgt[i - 1] >= v) return false;
    }
  }
  return true;
}

bf_status build_plan(bf_cch* c, const bf_cch_topo* t) {
  const uint32_t n = t->n_nodes;
  const uint64_t nu = t->up_offsets[n], nd = t->down_offsets[n];
  const uint64_t* uo = t->up_offsets;
  const uint32_t* ut = t->up_targets;
  c->n = n;
  c->nu = nu;
  c->nd = nd;
  // reverse DOWN adjacency (build_reverse_down_adj_for_relax, customization.rs:832-875)
  std::vector<uint64_t> ro((size_t)n + 1, 0);
  for (uint64_t i = 0; i < nd; ++i) ro[t->down_targets[i] + 1]++;
  for (uint32_t m = 0; m < n; ++m) ro[m + 1] += ro[m];
  std::vector<uint32_t> rs(nd), re(nd);
  {
    std::vector<uint64_t> pos(ro.begin(), ro.end() - 1);
    for (uint32_t u = 0; u < n; ++u)
      for (uint64_t i = t->down_offsets[u]; i < t->down_offsets[u + 1]; ++i) {
        const uint64_t p = pos[t->down_targets[i]]++;
        rs[p] = u;
        re[p] = (uint32_t)i;
      }
  }
  // pair rows: UP targets of j merged with the sources of DOWN edges into j
  std::vector<uint64_t> qo((size_t)n + 1, 0);
  std::vector<uint32_t> qt, up_pair(nu), dn_pair(nd), pair_up, pair_dn;
  std::vector<uint8_t> pf;
  qt.reserve(std::max(nu, nd));
  pf.reserve(std::max(nu, nd));
  pair_up.reserve(std::max(nu, nd));
  pair_dn.reserve(std::max(nu, nd));
  for (uint32_t j = 0; j < n; ++j) {
    uint64_t a = uo[j], b = ro[j];
    const uint64_t ae = uo[j + 1], be = ro[j + 1];
    while (a < ae || b < be) {
      const uint32_t va = a < ae ? ut[a] : INF, vb = b < be ? rs[b] : INF;
      const uint32_t v = std::min(va, vb);
      const uint32_t p = (uint32_t)qt.size();
      uint8_t f = 0;
      uint32_t eu = INF, ed = INF;
      if (va == v) {
        up_pair[a] = p;
        eu = (uint32_t)a;
        f |= P_UP | ((t->up_is_shortcut && t->up_is_shortcut[a]) ? P_UP_SHORT : 0);
        ++a;
      }
      if (vb == v) {
        dn_pair[re[b]] = p;
        ed = re[b];
        f |= P_DOWN | ((t->down_is_shortcut && t->down_is_shortcut[re[b]]) ? P_DOWN_SHORT : 0);
        ++b;
      }
      qt.push_back(v);
      pf.push_back(f);
      pair_up.push_back(eu);
      pair_dn.push_back(ed);
      if (qt.size() >= T_PAIR) {
        set_error("bf_cch_create: more than 2^30 - 1 node pairs");
        return BF_ERR_INVALID;
      }
    }
    qo[j + 1] = qt.size();
  }
  c->npair = qt.size();
  // Levels: elimination-tree heights (parent = lowest upper neighbour); kept
  // when they increase strictly along every edge, else longest-path levels.
  std::vector<uint32_t> lev(n, 0);
  for (uint32_t m = 0; m < n; ++m)
    if (qo[m + 1] > qo[m]) {
      const uint32_t par = qt[qo[m]];
      lev[par] = std::max(lev[par], lev[m] + 1);
    }
  bool ok = true;
  for (uint32_t u = 0; u < n && ok; ++u)
    for (uint64_t i = qo[u]; i < qo[u + 1]; ++i)
      if (lev[qt[i]] <= lev[u]) ok = false;
  c->etree_levels = ok;
  if (!ok) {
    std::fill(lev.begin(), lev.end(), 0);
    for (uint32_t m = 0; m < n; ++m)
      for (uint64_t i = qo[m]; i < qo[m + 1]; ++i)
        lev[qt[i]] = std::max(lev[qt[i]], lev[m] + 1);
  }
  uint32_t L = 0;
  for (uint32_t m = 0; m < n; ++m) L = std::max(L, lev[m] + 1);
  c->levels = L;
  // nodes by level (ascending rank within a level)
  std::vector<uint32_t> loff((size_t)L + 1, 0), order(n);
  for (uint32_t m = 0; m < n; ++m) loff[lev[m] + 1]++;
  for (uint32_t l = 0; l < L; ++l) loff[l + 1] += loff[l];
  {
    std::vector<uint32_t> pos(loff.begin(), loff.end() - 1);
    for (uint32_t m = 0; m < n; ++m) order[pos[lev[m]]++] = m;
  }
  // apexes (rows of at least two) with their pair-candidate prefix, and the
  // relaxation blocks: RC consecutive candidates of one level each
  std::vector<uint32_t> apex;
  std::vector<uint64_t> cpre(1, 0);
  std::vector<Blk> blks;
  c->lv_blk.assign((size_t)L + 1, 0);
  for (uint32_t l = 0; l < L; ++l) {
    const uint32_t a0 = (uint32_t)apex.size();
    const uint64_t c0 = cpre.back();
    for (uint32_t i = loff[l]; i < loff[l + 1]; ++i) {
      const uint32_t m = order[i];
      const uint64_t d = qo[m + 1] - qo[m];
      if (d < 2) continue;
      const uint64_t k = d * (d - 1) / 2;
      if (k >= (1ull << 30)) {
        set_error("bf_cch_create: a node has 2^30 or more triangles");
        return BF_ERR_INVALID;
      }
      apex.push_back(m);
      cpre.push_back(cpre.back() + k);
    }
    const uint32_t a1 = (uint32_t)apex.size();
    const uint64_t c1 = cpre.back();
    uint32_t k = a0;
    for (uint64_t cb = c0; cb < c1; cb += RC) {
      const uint64_t ce = std::min<uint64_t>(cb + RC, c1);
      while (k + 1 < a1 && cpre[k + 1] <= cb) ++k;
      uint32_t k1 = k;
      while (k1 + 1 < a1 && cpre[k1 + 1] < ce) ++k1;
      blks.push_back(Blk{cb, k, (uint16_t)(k1 - k + 1), (uint16_t)(ce - cb)});
    }
    c->lv_blk[l + 1] = blks.size();
  }
  c->napex = (uint32_t)apex.size();
  c->ncand = cpre.back();
  // bottom-up lists: shortcuts by the level of their lower endpoint
  std::vector<uint32_t> btail, bedge;
  c->lv_bu.assign((size_t)L + 1, 0);
  if (t->up_is_shortcut || t->down_is_shortcut) {
    for (uint32_t l = 0; l < L; ++l) {
      for (uint32_t i = loff[l]; i < loff[l + 1]; ++i) {
        const uint32_t j = order[i];
        if (t->up_is_shortcut)
          for (uint64_t e = uo[j]; e < uo[j + 1]; ++e)
            if (t->up_is_shortcut[e]) {
              btail.push_back(j);
              bedge.push_back((uint32_t)e);
            }
        if (t->down_is_shortcut)
          for (uint64_t r = ro[j]; r < ro[j + 1]; ++r)
            if (t->down_is_shortcut[re[r]]) {
              btail.push_back(rs[r]);
              bedge.push_back(re[r] | DIR_DOWN);
            }
      }
      c->lv_bu[l + 1] = btail.size();
    }
  }
  // device copies
  BF_CUDA(upload(&c->d_uo, uo, (uint64_t)n + 1));
  BF_CUDA(upload(&c->d_do, t->down_offsets, (uint64_t)n + 1));
  BF_CUDA(upload(&c->d_ut, ut, nu));
  BF_CUDA(upload(&c->d_dt, t->down_targets, nd));
  if (t->up_is_shortcut) BF_CUDA(upload(&c->d_us, t->up_is_shortcut, nu));
  if (t->down_is_shortcut) BF_CUDA(upload(&c->d_ds, t->down_is_shortcut, nd));
  if (t->up_middle) BF_CUDA(upload(&c->d_mu0, t->up_middle, nu));
  if (t->down_middle) BF_CUDA(upload(&c->d_md0, t->down_middle, nd));
  BF_CUDA(upload(&c->d_btail, btail.data(), btail.size()));
  BF_CUDA(upload(&c->d_bedge, bedge.data(), bedge.size()));
  BF_CUDA(upload(&c->d_qo, qo.data(), qo.size()));
  BF_CUDA(upload(&c->d_qt, qt.data(), qt.size()));
  BF_CUDA(upload(&c->d_pf, pf.data(), pf.size()));
  BF_CUDA(upload(&c->d_up_pair, up_pair.data(), nu));
  BF_CUDA(upload(&c->d_dn_pair, dn_pair.data(), nd));
  BF_CUDA(upload(&c->d_pair_up, pair_up.data(), pair_up.size()));
  BF_CUDA(upload(&c->d_pair_dn, pair_dn.data(), pair_dn.size()));
  BF_CUDA(upload(&c->d_apex, apex.data(), apex.size()));
  BF_CUDA(upload(&c->d_cpre, cpre.data(), cpre.size()));
  BF_CUDA(upload(&c->d_blk, blks.data(), blks.size()));
  const uint64_t nmax = std::max<uint64_t>(1, std::max(nu, nd));
  BF_CUDA(cudaMalloc(&c->d_sl, std::max<uint64_t>(1, c->npair) * sizeof(ulonglong2)));
  for (int i = 0; i < 4; ++i) BF_CUDA(cudaMalloc(&c->d_w[i], nmax * 4));
  for (int i = 0; i < 2; ++i) BF_CUDA(cudaMalloc(&c->d_l[i], nmax * 4));
  BF_CUDA(cudaMalloc(&c->d_err, 4));
  // target index: 4 bytes per pair candidate while that fits a quarter of free HBM
  size_t fr = 0, tot = 0;
  BF_CUDA(cudaMemGetInfo(&fr, &tot));
  if (!(t->flags & BF_CCH_SEARCH_TARGETS) && c->ncand && c->ncand * 4 <= fr / 4) {
    BF_CUDA(cudaMalloc(&c->d_tidx, c->ncand * 4));
    k_tidx<<<(unsigned)blks.size(), RT, 0, c->s>>>(c->dev(), c->d_blk, c->d_tidx);
    BF_CUDA(cudaGetLastError());
    BF_CUDA(cudaStreamSynchronize(c->s));
  }
  return BF_OK;
}

// The relaxation levels on c->s; captured into a graph on first use.
bf_status run_relax(bf_cch* c, bool lex) {
  cudaGraphExec_t& ge = c->g_relax[lex ? 1 : 0];
  if (!ge) {
    cudaGraph_t g = nullptr;
    BF_CUDA(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    bool first = true;
    const PlanDev p = c->dev();
    const Blk* blk = c->d_blk;
    const uint32_t* ti = c->d_tidx;
    for (size_t l = 0; l + 1 < c->lv_blk.size() && err == cudaSuccess; ++l) {
      const uint64_t b0 = c->lv_blk[l], b1 = c->lv_blk[l + 1];
      if (b1 == b0) continue;
      const dim3 grid((unsigned)(b1 - b0));
      if (ti)
        err = lex ? launch_level(k_relax<true, true>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_sl)
                  : launch_level(k_relax<false, true>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_sl);
      else
        err = lex ? launch_level(k_relax<true, false>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_sl)
                  : launch_level(k_relax<false, false>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_sl);
      first = false;
    }
    cudaError_t e2 = cudaStreamEndCapture(c->s, &g);
    if (err == cudaSuccess) err = e2;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&ge, g, 0);
    if (g) cudaGraphDestroy(g);
    if (err != cudaSuccess) {
      ge = nullptr;
      return cuda_status(err, "relaxation graph");
    }
  }
  BF_CUDA(cudaGraphLaunch(ge, c->s));
  return BF_OK;
}

// The bottom-up levels on c->s, reading the middles staged in d_w[2], d_w[3]
// (the captured graph bakes those pointers in).
bf_status run_bottom_up(bf_cch* c) {
  if (!c->g_bu) {
    const PlanDev p = c->dev();
    cudaGraph_t g = nullptr;
    BF_CUDA(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    bool first = true;
    for (size_t l = 0; l + 1 < c->lv_bu.size() && err == cudaSuccess; ++l) {
      const uint64_t b0 = c->lv_bu[l], b1 = c->lv_bu[l + 1];
      if (b1 == b0) continue;
      err = launch_level(k_bu_level, dim3((unsigned)((b1 - b0 + 255) / 256)), 256, !first, c->s, p,
                         b0, b1, (const uint32_t*)c->d_btail, (const uint32_t*)c->d_bedge,
                         (const uint32_t*)c->d_w[2], (const uint32_t*)c->d_w[3], c->d_w[0],
                         c->d_w[1], c->d_err);
      first = false;
    }
    cudaError_t e2 = cudaStreamEndCapture(c->s, &g);
    if (err == cudaSuccess) err = e2;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&c->g_bu, g, 0);
    if (g) cudaGraphDestroy(g);
    if (err != cudaSuccess) {
      c->g_bu = nullptr;
      return cuda_status(err, "bottom-up graph");
    }
  }
  BF_CUDA(cudaGraphLaunch(c->g_bu, c->s));
  return BF_OK;
}

bf_status h2d(bf_cch* c, uint32_t* d, const uint32_t* h, uint64_t count) {
  if (count) BF_CUDA(cudaMemcpyAsync(d, h, count * 4, cudaMemcpyHostToDevice, c->s));
  return BF_OK;
}
bf_status d2h(bf_cch* c, uint32_t* h, const uint32_t* d, uint64_t count) {
  if (count) BF_CUDA(cudaMemcpyAsync(h, d, count * 4, cudaMemcpyDeviceToHost, c->s));
  return BF_OK;
}

unsigned egrid(uint64_t n) { return grid_for(n, 256); }

// Pair slots from reference-layout weights (hi) and middles or lengths (lo).
bf_status scatter_all(bf_cch* c, const uint32_t* hu, const uint32_t* lu, const uint32_t* hd,
                      const uint32_t* ld, bool seeds) {
  if (c->npair)
    k_pack_pairs<<<egrid(c->npair), 256, 0, c->s>>>(c->npair, c->d_pair_up, c->d_pair_dn, hu, lu,
                                                    seeds ? c->d_us : nullptr, hd, ld,
                                                    seeds ? c->d_ds : nullptr, c->d_sl);
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

// Weights into d_w[0], d_w[1] and middles into d_w[2], d_w[3].
bf_status gather_all(bf_cch* c, const uint32_t* elected) {
  if (c->nu)
    k_gather<<<egrid(c->nu), 256, 0, c->s>>>(c->nu, c->d_up_pair, 0, c->d_sl, c->d_w[0],
                                             c->d_w[2], elected);
  if (c->nd)
    k_gather<<<egrid(c->nd), 256, 0, c->s>>>(c->nd, c->d_dn_pair, 1, c->d_sl, c->d_w[1],
                                             c->d_w[3], elected);
  BF_CUDA(cudaGetLastError());
  return BF_OK;
}

bf_status download_all(bf_cch* c, uint32_t* up_w, uint32_t* down_w, uint32_t* up_mid,
                       uint32_t* down_mid) {
  bf_status rc;
  if ((rc = d2h(c, up_w, c->d_w[0], c->nu)) || (rc = d2h(c, down_w, c->d_w[1], c->nd)) ||
      (rc = d2h(c, up_mid, c->d_w[2], c->nu)) || (rc = d2h(c, down_mid, c->d_w[3], c->nd)))
    return rc;
  return BF_OK;
}

bf_status finish(bf_cch* c, std::chrono::steady_clock::time_point t0) {
  BF_CUDA(cudaStreamSynchronize(c->s));
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_device_ms = ms;
  c->last_total_ms = (float)std::chrono::duration<double, std::milli>(
                         std::chrono::steady_clock::now() - t0)
                         .count();
  return BF_OK;
}

}  // namespace

extern "C" {

bf_status bf_cch_create(const bf_cch_topo* t, int device, bf_cch** out) {
  if (out) *out = nullptr;
  if (!t || !out || !t->up_offsets || !t->down_offsets || t->n_nodes == 0) {
    set_error("bf_cch_create: null argument or empty topology");
    return BF_ERR_INVALID;
  }
  if (t->flags & ~BF_CCH_SEARCH_TARGETS) {
    set_error("bf_cch_create: unknown flags");
    return BF_ERR_INVALID;
  }
  const uint32_t n = t->n_nodes;
  const uint64_t nu = t->up_offsets[n], nd = t->down_offsets[n];
  if ((nu && !t->up_targets) || (nd && !t->down_targets)) {
    set_error("bf_cch_create: target arrays missing");
    return BF_ERR_INVALID;
  }
  if (nu >= DIR_DOWN || nd >= DIR_DOWN) {
    set_error("bf_cch_create: more than 2^31 - 1 edges in one direction");
    return BF_ERR_INVALID;
  }
  if (!valid_csr(n, t->up_offsets, t->up_targets, true) ||
      !valid_csr(n, t->down_offsets, t->down_targets, false)) {
    set_error("bf_cch_create: UP targets must ascend above their node, DOWN targets below it");
    return BF_ERR_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device");
    return BF_ERR_DEVICE;
  }
  if (device < 0 || device >= ndev) {
    set_error("bf_cch_create: device ordinal out of range");
    return BF_ERR_INVALID;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaGetDeviceProperties failed");
    return BF_ERR_DEVICE;
  }
  if (prop.major != 10 || prop.minor != 3) {
    set_error(std::string("this library is built for sm_103 (GB300); device is ") + prop.name);
    return BF_ERR_DEVICE;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaSetDevice failed");
    return BF_ERR_DEVICE;
  }
  bf_cch* c = new (std::nothrow) bf_cch();
  if (!c) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  c->device = device;
  const auto t0 = std::chrono::steady_clock::now();
  bf_status rc = BF_OK;
  if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess)
    rc = cuda_status(cudaGetLastError(), "stream/event");
  try {
    if (rc == BF_OK) rc = build_plan(c, t);
  } catch (const std::bad_alloc&) {
    set_error("out of host memory");
    rc = BF_ERR_OOM;
  }
  if (rc != BF_OK) {
    free_plan(c);
    delete c;
    return rc;
  }
  c->plan_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  *out = c;
  return BF_OK;
}

void bf_cch_destroy(bf_cch* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->s);
  free_plan(c);
  delete c;
}

bf_status bf_cch_info(const bf_cch* c, bf_cch_stats* info) {
  if (!c || !info) {
    set_error("bf_cch_info: null argument");
    return BF_ERR_INVALID;
  }
  info->n_nodes = c->n;
  info->levels = c->levels;
  info->up_edges = c->nu;
  info->down_edges = c->nd;
  info->apexes = c->napex;
  info->etree_levels = c->etree_levels ? 1 : 0;
  info->target_index = c->d_tidx ? 1 : 0;
  info->pairs = (uint32_t)c->npair;
  info->triangles = 2 * c->ncand;
  info->bottom_up_shortcuts = c->lv_bu.empty() ? 0 : c->lv_bu.back();
  info->plan_ms = c->plan_ms;
  info->last_device_ms = c->last_device_ms;
  info->last_total_ms = c->last_total_ms;
  return BF_OK;
}

bf_status bf_cch_relax(bf_cch* c, uint32_t* up_w, uint32_t* down_w, uint32_t* up_mid,
                       uint32_t* down_mid) {
  if (!c || (c->nu && (!up_w || !up_mid)) || (c->nd && (!down_w || !down_mid))) {
    set_error("bf_cch_relax: null argument");
    return BF_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  bf_status rc;
  if ((rc = h2d(c, c->d_w[0], up_w, c->nu)) || (rc = h2d(c, c->d_w[1], down_w, c->nd)) ||
      (rc = h2d(c, c->d_w[2], up_mid, c->nu)) || (rc = h2d(c, c->d_w[3], down_mid, c->nd)))
    return rc;
  BF_CUDA(cudaEventRecord(c->ev0, c->s));
  if ((rc = scatter_all(c, c->d_w[0], c->d_w[2], c->d_w[1], c->d_w[3], false)) ||
      (rc = run_relax(c, false)) || (rc = gather_all(c, nullptr)))
    return rc;
  BF_CUDA(cudaEventRecord(c->ev1, c->s));
  if ((rc = download_all(c, up_w, down_w, up_mid, down_mid))) return rc;
  return finish(c, t0);
}

bf_status bf_cch_customize(bf_cch* c, const uint32_t* orig_up, const uint32_t* orig_down,
                           uint32_t* up_w, uint32_t* down_w, uint32_t* up_mid,
                           uint32_t* down_mid) {
  if (!c || (c->nu && (!orig_up || !up_w || !up_mid)) ||
      (c->nd && (!orig_down || !down_w || !down_mid))) {
    set_error("bf_cch_customize: null argument");
    return BF_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  bf_status rc;
  if ((rc = h2d(c, c->d_l[0], orig_up, c->nu)) || (rc = h2d(c, c->d_l[1], orig_down, c->nd)))
    return rc;
  BF_CUDA(cudaEventRecord(c->ev0, c->s));
  if ((rc = scatter_all(c, c->d_l[0], c->d_mu0, c->d_l[1], c->d_md0, true)) ||
      (rc = run_relax(c, false)) || (rc = gather_all(c, nullptr)))
    return rc;
  BF_CUDA(cudaEventRecord(c->ev1, c->s));
  if ((rc = download_all(c, up_w, down_w, up_mid, down_mid))) return rc;
  return finish(c, t0);
}

bf_status bf_cch_relax_lex(bf_cch* c, uint32_t* up_t, uint32_t* down_t, const uint32_t* up_len,
                           const uint32_t* down_len, uint32_t* up_mid, uint32_t* down_mid) {
  if (!c || (c->nu && (!up_t || !up_len || !up_mid)) ||
      (c->nd && (!down_t || !down_len || !down_mid))) {
    set_error("bf_cch_relax_lex: null argument");
    return BF_ERR_INVALID;
  }
  if ((c->nu && !c->d_us) || (c->nd && !c->d_ds)) {
    set_error("bf_cch_relax_lex: the topology was created without shortcut flags");
    return BF_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  if (!c->d_elect && c->npair)
    BF_CUDA(cudaMalloc(&c->d_elect, c->npair * 2 * sizeof(uint32_t)));
  const auto t0 = std::chrono::steady_clock::now();
  bf_status rc;
  if ((rc = h2d(c, c->d_w[0], up_t, c->nu)) || (rc = h2d(c, c->d_w[1], down_t, c->nd)) ||
      (rc = h2d(c, c->d_l[0], up_len, c->nu)) || (rc = h2d(c, c->d_l[1], down_len, c->nd)) ||
      (rc = h2d(c, c->d_w[2], up_mid, c->nu)) || (rc = h2d(c, c->d_w[3], down_mid, c->nd)))
    return rc;
  BF_CUDA(cudaEventRecord(c->ev0, c->s));
  if ((rc = scatter_all(c, c->d_w[0], c->d_l[0], c->d_w[1], c->d_l[1], false)) ||
      (rc = run_relax(c, true)))
    return rc;
  if (c->npair) BF_CUDA(cudaMemsetAsync(c->d_elect, 0xFF, c->npair * 2 * sizeof(uint32_t), c->s));
  if (c->ncand) {
    const unsigned blocks = (unsigned)c->lv_blk.back();
    if (c->d_tidx)
      k_recover<true><<<blocks, RT, 0, c->s>>>(c->dev(), c->d_blk, c->d_tidx, c->d_sl, c->d_elect);
    else
      k_recover<false><<<blocks, RT, 0, c->s>>>(c->dev(), c->d_blk, nullptr, c->d_sl, c->d_elect);
    BF_CUDA(cudaGetLastError());
  }
  if ((rc = gather_all(c, c->d_elect))) return rc;
  BF_CUDA(cudaEventRecord(c->ev1, c->s));
  if ((rc = download_all(c, up_t, down_t, up_mid, down_mid))) return rc;
  return finish(c, t0);
}

bf_status bf_cch_bottom_up(bf_cch* c, const uint32_t* orig_up, const uint32_t* orig_down,
                           const uint32_t* up_mid, const uint32_t* down_mid, uint32_t* up_w,
                           uint32_t* down_w) {
  if (!c || (c->nu && (!orig_up || !up_w)) || (c->nd && (!orig_down || !down_w))) {
    set_error("bf_cch_bottom_up: null argument");
    return BF_ERR_INVALID;
  }
  const bool any_short = c->d_us || c->d_ds;
  if (any_short && ((c->nu && !up_mid && !c->d_mu0) || (c->nd && !down_mid && !c->d_md0))) {
    set_error("bf_cch_bottom_up: shortcut middles missing (none given, none in the topology)");
    return BF_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  bf_status rc;
  if ((rc = h2d(c, c->d_l[0], orig_up, c->nu)) || (rc = h2d(c, c->d_l[1], orig_down, c->nd)))
    return rc;
  // middles staged in d_w[2], d_w[3] (the captured graph reads them there)
  if (up_mid) {
    if ((rc = h2d(c, c->d_w[2], up_mid, c->nu))) return rc;
  } else if (c->nu && c->d_mu0) {
    BF_CUDA(cudaMemcpyAsync(c->d_w[2], c->d_mu0, c->nu * 4, cudaMemcpyDeviceToDevice, c->s));
  }
  if (down_mid) {
    if ((rc = h2d(c, c->d_w[3], down_mid, c->nd))) return rc;
  } else if (c->nd && c->d_md0) {
    BF_CUDA(cudaMemcpyAsync(c->d_w[3], c->d_md0, c->nd * 4, cudaMemcpyDeviceToDevice, c->s));
  }
  BF_CUDA(cudaMemsetAsync(c->d_err, 0, 4, c->s));
  BF_CUDA(cudaEventRecord(c->ev0, c->s));
  if (c->nu) k_bu_orig<<<egrid(c->nu), 256, 0, c->s>>>(c->nu, c->d_l[0], c->d_us, c->d_w[0]);
  if (c->nd) k_bu_orig<<<egrid(c->nd), 256, 0, c->s>>>(c->nd, c->d_l[1], c->d_ds, c->d_w[1]);
  BF_CUDA(cudaGetLastError());
  if (any_short && (rc = run_bottom_up(c))) return rc;
  BF_CUDA(cudaEventRecord(c->ev1, c->s));
  uint32_t err = 0;
  BF_CUDA(cudaMemcpyAsync(&err, c->d_err, 4, cudaMemcpyDeviceToHost, c->s));
  if ((rc = d2h(c, up_w, c->d_w[0], c->nu)) || (rc = d2h(c, down_w, c->d_w[1], c->nd))) return rc;
  if ((rc = finish(c, t0))) return rc;
  if (err) {
    set_error("bf_cch_bottom_up: a shortcut's middle is not a rank");
    return BF_ERR_INVALID;
  }
  return BF_OK;
}

}  // extern "C"
