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
// height (every lower neighbour of a node sits in its subtree, so heights
// strictly increase along every edge, which the plan verifies), and a level
// pushes the candidates of all its apexes. Middles, tie-breaks and saturating
// sums therefore match the reference bit for bit, from any seeds.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "engine.cuh"

using namespace bf;

namespace {

constexpr int RT = 256;      // threads per relaxation block
constexpr int RI = 4;        // candidates per thread
constexpr int RC = RT * RI;  // candidates per block
constexpr uint32_t DIR_DOWN = 0x80000000u;

// Device view of a plan.
struct PlanDev {
  uint32_t n;
  const uint64_t* uo;    // UP CSR offsets [n + 1]
  const uint32_t* ut;    // UP targets
  const uint64_t* dof;   // DOWN CSR offsets [n + 1]
  const uint32_t* dt;    // DOWN targets
  const uint64_t* ro;    // reverse DOWN offsets [n + 1]: DOWN edges x -> m per m
  const uint32_t* rs;    //   their sources x (ascending)
  const uint32_t* re;    //   their DOWN edge ids
  const uint32_t* apex;  // apexes (>= 1 candidate) in level order
  const uint64_t* cpre;  // candidate prefix over `apex` [napex + 1]
};

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Index of edge u -> v in a CSR with targets ascending per node
// (find_edge_index, customization.rs:1507-1521), or ~0 when absent.
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
__device__ __forceinline__ bool candidate(uint64_t pxm, uint64_t pmy, uint32_t m, uint64_t* out) {
  const uint32_t a = (uint32_t)(pxm >> 32), b = (uint32_t)(pmy >> 32);
  if (a == INF || b == INF) return false;
  const uint32_t lo = LEX ? sat_add((uint32_t)pxm, (uint32_t)pmy) : m;
  *out = ((uint64_t)sat_add(a, b) << 32) | lo;
  return true;
}

// One block of RC consecutive candidates of a level, computed when the plan
// is built: its first candidate, the apexes [k0, k0 + na) it touches and its
// candidate count.
struct Blk {
  uint64_t cb;
  uint32_t k0;
  uint16_t na;
  uint16_t cnt;
};

// Block-level load-balanced search: the apexes of the block's candidates are
// staged in shared memory (prefix relative to the block's first apex, UP
// offset, UP count, reverse-DOWN offset, rank). Edge ids fit 31 bits.
struct Stage {
  uint32_t pre[RC + 1];
  uint32_t uoff[RC];
  uint32_t roff[RC];
  uint32_t m[RC];
  uint32_t nu[RC];
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
    const uint64_t u0 = __ldg(p.uo + m);
    st.m[i] = m;
    st.uoff[i] = (uint32_t)u0;
    st.nu[i] = (uint32_t)(__ldg(p.uo + m + 1) - u0);
    st.roff[i] = (uint32_t)__ldg(p.ro + m);
  }
  __syncthreads();
  return d;
}

// Locates the candidate at offset q from the block's first apex: local apex
// index k and the (reverse-DOWN entry, UP edge) pair it denotes.
__device__ __forceinline__ void locate(const Stage& st, uint32_t na, uint32_t q, uint32_t* k,
                                       uint32_t* ir, uint32_t* ey) {
  uint32_t lo = 0, hi = na;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (st.pre[mid] <= q)
      lo = mid;
    else
      hi = mid;
  }
  const uint32_t r = q - st.pre[lo];
  const uint32_t nu = st.nu[lo];
  const uint32_t i = r / nu;
  *k = lo;
  *ir = st.roff[lo] + i;
  *ey = st.uoff[lo] + (r - i * nu);
}

constexpr uint32_t NO_TARGET = 0xFFFFFFFFu;

// Target edge of a candidate as an edge id with DIR_DOWN set for a DOWN
// edge, NO_TARGET when y == x or the edge is absent; read from the plan's
// precomputed index or searched in x's list.
template <bool TIDX>
__device__ __forceinline__ uint32_t target_of(const PlanDev& p, const uint32_t* __restrict__ tidx,
                                              uint64_t c, uint32_t ir, uint32_t ey) {
  if (TIDX) return __ldcs(tidx + c);  // read once per call: streaming
  const uint32_t x = __ldg(p.rs + ir);
  const uint32_t y = __ldg(p.ut + ey);
  if (y == x) return NO_TARGET;
  if (y > x) {
    const uint64_t e = find_edge(p.uo, p.ut, x, y);
    return e == ~0ull ? NO_TARGET : (uint32_t)e;
  }
  const uint64_t e = find_edge(p.dof, p.dt, x, y);
  return e == ~0ull ? NO_TARGET : ((uint32_t)e | DIR_DOWN);
}

// The target index of every candidate, once per plan.
__global__ void __launch_bounds__(RT) k_tidx(PlanDev p, const Blk* __restrict__ blk,
                                             uint32_t* __restrict__ tidx) {
  __shared__ Stage st;
  const Blk d = stage_block(p, blk, blockIdx.x, st);
  const uint32_t q0 = (uint32_t)(d.cb - __ldg(p.cpre + d.k0));
  for (uint32_t r = threadIdx.x; r < d.cnt; r += RT) {
    uint32_t k, ir, ey;
    locate(st, d.na, q0 + r, &k, &ir, &ey);
    tidx[d.cb + r] = target_of<false>(p, nullptr, 0, ir, ey);
  }
}

// One level of the relaxation: every candidate of the level's blocks is
// offered to its target edge with a 64-bit atomicMin on the packed value. A
// fresh L2 read first drops candidates that cannot win (values only
// decrease, so the read is an upper bound). Everything that depends on the
// plan alone (apex staging, target edge, DOWN leg id) is fetched before the
// wait on the previous level; after it, each candidate issues its three
// state loads at once, for all of the thread's candidates together.
template <bool LEX, bool TIDX>
__global__ void __launch_bounds__(RT) k_relax(PlanDev p, const Blk* __restrict__ blk, uint64_t b0,
                                              const uint32_t* __restrict__ tidx,
                                              uint64_t* __restrict__ pu,
                                              uint64_t* __restrict__ pd) {
  __shared__ Stage st;
  const Blk d = stage_block(p, blk, b0 + blockIdx.x, st);
  pdl_launch();
  const uint32_t q0 = (uint32_t)(d.cb - __ldg(p.cpre + d.k0));
  uint32_t tg[RI], lx[RI], ly[RI], am[RI];
#pragma unroll
  for (int i = 0; i < RI; ++i) {
    const uint32_t r = threadIdx.x + i * RT;
    tg[i] = NO_TARGET;
    if (r < d.cnt) {
      uint32_t k, ir, ey;
      locate(st, d.na, q0 + r, &k, &ir, &ey);
      tg[i] = target_of<TIDX>(p, tidx, d.cb + r, ir, ey);
      lx[i] = __ldg(p.re + ir);
      ly[i] = ey;
      am[i] = st.m[k];
    }
  }
  pdl_wait();
  uint64_t a[RI], b[RI], cur[RI];
#pragma unroll
  for (int i = 0; i < RI; ++i) {
    if (tg[i] == NO_TARGET) continue;
    a[i] = __ldcg(pd + lx[i]);
    b[i] = __ldcg(pu + ly[i]);
    cur[i] = __ldcg((tg[i] & DIR_DOWN ? pd : pu) + (tg[i] & ~DIR_DOWN));
  }
#pragma unroll
  for (int i = 0; i < RI; ++i) {
    if (tg[i] == NO_TARGET) continue;
    uint64_t cand;
    if (!candidate<LEX>(a[i], b[i], am[i], &cand) || !(cand < cur[i])) continue;
    atomicMin((unsigned long long*)((tg[i] & DIR_DOWN ? pd : pu) + (tg[i] & ~DIR_DOWN)),
              (unsigned long long)cand);
  }
}

// Middle election of the lexicographic relaxation on converged values
// (customization.rs:1340-1400): the smallest apex whose candidate equals a
// SHORTCUT edge's packed value.
template <bool TIDX>
__global__ void __launch_bounds__(RT) k_recover(PlanDev p, const Blk* __restrict__ blk,
                                                const uint32_t* __restrict__ tidx,
                                                const uint64_t* __restrict__ pu,
                                                const uint64_t* __restrict__ pd,
                                                const uint8_t* __restrict__ us,
                                                const uint8_t* __restrict__ ds,
                                                uint32_t* __restrict__ mu,
                                                uint32_t* __restrict__ md) {
  __shared__ Stage st;
  const Blk d = stage_block(p, blk, blockIdx.x, st);
  const uint32_t q0 = (uint32_t)(d.cb - __ldg(p.cpre + d.k0));
  for (uint32_t r = threadIdx.x; r < d.cnt; r += RT) {
    uint32_t k, ir, ey;
    locate(st, d.na, q0 + r, &k, &ir, &ey);
    const uint32_t t = target_of<TIDX>(p, tidx, d.cb + r, ir, ey);
    if (t == NO_TARGET) continue;
    const bool down = t & DIR_DOWN;
    const uint32_t e = t & ~DIR_DOWN;
    if (!(down ? ds[e] : us[e])) continue;
    uint64_t cand;
    if (!candidate<true>(__ldg(pd + __ldg(p.re + ir)), __ldg(pu + ey), 0, &cand)) continue;
    if (__ldg((down ? pd : pu) + e) != cand) continue;
    atomicMin((down ? md : mu) + e, st.m[k]);
  }
}

__global__ void k_pack(uint64_t n, const uint32_t* __restrict__ hi, const uint32_t* __restrict__ lo,
                       uint64_t* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = ((uint64_t)hi[i] << 32) | lo[i];
}

// Unpacks weights; middles from the packed low word (relax) or from the
// election with the given middle as fallback (lexicographic).
__global__ void k_unpack(uint64_t n, const uint64_t* __restrict__ packed, uint32_t* __restrict__ w,
                         uint32_t* __restrict__ mid, const uint32_t* __restrict__ elected) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = packed[i];
    w[i] = (uint32_t)(v >> 32);
    if (!elected)
      mid[i] = (uint32_t)v;
    else if (elected[i] != INF)
      mid[i] = elected[i];
  }
}

// Seeds of a full customization (bottom_up_customize + relaxation): the
// original weight on an original edge, u32::MAX on a shortcut (its bottom-up
// value is dominated by the triangle through its contraction middle, so the
// fixed point is the same), packed with the topology's middle.
__global__ void k_seed(uint64_t n, const uint32_t* __restrict__ orig,
                       const uint8_t* __restrict__ is_short, const uint32_t* __restrict__ mid,
                       uint64_t* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t w = (is_short && is_short[i]) ? INF : orig[i];
    out[i] = ((uint64_t)w << 32) | (mid ? mid[i] : INF);
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
  uint64_t nu = 0, nd = 0;
  cudaStream_t s = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // device topology and plan
  uint64_t *d_uo = nullptr, *d_do = nullptr, *d_ro = nullptr, *d_cpre = nullptr;
  uint32_t *d_ut = nullptr, *d_dt = nullptr, *d_rs = nullptr, *d_re = nullptr, *d_apex = nullptr;
  uint8_t *d_us = nullptr, *d_ds = nullptr;  // shortcut flags (null: none given)
  uint32_t *d_mu0 = nullptr, *d_md0 = nullptr;  // topology middles (null: all u32::MAX)
  uint32_t *d_btail = nullptr, *d_bedge = nullptr;  // bottom-up lists by level
  Blk* d_blk = nullptr;                               // relaxation blocks, level after level
  uint32_t* d_tidx = nullptr;                         // target edge per candidate (or null)
  std::vector<uint64_t> lv_blk;                       // [levels + 1] first block per level
  // relaxation levels: apex ranges and candidate ranges
  std::vector<uint32_t> lv_apex;   // [levels + 1]
  std::vector<uint64_t> lv_cand;   // [levels + 1]
  std::vector<uint64_t> lv_bu;     // [levels + 1] bottom-up entries per level
  uint32_t napex = 0;
  uint64_t ncand = 0;
  // working state
  uint64_t *d_pu = nullptr, *d_pd = nullptr;
  uint32_t *d_w[4] = {nullptr, nullptr, nullptr, nullptr};  // up/down weight, up/down middle
  uint32_t *d_l[2] = {nullptr, nullptr};                    // up/down length or original
  uint32_t* d_err = nullptr;
  cudaGraphExec_t g_relax[2] = {nullptr, nullptr};  // plain, lexicographic
  cudaGraphExec_t g_bu = nullptr;
  double plan_ms = 0;
  uint32_t levels = 0;
  bool etree_levels = true;
  float last_device_ms = 0, last_total_ms = 0;

  PlanDev dev() const {
    return PlanDev{n, d_uo, d_ut, d_do, d_dt, d_ro, d_rs, d_re, d_apex, d_cpre};
  }
};

namespace {

void free_plan(bf_cch* c) {
  for (auto& g : c->g_relax)
    if (g) cudaGraphExecDestroy(g);
  if (c->g_bu) cudaGraphExecDestroy(c->g_bu);
  void* ptrs[] = {c->d_uo, c->d_do, c->d_ro, c->d_cpre, c->d_ut, c->d_dt, c->d_rs, c->d_re,
                  c->d_apex, c->d_us, c->d_ds, c->d_mu0, c->d_md0, c->d_btail, c->d_bedge, c->d_blk, c->d_tidx,
                  c->d_pu, c->d_pd, c->d_w[0], c->d_w[1], c->d_w[2], c->d_w[3], c->d_l[0],
                  c->d_l[1], c->d_err};
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
  // Levels: elimination-tree heights (parent = lowest upper neighbour); kept
  // when they increase strictly along every edge, else longest-path levels.
  std::vector<uint32_t> lev(n, 0);
  for (uint32_t m = 0; m < n; ++m) {
    uint32_t par = INF;
    if (t->up_offsets[m + 1] > t->up_offsets[m]) par = t->up_targets[t->up_offsets[m]];
    if (ro[m + 1] > ro[m]) par = std::min(par, rs[ro[m]]);
    if (par != INF) lev[par] = std::max(lev[par], lev[m] + 1);
  }
  bool ok = true;
  for (uint32_t u = 0; u < n && ok; ++u) {
    for (uint64_t i = t->up_offsets[u]; i < t->up_offsets[u + 1]; ++i)
      if (lev[t->up_targets[i]] <= lev[u]) ok = false;
    for (uint64_t i = t->down_offsets[u]; i < t->down_offsets[u + 1]; ++i)
      if (lev[u] <= lev[t->down_targets[i]]) ok = false;
  }
  c->etree_levels = ok;
  if (!ok) {
    std::fill(lev.begin(), lev.end(), 0);
    for (uint32_t m = 0; m < n; ++m) {
      for (uint64_t i = t->up_offsets[m]; i < t->up_offsets[m + 1]; ++i)
        lev[t->up_targets[i]] = std::max(lev[t->up_targets[i]], lev[m] + 1);
      for (uint64_t i = ro[m]; i < ro[m + 1]; ++i) lev[rs[i]] = std::max(lev[rs[i]], lev[m] + 1);
    }
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
  // apexes with at least one candidate, and the candidate prefix
  std::vector<uint32_t> apex;
  std::vector<uint64_t> cpre(1, 0);
  c->lv_apex.assign((size_t)L + 1, 0);
  c->lv_cand.assign((size_t)L + 1, 0);
  for (uint32_t l = 0; l < L; ++l) {
    for (uint32_t i = loff[l]; i < loff[l + 1]; ++i) {
      const uint32_t m = order[i];
      const uint64_t k = (ro[m + 1] - ro[m]) * (t->up_offsets[m + 1] - t->up_offsets[m]);
      if (!k) continue;
      if (k >= (1ull << 30)) {
        set_error("bf_cch_create: a node has 2^30 or more triangles");
        return BF_ERR_INVALID;
      }
      apex.push_back(m);
      cpre.push_back(cpre.back() + k);
    }
    c->lv_apex[l + 1] = (uint32_t)apex.size();
    c->lv_cand[l + 1] = cpre.back();
  }
  c->napex = (uint32_t)apex.size();
  c->ncand = cpre.back();
  // relaxation blocks: RC consecutive candidates of one level each
  std::vector<Blk> blks;
  c->lv_blk.assign((size_t)L + 1, 0);
  for (uint32_t l = 0; l < L; ++l) {
    uint32_t k = c->lv_apex[l];
    const uint32_t a1 = c->lv_apex[l + 1];
    for (uint64_t cb = c->lv_cand[l]; cb < c->lv_cand[l + 1]; cb += RC) {
      const uint64_t ce = std::min<uint64_t>(cb + RC, c->lv_cand[l + 1]);
      while (k + 1 < a1 && cpre[k + 1] <= cb) ++k;
      uint32_t k1 = k;
      while (k1 + 1 < a1 && cpre[k1 + 1] < ce) ++k1;
      blks.push_back(Blk{cb, k, (uint16_t)(k1 - k + 1), (uint16_t)(ce - cb)});
    }
    c->lv_blk[l + 1] = blks.size();
  }
  // bottom-up lists: shortcuts by the level of their lower endpoint
  std::vector<uint32_t> btail, bedge;
  c->lv_bu.assign((size_t)L + 1, 0);
  if (t->up_is_shortcut || t->down_is_shortcut) {
    for (uint32_t l = 0; l < L; ++l) {
      for (uint32_t i = loff[l]; i < loff[l + 1]; ++i) {
        const uint32_t j = order[i];
        if (t->up_is_shortcut)
          for (uint64_t e = t->up_offsets[j]; e < t->up_offsets[j + 1]; ++e)
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
  BF_CUDA(upload(&c->d_uo, t->up_offsets, (uint64_t)n + 1));
  BF_CUDA(upload(&c->d_do, t->down_offsets, (uint64_t)n + 1));
  BF_CUDA(upload(&c->d_ut, t->up_targets, nu));
  BF_CUDA(upload(&c->d_dt, t->down_targets, nd));
  BF_CUDA(upload(&c->d_ro, ro.data(), (uint64_t)n + 1));
  BF_CUDA(upload(&c->d_rs, rs.data(), nd));
  BF_CUDA(upload(&c->d_re, re.data(), nd));
  BF_CUDA(upload(&c->d_apex, apex.data(), apex.size()));
  BF_CUDA(upload(&c->d_cpre, cpre.data(), cpre.size()));
  if (t->up_is_shortcut) BF_CUDA(upload(&c->d_us, t->up_is_shortcut, nu));
  if (t->down_is_shortcut) BF_CUDA(upload(&c->d_ds, t->down_is_shortcut, nd));
  if (t->up_middle) BF_CUDA(upload(&c->d_mu0, t->up_middle, nu));
  if (t->down_middle) BF_CUDA(upload(&c->d_md0, t->down_middle, nd));
  BF_CUDA(upload(&c->d_btail, btail.data(), btail.size()));
  BF_CUDA(upload(&c->d_blk, blks.data(), blks.size()));
  BF_CUDA(upload(&c->d_bedge, bedge.data(), bedge.size()));
  const uint64_t nmax = std::max<uint64_t>(1, std::max(nu, nd));
  BF_CUDA(cudaMalloc(&c->d_pu, std::max<uint64_t>(1, nu) * 8));
  BF_CUDA(cudaMalloc(&c->d_pd, std::max<uint64_t>(1, nd) * 8));
  for (int i = 0; i < 4; ++i) BF_CUDA(cudaMalloc(&c->d_w[i], nmax * 4));
  for (int i = 0; i < 2; ++i) BF_CUDA(cudaMalloc(&c->d_l[i], nmax * 4));
  BF_CUDA(cudaMalloc(&c->d_err, 4));
  // target index: 4 bytes per candidate while that fits a quarter of free HBM
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
    for (size_t l = 0; l + 1 < c->lv_blk.size() && err == cudaSuccess; ++l) {
      const uint64_t b0 = c->lv_blk[l], b1 = c->lv_blk[l + 1];
      if (b1 == b0) continue;
      const Blk* blk = c->d_blk;
      const uint32_t* ti = c->d_tidx;
      const dim3 grid((unsigned)(b1 - b0));
      if (ti)
        err = lex ? launch_level(k_relax<true, true>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_pu, c->d_pd)
                  : launch_level(k_relax<false, true>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_pu, c->d_pd);
      else
        err = lex ? launch_level(k_relax<true, false>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_pu, c->d_pd)
                  : launch_level(k_relax<false, false>, grid, RT, !first, c->s, p, blk, b0, ti,
                                 c->d_pu, c->d_pd);
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

bf_status run_bottom_up(bf_cch* c, const uint32_t* d_mu, const uint32_t* d_md) {
  const PlanDev p = c->dev();
  // the graph bakes the middle pointers in; they are always the plan's staging buffers
  if (!c->g_bu) {
    cudaGraph_t g = nullptr;
    BF_CUDA(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    bool first = true;
    for (size_t l = 0; l + 1 < c->lv_bu.size() && err == cudaSuccess; ++l) {
      const uint64_t b0 = c->lv_bu[l], b1 = c->lv_bu[l + 1];
      if (b1 == b0) continue;
      err = launch_level(k_bu_level, dim3((unsigned)((b1 - b0 + 255) / 256)), 256, !first, c->s, p,
                         b0, b1, (const uint32_t*)c->d_btail, (const uint32_t*)c->d_bedge, d_mu,
                         d_md, c->d_w[0], c->d_w[1], c->d_err);
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

unsigned pack_grid(uint64_t n) { return grid_for(n, 256); }

bf_status finish(bf_cch* c, std::chrono::steady_clock::time_point t0) {
  BF_CUDA(cudaStreamSynchronize(c->s));
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_device_ms = ms;
  c->last_total_ms =
      (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
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
  info->triangles = c->ncand;
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
  if (c->nu) k_pack<<<pack_grid(c->nu), 256, 0, c->s>>>(c->nu, c->d_w[0], c->d_w[2], c->d_pu);
  if (c->nd) k_pack<<<pack_grid(c->nd), 256, 0, c->s>>>(c->nd, c->d_w[1], c->d_w[3], c->d_pd);
  if ((rc = run_relax(c, false))) return rc;
  if (c->nu) k_unpack<<<pack_grid(c->nu), 256, 0, c->s>>>(c->nu, c->d_pu, c->d_w[0], c->d_w[2], nullptr);
  if (c->nd) k_unpack<<<pack_grid(c->nd), 256, 0, c->s>>>(c->nd, c->d_pd, c->d_w[1], c->d_w[3], nullptr);
  BF_CUDA(cudaEventRecord(c->ev1, c->s));
  if ((rc = d2h(c, up_w, c->d_w[0], c->nu)) || (rc = d2h(c, down_w, c->d_w[1], c->nd)) ||
      (rc = d2h(c, up_mid, c->d_w[2], c->nu)) || (rc = d2h(c, down_mid, c->d_w[3], c->nd)))
    return rc;
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
  if (c->nu) k_seed<<<pack_grid(c->nu), 256, 0, c->s>>>(c->nu, c->d_l[0], c->d_us, c->d_mu0, c->d_pu);
  if (c->nd) k_seed<<<pack_grid(c->nd), 256, 0, c->s>>>(c->nd, c->d_l[1], c->d_ds, c->d_md0, c->d_pd);
  if ((rc = run_relax(c, false))) return rc;
  if (c->nu) k_unpack<<<pack_grid(c->nu), 256, 0, c->s>>>(c->nu, c->d_pu, c->d_w[0], c->d_w[2], nullptr);
  if (c->nd) k_unpack<<<pack_grid(c->nd), 256, 0, c->s>>>(c->nd, c->d_pd, c->d_w[1], c->d_w[3], nullptr);
  BF_CUDA(cudaEventRecord(c->ev1, c->s));
  if ((rc = d2h(c, up_w, c->d_w[0], c->nu)) || (rc = d2h(c, down_w, c->d_w[1], c->nd)) ||
      (rc = d2h(c, up_mid, c->d_w[2], c->nu)) || (rc = d2h(c, down_mid, c->d_w[3], c->nd)))
    return rc;
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
  const auto t0 = std::chrono::steady_clock::now();
  bf_status rc;
  if ((rc = h2d(c, c->d_w[0], up_t, c->nu)) || (rc = h2d(c, c->d_w[1], down_t, c->nd)) ||
      (rc = h2d(c, c->d_l[0], up_len, c->nu)) || (rc = h2d(c, c->d_l[1], down_len, c->nd)) ||
      (rc = h2d(c, c->d_w[2], up_mid, c->nu)) || (rc = h2d(c, c->d_w[3], down_mid, c->nd)))
    return rc;
  BF_CUDA(cudaEventRecord(c->ev0, c->s));
  if (c->nu) k_pack<<<pack_grid(c->nu), 256, 0, c->s>>>(c->nu, c->d_w[0], c->d_l[0], c->d_pu);
  if (c->nd) k_pack<<<pack_grid(c->nd), 256, 0, c->s>>>(c->nd, c->d_w[1], c->d_l[1], c->d_pd);
  if ((rc = run_relax(c, true))) return rc;
  // elected middles reuse the length buffers (no longer read)
  if (c->nu) BF_CUDA(cudaMemsetAsync(c->d_l[0], 0xFF, c->nu * 4, c->s));
  if (c->nd) BF_CUDA(cudaMemsetAsync(c->d_l[1], 0xFF, c->nd * 4, c->s));
  if (c->ncand) {
    const uint64_t blocks = c->lv_blk.back();
    if (c->d_tidx)
      k_recover<true><<<(unsigned)blocks, RT, 0, c->s>>>(c->dev(), c->d_blk, c->d_tidx, c->d_pu,
                                                         c->d_pd, c->d_us, c->d_ds, c->d_l[0],
                                                         c->d_l[1]);
    else
      k_recover<false><<<(unsigned)blocks, RT, 0, c->s>>>(c->dev(), c->d_blk, nullptr, c->d_pu,
                                                          c->d_pd, c->d_us, c->d_ds, c->d_l[0],
                                                          c->d_l[1]);
    BF_CUDA(cudaGetLastError());
  }
  if (c->nu) k_unpack<<<pack_grid(c->nu), 256, 0, c->s>>>(c->nu, c->d_pu, c->d_w[0], c->d_w[2], c->d_l[0]);
  if (c->nd) k_unpack<<<pack_grid(c->nd), 256, 0, c->s>>>(c->nd, c->d_pd, c->d_w[1], c->d_w[3], c->d_l[1]);
  BF_CUDA(cudaEventRecord(c->ev1, c->s));
  if ((rc = d2h(c, up_t, c->d_w[0], c->nu)) || (rc = d2h(c, down_t, c->d_w[1], c->nd)) ||
      (rc = d2h(c, up_mid, c->d_w[2], c->nu)) || (rc = d2h(c, down_mid, c->d_w[3], c->nd)))
    return rc;
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
  const uint32_t* mu = up_mid ? up_mid : nullptr;
  const uint32_t* md = down_mid ? down_mid : nullptr;
  if (any_short && ((c->nu && !mu && !c->d_mu0) || (c->nd && !md && !c->d_md0))) {
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
  if (mu) {
    if ((rc = h2d(c, c->d_w[2], mu, c->nu))) return rc;
  } else if (c->nu && c->d_mu0) {
    BF_CUDA(cudaMemcpyAsync(c->d_w[2], c->d_mu0, c->nu * 4, cudaMemcpyDeviceToDevice, c->s));
  }
  if (md) {
    if ((rc = h2d(c, c->d_w[3], md, c->nd))) return rc;
  } else if (c->nd && c->d_md0) {
    BF_CUDA(cudaMemcpyAsync(c->d_w[3], c->d_md0, c->nd * 4, cudaMemcpyDeviceToDevice, c->s));
  }
  BF_CUDA(cudaMemsetAsync(c->d_err, 0, 4, c->s));
  BF_CUDA(cudaEventRecord(c->ev0, c->s));
  if (c->nu) k_bu_orig<<<pack_grid(c->nu), 256, 0, c->s>>>(c->nu, c->d_l[0], c->d_us, c->d_w[0]);
  if (c->nd) k_bu_orig<<<pack_grid(c->nd), 256, 0, c->s>>>(c->nd, c->d_l[1], c->d_ds, c->d_w[1]);
  if (any_short && (rc = run_bottom_up(c, c->d_w[2], c->d_w[3]))) return rc;
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
