// isochrone.cu — bulk isochrone reachable sets on the GPU.
//
// Restates the PHAST part of the reference's bulk isochrones
// (isochrone_bulk_handler, route/src/server/isochrone_handler.rs:1668-1709,
// and BatchedIsochroneEngine::query_many, route/src/range/batched_isochrone.rs:216):
// for origin i with threshold T_i the reachable set is
// {rank r : dist(origin_i, r) <= T_i}, the settled set that
// run_phast_bounded_fast_seeded (isochrone_handler.rs:338-491) returns.
//
// Origins are the lanes of a full-graph sweep (every node is a row; waves of
// as many lanes as the HBM budget allows). Distances are computed unbounded,
// which is exact, and the threshold is applied when the bitsets are emitted:
// k_bits stages a 256-rank x 32-lane tile of the slab in shared memory and
// turns each lane's 256 comparisons into eight ballot words (one 32-byte
// sector of that origin's bitset row).

#include <algorithm>
#include <cstring>

#include "engine.cuh"

namespace bf {

namespace {

constexpr uint32_t TILE_R = 256;  // ranks per tile
constexpr uint32_t TILE_L = 32;   // lanes per tile
constexpr uint32_t LANE_TILES_PER_BLOCK = 8;
// blocks of the 16-bit gated sweep per level: 16 resident 128-thread blocks
// on each of the 152 SMs
constexpr uint32_t GATED16_BLOCKS = 152 * 16;

// min of the two halfwords of *p and v, one lane per halfword, by
// compare-and-swap (there is no 16-bit atomicMin). Lock-free: a failed swap
// means another thread lowered the word; the loop is bounded all the same.
__device__ __forceinline__ void atomic_min_u16x2(uint32_t* p, uint32_t v, uint32_t* err) {
  uint32_t old = *(volatile uint32_t*)p;
  for (uint32_t guard = 0; guard < (1u << 20); ++guard) {
    const uint32_t nv = __vminu2(old, v);
    if (nv == old) return;
    const uint32_t seen = atomicCAS(p, old, nv);
    if (seen == old) return;
    old = seen;
  }
  atomicOr(err, DEVERR_TIMEOUT);
}

// Gated sweep with 16-bit lanes, for isochrone waves whose thresholds are all
// below 0xFFFF. A lane holds its distance while it is within the lane's
// threshold and 0xFFFF otherwise: a value above a threshold only leads to
// values above it, so the clamp keeps every distance within the threshold
// exact and halves the bytes of every gather and row write. A thread owns 8
// lanes (one 16-byte load per gathered row), adds with halfword saturation and
// clamps once per item. Gating as in the 32-bit form: items with no active
// source are skipped, inactive sources are not gathered, and a row becomes
// active when any lane is within its threshold.
//
// A full-graph wave has millions of small items, most of them inactive, so a
// block does not own one item: the level's items [i0, i1) are dealt out
// block-stride over a grid sized to the GPU, and a skipped item costs one
// warp ballot instead of a block launch.
// One work item of the 16-bit gated sweep for this thread's 8 lanes: every
// warp evaluates the item's in-edges 32 at a time (warp lane t holds edge
// base + t, preloaded in r0 for the first 32) and a ballot gives the edges
// whose source row is active (the same masks in every warp of the item).
// With CG, rows and activity bits are read through L2: other warps of the
// same launch may have written them. Every thread of the warp calls it.
template <bool CG>
__device__ __forceinline__ void gated16_item(const uint4 it, const uint2 r0,
                                             const uint2* __restrict__ erec,
                                             uint16_t* __restrict__ slab, uint32_t Kp,
                                             uint32_t* __restrict__ active,
                                             const uint32_t* __restrict__ thr, uint32_t lane,
                                             bool live, uint32_t valid_lanes,
                                             const uint32_t* __restrict__ seeded,
                                             uint32_t* __restrict__ err) {
  const unsigned FULL = 0xFFFFFFFFu;
  const uint32_t t = threadIdx.x & 31;
  uint4 acc = make_uint4(~0u, ~0u, ~0u, ~0u);
  bool any = false;
  for (uint32_t base = it.y; base < it.z; base += 32) {
    const uint32_t e = base + t;
    uint2 r = make_uint2(0, 0);
    bool a = false;
    if (e < it.z) {
      r = base == it.y ? r0 : erec[e];
      const uint32_t aw = CG ? __ldcg(active + (r.x >> 5)) : active[r.x >> 5];
      a = (aw >> (r.x & 31)) & 1u;
    }
    uint32_t m = __ballot_sync(FULL, a);
    any |= m != 0;
    // gather the active sources four at a time (loads in flight together)
    while (m) {
      uint32_t j[4], k = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        j[q] = m ? (uint32_t)(__ffs(m) - 1) : 0u;
        if (m) {
          m &= m - 1;
          ++k;
        }
      }
      uint32_t src[4], w[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        src[q] = __shfl_sync(FULL, r.x, j[q]);
        w[q] = __shfl_sync(FULL, r.y, j[q]);
      }
      if (live) {
        uint4 v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint4* row = reinterpret_cast<const uint4*>(slab + (size_t)src[q] * Kp + lane);
          v[q] = q < (int)k ? (CG ? __ldcg(row) : *row) : make_uint4(~0u, ~0u, ~0u, ~0u);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t w16 = min(w[q], 0xFFFFu), ww = w16 | (w16 << 16);
          acc.x = __vminu2(acc.x, __vaddus2(v[q].x, ww));
          acc.y = __vminu2(acc.y, __vaddus2(v[q].y, ww));
          acc.z = __vminu2(acc.z, __vaddus2(v[q].z, ww));
          acc.w = __vminu2(acc.w, __vaddus2(v[q].w, ww));
        }
      }
    }
  }
  if (!any) return;  // uniform across the item's warps: the row keeps its seed or INF
  // clamp each lane to its threshold
  uint32_t* aw = &acc.x;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t lo = aw[q] & 0xFFFFu, hi = aw[q] >> 16;
    if (2 * q >= (int)valid_lanes || lo > thr[lane + 2 * q]) lo = 0xFFFFu;
    if (2 * q + 1 >= (int)valid_lanes || hi > thr[lane + 2 * q + 1]) hi = 0xFFFFu;
    aw[q] = lo | (hi << 16);
  }
  if (live) {
    uint32_t* dst = reinterpret_cast<uint32_t*>(slab + (size_t)it.x * Kp + lane);
    if (it.w) {
      atomic_min_u16x2(dst + 0, acc.x, err);
      atomic_min_u16x2(dst + 1, acc.y, err);
      atomic_min_u16x2(dst + 2, acc.z, err);
      atomic_min_u16x2(dst + 3, acc.w, err);
    } else {
      // without a full slab reset only seeded rows hold valid data here
      const bool valid = (seeded[it.x >> 5] >> (it.x & 31)) & 1u;
      const uint4* d4 = reinterpret_cast<const uint4*>(dst);
      const uint4 c = valid ? (CG ? __ldcg(d4) : *d4) : make_uint4(~0u, ~0u, ~0u, ~0u);
      uint4 v;
      v.x = __vminu2(c.x, acc.x);
      v.y = __vminu2(c.y, acc.y);
      v.z = __vminu2(c.z, acc.z);
      v.w = __vminu2(c.w, acc.w);
      *reinterpret_cast<uint4*>(dst) = v;
    }
  }
  const bool act = live && (acc.x & acc.y & acc.z & acc.w) != ~0u;
  const unsigned am = __ballot_sync(FULL, act);
  if (am && t == (unsigned)(__ffs(am) - 1)) atomicOr(&active[it.x >> 5], 1u << (it.x & 31));
}

// IPB = 1: the block's warps share each item (lane slices of blockDim.x * 8
// lanes per y-block); IPB > 1 (waves of at most 256 lanes): each of the
// block's IPB warps takes its own item, so small waves keep as many items in
// flight per SM as large ones.
template <uint32_t IPB>
__global__ void __launch_bounds__(128, IPB > 1 ? 12 : 16)
    k_sweep_gated16(const uint4* __restrict__ item, uint32_t i0, uint32_t i1,
                    const uint2* __restrict__ erec, uint16_t* __restrict__ slab, uint32_t Kp,
                    uint32_t* __restrict__ active, const uint32_t* __restrict__ thr, uint32_t kw,
                    const uint32_t* __restrict__ seeded, uint32_t* __restrict__ err) {
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t t = threadIdx.x & 31;
  constexpr uint32_t ipb = IPB;
  const uint32_t lane = ipb > 1 ? t * 8 : (blockIdx.y * blockDim.x + threadIdx.x) * 8;
  const uint32_t wbase = lane - 8 * t;
  if (wbase >= Kp) return;  // the whole warp is past the last lane
  const bool live = lane < Kp;
  // lanes of this thread inside the wave (the rest clamp to 0xFFFF)
  const uint32_t valid_lanes = live ? min(8u, kw > lane ? kw - lane : 0u) : 0u;
  const uint32_t first = ipb > 1 ? blockIdx.x * ipb + (threadIdx.x >> 5) : blockIdx.x;
  const uint32_t stride = gridDim.x * ipb;
  // the first item and its edge records do not depend on the previous
  // level: load them while that level drains
  uint4 it = make_uint4(0, 0, 0, 0);
  uint2 r0 = make_uint2(0, 0);
  uint32_t ii = i0 + first;
  if (ii < i1) {
    it = item[ii];
    r0 = it.y + t < it.z ? erec[it.y + t] : make_uint2(0, 0);
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  for (; ii < i1; ii += stride) {
    if (ii != i0 + first) {
      it = item[ii];
      r0 = it.y + t < it.z ? erec[it.y + t] : make_uint2(0, 0);
    }
    gated16_item<false>(it, r0, erec, slab, Kp, active, thr, lane, live, valid_lanes, seeded, err);
  }
}

// One work item for one thread of a group of Kp / 8 threads (8 lanes each):
// the thread walks the item's in-edges four at a time (edge records,
// activity words and rows of four edges in flight together). With CG, rows
// and activity bits are read through L2 (other blocks may have written them).
template <bool CG>
__device__ __forceinline__ void group16_item(const uint4 it, const uint2* __restrict__ erec,
                                             uint16_t* __restrict__ slab, uint32_t Kp,
                                             uint32_t* __restrict__ active,
                                             const uint32_t* __restrict__ thr, uint32_t lane,
                                             bool live, uint32_t valid_lanes,
                                             const uint32_t* __restrict__ seeded,
                                             uint32_t* __restrict__ err) {
  uint4 acc = make_uint4(~0u, ~0u, ~0u, ~0u);
  bool any = false;
  for (uint32_t e0 = it.y; e0 < it.z; e0 += 4) {
    uint2 r[4];
    uint32_t aw[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) r[q] = e0 + q < it.z ? erec[e0 + q] : make_uint2(0, 0);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      aw[q] = e0 + q < it.z ? (CG ? __ldcg(active + (r[q].x >> 5)) : active[r[q].x >> 5]) : 0u;
    uint4 v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool a = (aw[q] >> (r[q].x & 31)) & 1u;
      any |= a;
      const uint4* row = reinterpret_cast<const uint4*>(slab + (size_t)r[q].x * Kp + lane);
      v[q] = a && live ? (CG ? __ldcg(row) : *row) : make_uint4(~0u, ~0u, ~0u, ~0u);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t w16 = min(r[q].y, 0xFFFFu), ww = w16 | (w16 << 16);
      acc.x = __vminu2(acc.x, __vaddus2(v[q].x, ww));
      acc.y = __vminu2(acc.y, __vaddus2(v[q].y, ww));
      acc.z = __vminu2(acc.z, __vaddus2(v[q].z, ww));
      acc.w = __vminu2(acc.w, __vaddus2(v[q].w, ww));
    }
  }
  if (!any) return;  // the row keeps its seed or INF
  uint32_t* a4 = &acc.x;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t lo = a4[q] & 0xFFFFu, hi = a4[q] >> 16;
    if (2 * q >= (int)valid_lanes || lo > thr[lane + 2 * q]) lo = 0xFFFFu;
    if (2 * q + 1 >= (int)valid_lanes || hi > thr[lane + 2 * q + 1]) hi = 0xFFFFu;
    a4[q] = lo | (hi << 16);
  }
  if (!live) return;
  uint32_t* dst = reinterpret_cast<uint32_t*>(slab + (size_t)it.x * Kp + lane);
  if (it.w) {
    atomic_min_u16x2(dst + 0, acc.x, err);
    atomic_min_u16x2(dst + 1, acc.y, err);
    atomic_min_u16x2(dst + 2, acc.z, err);
    atomic_min_u16x2(dst + 3, acc.w, err);
  } else {
    const bool valid = (seeded[it.x >> 5] >> (it.x & 31)) & 1u;
    const uint4* d4 = reinterpret_cast<const uint4*>(dst);
    const uint4 c = valid ? (CG ? __ldcg(d4) : *d4) : make_uint4(~0u, ~0u, ~0u, ~0u);
    uint4 nv;
    nv.x = __vminu2(c.x, acc.x);
    nv.y = __vminu2(c.y, acc.y);
    nv.z = __vminu2(c.z, acc.z);
    nv.w = __vminu2(c.w, acc.w);
    *reinterpret_cast<uint4*>(dst) = nv;
  }
  if ((acc.x & acc.y & acc.z & acc.w) != ~0u) atomicOr(&active[it.x >> 5], 1u << (it.x & 31));
}

// Waves of at most 128 lanes: G = Kp / 8 threads (8 lanes each) per item, so
// a warp holds 32 / G items. Each thread walks its item's in-edges itself,
// four at a time (edge records, activity words and rows of four edges in
// flight together); the G threads of an item read the same edges and
// activity bits, so they agree on whether any source is active. Items whose
// edge counts differ simply leave the loop at different times.
template <uint32_t G>
__global__ void __launch_bounds__(128, 12)
    k_sweep_group16(const uint4* __restrict__ item, uint32_t i0, uint32_t i1,
                    const uint2* __restrict__ erec, uint16_t* __restrict__ slab, uint32_t Kp,
                    uint32_t* __restrict__ active, const uint32_t* __restrict__ thr, uint32_t kw,
                    const uint32_t* __restrict__ seeded, uint32_t* __restrict__ err) {
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = (tid % G) * 8;
  const bool live = lane < Kp;
  const uint32_t valid_lanes = live ? min(8u, kw > lane ? kw - lane : 0u) : 0u;
  const uint32_t groups = gridDim.x * (blockDim.x / G);
  // the first item record does not depend on the previous level: load it,
  // and bring its edge records towards L2, while that level drains
  const uint32_t f = i0 + tid / G;
  uint4 it0 = make_uint4(0, 0, 0, 0);
  if (f < i1) {
    it0 = item[f];
    asm volatile("prefetch.global.L2 [%0];" ::"l"(erec + it0.y));
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  for (uint32_t ii = f; ii < i1; ii += groups)
    group16_item<false>(ii == f ? it0 : item[ii], erec, slab, Kp, active, thr, lane, live,
                        valid_lanes, seeded, err);
}

// A run of consecutive small levels [l0, l1) of the 16-bit gated sweep in one
// block of 1024 threads instead of a launch per level: wpi = ceil(Kp / 256)
// warps share an item (a 256-lane slice each), the block takes 32 / wpi items
// at a time, and __syncthreads separates the levels (the block's global
// writes before it are visible to the block after it). Each warp loads its
// first item record and edge records of the next level before the barrier:
// they do not depend on the sweep's values. lvl: level -> first item.
__global__ void __launch_bounds__(1024, 1)
    k_sweep_run16(const uint4* __restrict__ item, const uint32_t* __restrict__ lvl, uint32_t l0,
                  uint32_t l1, const uint2* __restrict__ erec, uint16_t* __restrict__ slab,
                  uint32_t Kp, uint32_t* __restrict__ active, const uint32_t* __restrict__ thr,
                  uint32_t kw, const uint32_t* __restrict__ seeded, uint32_t* __restrict__ err) {
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t t = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t wpi = (Kp + 255) / 256;  // 1..32 (the host launches this for Kp <= 8192)
  const uint32_t slots = 32 / wpi, slot = warp / wpi;
  const uint32_t lane = (warp % wpi) * 256 + t * 8;
  const bool warp_live = slot < slots && (warp % wpi) * 256 < Kp;
  const bool live = warp_live && lane < Kp;
  const uint32_t valid_lanes = live ? min(8u, kw > lane ? kw - lane : 0u) : 0u;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  uint32_t i1 = lvl[l0 + 1], ii = lvl[l0] + slot;
  uint4 it = make_uint4(0, 0, 0, 0);
  uint2 r0 = make_uint2(0, 0);
  if (warp_live && ii < i1) {
    it = item[ii];
    r0 = it.y + t < it.z ? erec[it.y + t] : make_uint2(0, 0);
  }
  for (uint32_t l = l0; l < l1; ++l) {
    for (bool first = true; warp_live && ii < i1; ii += slots, first = false) {
      if (!first) {
        it = item[ii];
        r0 = it.y + t < it.z ? erec[it.y + t] : make_uint2(0, 0);
      }
      gated16_item<true>(it, r0, erec, slab, Kp, active, thr, lane, live, valid_lanes, seeded, err);
    }
    if (l + 1 < l1) {  // the next level's first item, before the barrier
      i1 = lvl[l + 2];
      ii = lvl[l + 1] + slot;
      if (warp_live && ii < i1) {
        it = item[ii];
        r0 = it.y + t < it.z ? erec[it.y + t] : make_uint2(0, 0);
      }
    }
    __syncthreads();
  }
}

// ---- bulk-copy staging of a level's schedule -------------------------------
// mbarrier and cp.async.bulk helpers (shared memory of this CTA).
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bytes (a multiple of 16) from 16-byte aligned global src to shared dst
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

constexpr uint32_t STAGE_ITEMS = 128;   // items of a staged level at most
constexpr uint32_t STAGE_EREC = 2048;   // edge records of a staged level at most
constexpr uint32_t STAGE_POLLS = 1u << 22;  // bound on a wait for a staged level

// The variant of k_sweep_run16 whose levels come through shared memory:
// thread 0 bulk-copies the next level's work items and the edge records of
// its rows (one contiguous range, start rounded down and end up to 16
// bytes) into the other of two buffers while the block sweeps the current
// level from its buffer, each buffer completing on its own mbarrier. A
// level too large for a buffer, or a wait that gives up after STAGE_POLLS
// polls (the thread then sets DEVERR_TIMEOUT), reads the same records from
// global memory: the result does not depend on the staging.
__global__ void __launch_bounds__(1024, 1)
    k_sweep_run16_staged(const uint4* __restrict__ item, const uint32_t* __restrict__ lvl,
                         const uint32_t* __restrict__ lvl_erec, uint32_t l0, uint32_t l1,
                         const uint2* __restrict__ erec, uint16_t* __restrict__ slab, uint32_t Kp,
                         uint32_t* __restrict__ active, const uint32_t* __restrict__ thr,
                         uint32_t kw, const uint32_t* __restrict__ seeded,
                         uint32_t* __restrict__ err) {
  __shared__ __align__(16) uint4 s_item[2][STAGE_ITEMS];
  __shared__ __align__(16) uint2 s_erec[2][STAGE_EREC];
  __shared__ __align__(8) uint64_t s_bar[2];
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t t = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t wpi = (Kp + 255) / 256;  // 1..32 (launched for Kp <= 8192)
  const uint32_t slots = 32 / wpi, slot = warp / wpi;
  const uint32_t lane = (warp % wpi) * 256 + t * 8;
  const bool warp_live = slot < slots && (warp % wpi) * 256 < Kp;
  const bool live = warp_live && lane < Kp;
  const uint32_t valid_lanes = live ? min(8u, kw > lane ? kw - lane : 0u) : 0u;
  if (threadIdx.x == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // whether level l fits a buffer (every thread computes the same answer)
  auto fits = [&](uint32_t l, uint32_t* e0, uint32_t* eb) {
    const uint32_t n_it = lvl[l + 1] - lvl[l];
    const uint32_t a = lvl_erec[l] & ~1u, b = (lvl_erec[l + 1] + 1) & ~1u;
    *e0 = a;
    *eb = b - a;
    return n_it <= STAGE_ITEMS && b - a <= STAGE_EREC;
  };
  auto issue = [&](uint32_t l, uint32_t buf) {  // thread 0 only
    uint32_t e0, ne;
    if (!fits(l, &e0, &ne)) return;
    const uint32_t n_it = lvl[l + 1] - lvl[l];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&s_bar[buf], n_it * 16 + ne * 8);
    if (n_it) bulk_copy(s_item[buf], item + lvl[l], n_it * 16, &s_bar[buf]);
    if (ne) bulk_copy(s_erec[buf], erec + e0, ne * 8, &s_bar[buf]);
  };
  __shared__ int s_giveup;
  if (threadIdx.x == 0) s_giveup = 0;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __syncthreads();
  // per buffer: the phase to wait for and whether a copy into it is pending
  // (the same in every thread: fits() and the give-up flag are uniform)
  uint32_t phase[2] = {0, 0};
  bool pending[2] = {false, false};
  bool giveup = false;
  uint32_t e0, ne;
  if (fits(l0, &e0, &ne)) {
    if (threadIdx.x == 0) issue(l0, 0);
    pending[0] = true;
  }
  for (uint32_t l = l0; l < l1; ++l) {
    const uint32_t buf = (l - l0) & 1u;
    if (!giveup && l + 1 < l1 && fits(l + 1, &e0, &ne)) {
      if (threadIdx.x == 0) issue(l + 1, buf ^ 1u);
      pending[buf ^ 1u] = true;
    }
    const bool staged = fits(l, &e0, &ne) && pending[buf] && !giveup;
    bool ready = false;
    if (staged) {
      ready = true;
      for (uint32_t polls = 0; !mbar_try_wait(&s_bar[buf], phase[buf]);)
        if (++polls >= STAGE_POLLS) {  // give up staging: global records from here on
          atomicOr(err, DEVERR_TIMEOUT);
          s_giveup = 1;
          ready = false;
          break;
        }
      if (ready) {
        phase[buf] ^= 1u;
        pending[buf] = false;
      }
    }
    // records through shared memory when staged, else from global memory;
    // erec indices stay global: the staged copy starts at record e0
    const uint4* it_src = ready ? s_item[buf] - lvl[l] : item;
    const uint2* er_src = ready ? s_erec[buf] - e0 : erec;
    const uint32_t i1 = lvl[l + 1];
    if (warp_live)
      for (uint32_t ii = lvl[l] + slot; ii < i1; ii += slots) {
        const uint4 it = it_src[ii];
        const uint2 r0 = it.y + t < it.z ? er_src[it.y + t] : make_uint2(0, 0);
        gated16_item<true>(it, r0, er_src, slab, Kp, active, thr, lane, live, valid_lanes,
                           seeded, err);
      }
    __syncthreads();
    giveup = s_giveup != 0;
  }
  // no copy may still be writing this block's shared memory when it exits:
  // wait (bounded) for any copy issued but not consumed
  for (uint32_t b = 0; b < 2; ++b)
    if (pending[b])
      for (uint32_t polls = 0; !mbar_try_wait(&s_bar[b], phase[b]) && polls < STAGE_POLLS;)
        ++polls;
}

// A whole 16-bit gated wave sweep in one cooperative launch (waves of at most
// 4096 lanes): the blocks walk the level program, a level's items spread
// over the grid's item slots or a run of small levels swept by block 0
// alone, with a grid barrier between segments. G > 0: groups of G = Kp / 8
// threads per item (group16_item); G = 0: wpi = ceil(Kp / 256) warps per
// item, a 256-lane slice each (gated16_item). `withhold` is the test hook of
// the grid barrier (a block that leaves before its first arrival; NONE
// otherwise). lvl: level -> first item.
template <uint32_t G>
__global__ void __launch_bounds__(512, 2)
    k_iso_persist(const uint2* __restrict__ prog, uint32_t P, const uint32_t* __restrict__ lvl,
                  const uint4* __restrict__ item, const uint2* __restrict__ erec,
                  uint16_t* __restrict__ slab, uint32_t Kp, uint32_t* __restrict__ active,
                  const uint32_t* __restrict__ thr, uint32_t kw,
                  const uint32_t* __restrict__ seeded, uint32_t* __restrict__ bar,
                  long long timeout, uint32_t withhold, uint32_t* __restrict__ err) {
  const uint32_t t = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t lane, slot, slots;  // this thread's lanes, item slot in the block, slots per block
  bool live, slot_live;
  if (G) {
    constexpr uint32_t g1 = G ? G : 1;  // (G = 0 never takes this branch)
    lane = (threadIdx.x % g1) * 8;
    slot = threadIdx.x / g1;
    slots = blockDim.x / g1;
    slot_live = true;
  } else {
    const uint32_t wpi = (Kp + 255) / 256;
    lane = (warp % wpi) * 256 + t * 8;
    slot = warp / wpi;
    slots = (blockDim.x >> 5) / wpi;
    slot_live = slot < slots && (warp % wpi) * 256 < Kp;
  }
  live = slot_live && lane < Kp;
  const uint32_t valid_lanes = live ? min(8u, kw > lane ? kw - lane : 0u) : 0u;
  // The first item of this slot in the next level is loaded before the
  // barrier (or __syncthreads) that precedes that level: the schedule does
  // not depend on the sweep's values, so only the activity and row loads
  // remain after the wait.
  uint32_t pre_ii = NONE;
  uint4 pre_it = make_uint4(0, 0, 0, 0);
  for (uint32_t s = 0; s < P; ++s) {
    const uint2 sg = prog[s];
    const bool run = (sg.y & PROG_RUN) != 0;
    const uint32_t l0 = sg.x, l1 = run ? (blockIdx.x == 0 ? sg.y & ~PROG_RUN : l0) : l0 + 1;
    // a run is swept by block 0 level by level; a grid segment by every block
    const uint32_t first = run ? slot : blockIdx.x * slots + slot;
    const uint32_t stride = run ? slots : gridDim.x * slots;
    for (uint32_t l = l0; l < l1; ++l) {
      const uint32_t i1 = lvl[l + 1];
      if (slot_live)
        for (uint32_t ii = lvl[l] + first; ii < i1; ii += stride) {
          const uint4 it = ii == pre_ii ? pre_it : item[ii];
          if (G) {
            group16_item<true>(it, erec, slab, Kp, active, thr, lane, live, valid_lanes, seeded,
                               err);
          } else {
            const uint2 r0 = it.y + t < it.z ? erec[it.y + t] : make_uint2(0, 0);
            gated16_item<true>(it, r0, erec, slab, Kp, active, thr, lane, live, valid_lanes,
                               seeded, err);
          }
        }
      if (run) {
        pre_ii = NONE;
        if (slot_live && l + 1 < l1) {
          const uint32_t nx = lvl[l + 1] + first;
          if (nx < lvl[l + 2]) {
            pre_ii = nx;
            pre_it = item[nx];
          }
        }
        __syncthreads();
      }
    }
    if (s + 1 == P) break;
    pre_ii = NONE;
    {  // this slot's first item of the next segment
      const uint2 nsg = prog[s + 1];
      const bool nrun = (nsg.y & PROG_RUN) != 0;
      if (slot_live && (!nrun || blockIdx.x == 0)) {
        const uint32_t nx = lvl[nsg.x] + (nrun ? slot : blockIdx.x * slots + slot);
        if (nx < lvl[nsg.x + 1]) {
          pre_ii = nx;
          pre_it = item[nx];
        }
      }
    }
    if (blockIdx.x == withhold) return;
    if (!grid_barrier(bar, s, timeout, err)) return;
  }
}

// bits: rows of w32 u32 words; lane l writes output row out_row[l]. A block
// owns 256 ranks and walks all lane tiles of the wave: the ranks' slab rows
// and activity are looked up once, inactive rows (no value within any lane's
// threshold) are never read, and a tile with no active row only writes zeros.
__global__ void __launch_bounds__(256)
    k_bits(const uint32_t* __restrict__ slab, uint32_t Kp, const uint32_t* __restrict__ cidx,
           uint32_t n, const uint32_t* __restrict__ thr, uint32_t kw, uint32_t* __restrict__ bits,
           uint64_t w32, unsigned long long* __restrict__ counts,
           const uint32_t* __restrict__ active, const uint32_t* __restrict__ out_row) {
  __shared__ uint32_t tile[TILE_R][TILE_L + 1];
  __shared__ uint32_t srow[TILE_R];
  __shared__ int any_active;
  const uint32_t r0 = blockIdx.x * TILE_R;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) any_active = 0;
  __syncthreads();
  {
    const uint32_t rank = r0 + threadIdx.x;
    uint32_t row = NONE;
    if (rank < n) {
      const uint32_t c = cidx[rank];
      if ((active[c >> 5] >> (c & 31)) & 1u) row = c;
    }
    srow[threadIdx.x] = row;
    if (__any_sync(0xFFFFFFFFu, row != NONE) && lane == 0) any_active = 1;
  }
  __syncthreads();
  const bool live = any_active != 0;
  const uint64_t wbase = r0 / 32;
  const uint32_t lend = min(kw, (blockIdx.y + 1) * TILE_L * LANE_TILES_PER_BLOCK);
  for (uint32_t l0 = blockIdx.y * TILE_L * LANE_TILES_PER_BLOCK; l0 < lend; l0 += TILE_L) {
    if (live) {
      for (uint32_t r = warp; r < TILE_R; r += 8) {
        const uint32_t row = srow[r], l = l0 + lane;
        tile[r][lane] = (row != NONE && l < lend) ? slab[(size_t)row * Kp + l] : INF;
      }
      __syncthreads();
    }
    for (uint32_t q = 0; q < 4; ++q) {
      const uint32_t li = warp * 4 + q, l = l0 + li;
      if (l >= lend) continue;  // warp-uniform
      const uint64_t orow = out_row[l];
      uint32_t mine = 0;
      if (live) {
        const uint32_t t = thr[l];
        for (uint32_t c = 0; c < TILE_R / 32; ++c) {
          const uint32_t d = tile[c * 32 + lane][li];
          const uint32_t word = __ballot_sync(0xFFFFFFFFu, d != INF && d <= t);
          if (lane == c) mine = word;
        }
      }
      const uint64_t wi = wbase + lane;
      uint32_t pc = 0;
      if (lane < TILE_R / 32 && wi < w32) {
        bits[orow * w32 + wi] = mine;
        pc = __popc(mine);
      }
      if (live) {
        for (int o = 16; o > 0; o >>= 1) pc += __shfl_down_sync(0xFFFFFFFFu, pc, o);
        if (lane == 0 && pc) atomicAdd(&counts[orow], (unsigned long long)pc);
      }
    }
    if (live) __syncthreads();
  }
}

// 16-bit form of k_bits, written for the output's layout: a block owns
// 2048 ranks x 64 lanes, so every lane's 64 words (256 bytes) of output are
// written as one contiguous run (each origin's bitset row is 1.5 MB long on
// the country graph; 32-byte pieces scattered over a wave's rows cost more
// than the rest of the wave). A warp takes 32 ranks at a time: each thread
// loads its rank's row of 64 lanes (128 bytes, active rows only), and 64
// ballots turn the 32 x 64 lane values into one word per lane, staged in
// shared memory and written lane by lane. Lanes hold 0xFFFF beyond their
// threshold (the sweep and the upward pass clamp), so a bit is just
// "not 0xFFFF" on an active row.
constexpr uint32_t BT_RANKS = 2048;  // ranks per block: 64 words per lane
constexpr uint32_t BT_LANES = 64;    // lanes per block

__global__ void __launch_bounds__(256)
    k_bits16(const uint16_t* __restrict__ slab, uint32_t Kp, const uint32_t* __restrict__ cidx,
             uint32_t n, uint32_t kw, uint32_t* __restrict__ bits, uint64_t w32,
             unsigned long long* __restrict__ counts, const uint32_t* __restrict__ active,
             const uint32_t* __restrict__ out_row) {
  __shared__ uint32_t sw[BT_LANES][BT_RANKS / 32 + 1];
  const uint32_t r0 = blockIdx.x * BT_RANKS, l0 = blockIdx.y * BT_LANES;
  const uint32_t warp = threadIdx.x >> 5, t = threadIdx.x & 31;
  const unsigned FULL = 0xFFFFFFFFu;
  for (uint32_t gi = warp; gi < BT_RANKS / 32; gi += 8) {
    const uint32_t rank = r0 + gi * 32 + t;
    uint32_t row = NONE;
    if (rank < n) {
      const uint32_t c = cidx[rank];
      if ((active[c >> 5] >> (c & 31)) & 1u) row = c;
    }
    if (!__any_sync(FULL, row != NONE)) {  // no active rank here: zero words
      sw[t][gi] = 0;
      sw[t + 32][gi] = 0;
      continue;
    }
    uint4 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      v[q] = (row != NONE && l0 + 8 * q < Kp)
                 ? *reinterpret_cast<const uint4*>(slab + (size_t)row * Kp + l0 + 8 * q)
                 : make_uint4(~0u, ~0u, ~0u, ~0u);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint32_t w4[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
      for (int h = 0; h < 8; ++h) {
        const uint32_t d = (w4[h >> 1] >> ((h & 1) * 16)) & 0xFFFFu;
        const uint32_t word = __ballot_sync(FULL, d != 0xFFFFu);
        const uint32_t j = 8 * q + h;  // lane within the block
        if (t == (j & 31)) sw[j][gi] = word;
      }
    }
  }
  __syncthreads();
  const uint32_t nl = kw > l0 ? min(BT_LANES, kw - l0) : 0u;
  const uint64_t wbase = r0 >> 5;
  for (uint32_t j = warp; j < nl; j += 8) {
    const uint64_t orow = out_row[l0 + j];
    uint32_t pc = 0;
    for (uint32_t k = t; k < BT_RANKS / 32; k += 32) {
      const uint64_t wi = wbase + k;
      if (wi < w32) {
        const uint32_t word = sw[j][k];
        bits[orow * w32 + wi] = word;
        pc += __popc(word);
      }
    }
    for (int o = 16; o > 0; o >>= 1) pc += __shfl_down_sync(FULL, pc, o);
    if (t == 0 && pc) atomicAdd(&counts[orow], (unsigned long long)pc);
  }
}

// Settled lists of a wave. Lane l's bitset (row lane_row[l] of `bits`, w32
// words, ranks ascending) gives its settled ranks; k_lane_prefix turns word
// popcounts into each word's first output position, k_emit writes
// (rank, distance) pairs from the slab in rank order.
__global__ void __launch_bounds__(1024)
    k_lane_prefix(const uint32_t* __restrict__ bits, uint64_t w32,
                  const uint32_t* __restrict__ lane_row, uint32_t* __restrict__ pre) {
  __shared__ uint32_t wsum[32];
  const uint32_t l = blockIdx.x;
  const uint32_t* b = bits + (uint64_t)lane_row[l] * w32;
  uint32_t* o = pre + (uint64_t)l * w32;
  uint32_t carry = 0;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint64_t w0 = 0; w0 < w32; w0 += blockDim.x) {
    const uint64_t w = w0 + threadIdx.x;
    const uint32_t v = w < w32 ? __popc(b[w]) : 0;
    uint32_t x = v;  // inclusive warp scan
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t s = lane < (blockDim.x >> 5) ? wsum[lane] : 0;
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, d);
        if (lane >= d) s += y;
      }
      wsum[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = (warp ? wsum[warp - 1] : 0) + x - v;
    if (w < w32) o[w] = carry + before;
    carry += wsum[(blockDim.x >> 5) - 1];
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_emit(const T* __restrict__ slab, uint32_t Kp, const uint32_t* __restrict__ cidx, uint32_t n,
           const uint32_t* __restrict__ bits, uint64_t w32, const uint32_t* __restrict__ lane_row,
           const uint32_t* __restrict__ pre, const uint64_t* __restrict__ lane_off,
           uint64_t total, uint32_t* __restrict__ out_rank, uint32_t* __restrict__ out_dist) {
  const uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint32_t l = blockIdx.y;
  if (w >= w32) return;
  uint32_t m = bits[(uint64_t)lane_row[l] * w32 + w];
  if (!m) return;
  uint64_t pos = lane_off[l] + pre[(uint64_t)l * w32 + w];
  while (m) {
    const uint32_t bit = __ffs(m) - 1;
    m &= m - 1;
    const uint32_t rank = (uint32_t)(w * 32 + bit);
    if (rank < n && pos < total) {
      out_rank[pos] = rank;
      out_dist[pos] = (uint32_t)slab[(size_t)cidx[rank] * Kp + l];
    }
    ++pos;
  }
}

template <typename T>
bf_status emit_settled(const T* slab, uint32_t Kp, Graph* g, Sched& sc, const uint32_t* bits,
                       uint64_t w32, const uint32_t* d_lane_row, const uint32_t* h_lane_row,
                       uint32_t kw, const uint64_t* d_counts, uint64_t n_all, SettledSink* sink,
                       cudaStream_t st) {
  std::vector<uint64_t> cnt(n_all);
  BF_CUDA(cudaMemcpyAsync(cnt.data(), d_counts, n_all * 8, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  std::vector<uint64_t> off(kw + 1, 0);
  for (uint32_t l = 0; l < kw; ++l) off[l + 1] = off[l] + cnt[h_lane_row[l]];
  const uint64_t total = off[kw];
  auto grow = [&](auto** p, size_t& cap, size_t need) -> cudaError_t {
    if (cap >= need) return cudaSuccess;
    if (*p) cudaFree(*p);
    g->device_bytes -= cap;
    *p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc((void**)p, need);
    if (e == cudaSuccess) {
      cap = need;
      g->device_bytes += need;
    }
    return e;
  };
  BF_CUDA(grow(&g->d_set_pre, g->set_pre_bytes, std::max<size_t>(16, (size_t)kw * w32 * 4)));
  BF_CUDA(grow(&g->d_set_out, g->set_out_bytes, std::max<size_t>(16, (size_t)total * 8)));
  BF_CUDA(grow(&g->d_set_off, g->set_off_bytes, (size_t)(kw + 1) * 8));
  BF_CUDA(cudaMemcpyAsync(g->d_set_off, off.data(), (kw + 1) * 8, cudaMemcpyHostToDevice, st));
  k_lane_prefix<<<kw, 1024, 0, st>>>(bits, w32, d_lane_row, g->d_set_pre);
  dim3 eg((unsigned)((w32 + 255) / 256), kw);
  k_emit<T><<<eg, 256, 0, st>>>(slab, Kp, sc.d_cidx, g->n, bits, w32, d_lane_row, g->d_set_pre,
                                g->d_set_off, total, g->d_set_out, g->d_set_out + total);
  BF_CUDA(cudaGetLastError());
  if (sink->on_wave) {
    std::vector<uint32_t> rows(kw);
    for (uint32_t l = 0; l < kw; ++l) rows[l] = (uint32_t)(sink->base + h_lane_row[l]);
    return sink->on_wave(g->d_set_out, g->d_set_out + total, g->d_set_off, off, rows, st);
  }
  // the wave's ranks then distances, appended to the page-locked staging
  const uint64_t need = sink->used + 2 * total;
  if (need > g->set_stage_cap) {
    const uint64_t cap = need + need / 4;
    uint32_t* p = nullptr;
    BF_CUDA(cudaHostAlloc((void**)&p, cap * 4, cudaHostAllocDefault));
    if (sink->used) std::memcpy(p, g->h_set_stage, sink->used * 4);
    if (g->h_set_stage) cudaFreeHost(g->h_set_stage);
    g->h_set_stage = p;
    g->set_stage_cap = cap;
  }
  if (total)
    BF_CUDA(cudaMemcpyAsync(g->h_set_stage + sink->used, g->d_set_out, total * 8,
                            cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  for (uint32_t l = 0; l < kw; ++l) {
    const uint64_t o = sink->base + h_lane_row[l];
    sink->r_at[o] = sink->used + off[l];
    sink->d_at[o] = sink->used + total + off[l];
    sink->cnt[o] = off[l + 1] - off[l];
  }
  sink->used = need;
  return BF_OK;
}

// Algorithmic bytes of one gated wave sweep, counted after it from its final
// activity bitmap: an item is processed when one of its in-edge source rows
// is active; it then gathers each active source row and writes its row
// (row_bytes each). Block sums go to counts[0] (bytes) and counts[1] (rows).
__global__ void __launch_bounds__(256)
    k_iso_count(const uint4* __restrict__ item, uint64_t n_items, const uint2* __restrict__ erec,
                const uint32_t* __restrict__ active, uint32_t row_bytes,
                unsigned long long* __restrict__ counts) {
  uint64_t bytes = 0, rows = 0;
  for (uint64_t ii = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; ii < n_items;
       ii += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 it = item[ii];
    uint32_t a = 0;
    for (uint32_t e = it.y; e < it.z; ++e) {
      const uint32_t r = erec[e].x;
      a += (active[r >> 5] >> (r & 31)) & 1u;
    }
    if (a) {
      bytes += (uint64_t)(a + 1) * row_bytes;
      ++rows;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    bytes += __shfl_down_sync(0xFFFFFFFFu, bytes, o);
    rows += __shfl_down_sync(0xFFFFFFFFu, rows, o);
  }
  if ((threadIdx.x & 31) == 0 && bytes) {
    atomicAdd(&counts[0], (unsigned long long)bytes);
    atomicAdd(&counts[1], (unsigned long long)rows);
  }
}

constexpr unsigned ISO_PERSIST_TPB = 512;

// One persistent launch of k_iso_persist for a wave of Kp <= 4096 lanes; the
// level program (runs of levels with at most two rounds of block 0's item
// slots) is cached per context and lane width.
bf_status iso_sweep_persistent(Graph* g, Ctx& c, Sched& sc, uint16_t* slab16, uint32_t Kp,
                               uint32_t* d_active, const uint32_t* d_thr, uint32_t kw,
                               const uint32_t* d_seeded, cudaStream_t st) {
  const uint32_t G = Kp <= 8 ? 1 : Kp <= 16 ? 2 : Kp <= 32 ? 4 : Kp <= 64 ? 8 : Kp <= 128 ? 16 : 0;
  const uint32_t slots = G ? ISO_PERSIST_TPB / G : (ISO_PERSIST_TPB / 32) / ((Kp + 255) / 256);
  bf_status s;
  if ((s = ensure_barrier(g))) return s;
  if (c.iso_prog_slots != slots || c.iso_prog_levels != sc.lvl_item.size()) {
    c.iso_prog = level_program(sc.lvl_item, g->n_levels, 2 * slots);
    const size_t bytes = std::max<size_t>(c.iso_prog.size(), 1) * sizeof(uint2);
    if (bytes > c.iso_prog_bytes) {
      if (c.d_iso_prog) {
        cudaFree(c.d_iso_prog);
        g->device_bytes -= c.iso_prog_bytes;
      }
      c.d_iso_prog = nullptr;
      c.iso_prog_bytes = 0;
      BF_CUDA(cudaMalloc(&c.d_iso_prog, bytes));
      c.iso_prog_bytes = bytes;
      g->device_bytes += bytes;
    }
    BF_CUDA(cudaMemcpyAsync(c.d_iso_prog, c.iso_prog.data(), c.iso_prog.size() * sizeof(uint2),
                            cudaMemcpyHostToDevice, st));
    c.iso_prog_slots = slots;
    c.iso_prog_levels = sc.lvl_item.size();
  }
  auto kern = G == 1 ? k_iso_persist<1> : G == 2 ? k_iso_persist<2> : G == 4 ? k_iso_persist<4>
            : G == 8 ? k_iso_persist<8> : G == 16 ? k_iso_persist<16> : k_iso_persist<0>;
  const bool hook = test_withhold_arrival();
  const unsigned blocks = persistent_blocks(g, (const void*)kern, ISO_PERSIST_TPB, 2 * g->sm_count);
  uint32_t* bar = g->d_bar + 2;  // the plain engine's sweep uses words 0-1
  BF_CUDA(cudaMemsetAsync(bar, 0, 8, st));
  BF_CUDA(launch_persistent(kern, blocks, ISO_PERSIST_TPB, st, (const uint2*)c.d_iso_prog,
                            (uint32_t)c.iso_prog.size(), (const uint32_t*)sc.d_lvl,
                            (const uint4*)sc.d_item, (const uint2*)sc.d_erec, slab16, Kp, d_active,
                            d_thr, kw, d_seeded, bar, hook ? 2000000ll : BARRIER_TIMEOUT_CYCLES,
                            hook ? 1u : NONE, g->d_err));
  return BF_OK;
}

}  // namespace

// d_bits: n rows of ceil(n_nodes / 64) u64 words; d_counts: n u64.
// Origins are processed in (threshold, rank) order so that the lanes of a
// wave share a threshold and lie close together in the nested-dissection
// order, which keeps the set of active rows of the gated sweep small.
bf_status isochrone_bitsets(Graph* g, Ctx& c, const uint32_t* d_orig, const uint32_t* d_thr, uint64_t n,
                            uint64_t* d_bits, uint64_t* d_counts, cudaStream_t st,
                            bf_stats* stats, SettledSink* sink) {
  bf_status s;
  if (!c.shared_full && (s = build_schedule(g, c, c.full, nullptr, 0, true, st))) return s;
  Sched& sc = c.shared_full ? *c.shared_full : c.full;
  const uint64_t rows = g->n;
  const uint64_t w64 = (g->n + 63) / 64;
  const uint64_t aw = (rows + 31) / 32;  // active-bitmap words
  // permutation: (threshold, rank) order
  std::vector<uint32_t> ho(n), ht(n), perm(n);
  BF_CUDA(cudaMemcpyAsync(ho.data(), d_orig, n * 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaMemcpyAsync(ht.data(), d_thr, n * 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  for (uint64_t i = 0; i < n; ++i)
    if (ho[i] >= g->n) {
      set_error("origins[" + std::to_string(i) + "] is not a node of the graph");
      return BF_ERR_INVALID;
    }
  for (uint64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
  std::sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) {
    return ht[a] != ht[b] ? ht[a] < ht[b] : ho[a] < ho[b];
  });
  std::vector<uint32_t> pk(3 * n);
  for (uint64_t i = 0; i < n; ++i) {
    pk[i] = ho[perm[i]];
    pk[n + i] = ht[perm[i]];
    pk[2 * n + i] = perm[i];
  }
  const size_t need = pk.size() * 4 + 2 * aw * 4 + 16;
  if (need > c.iso_tmp_bytes) {
    if (c.d_iso_tmp) {
      cudaFree(c.d_iso_tmp);
      g->device_bytes -= c.iso_tmp_bytes;
      c.d_iso_tmp = nullptr;
      c.iso_tmp_bytes = 0;
    }
    if (cudaMalloc(&c.d_iso_tmp, need) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc for isochrone scratch failed");
      return BF_ERR_OOM;
    }
    c.iso_tmp_bytes = need;
    g->device_bytes += need;
  }
  uint32_t* p_orig = c.d_iso_tmp;
  uint32_t* p_thr = p_orig + n;
  uint32_t* p_row = p_thr + n;
  uint32_t* d_active = p_row + n;
  uint32_t* d_seeded = d_active + aw;
  BF_CUDA(cudaMemcpyAsync(p_orig, pk.data(), pk.size() * 4, cudaMemcpyHostToDevice, st));
  // 16-bit lanes when every threshold fits below 0xFFFF (the clamp keeps
  // distances within the thresholds exact and halves the bytes moved)
  uint32_t tmax = 0;
  for (uint64_t i = 0; i < n; ++i) tmax = std::max(tmax, ht[i]);
  const bool half = g->tune.iso_half && tmax < 0xFFFFu;
  const uint32_t lb = half ? 2 : 4;      // bytes per lane
  const uint32_t lq = half ? 8 : 4;      // lanes per thread (one 16-byte load)
  // the slab is the only per-lane device memory here
  uint64_t max_lanes = ctx_budget(g, c) / (rows * lb);
  max_lanes = max_lanes >= 32 ? max_lanes & ~31ull : 0;
  if (!max_lanes) {
    set_error("HBM budget too small for one 32-lane isochrone wave");
    return BF_ERR_OOM;
  }
  if (g->tune.iso_lanes) max_lanes = std::min<uint64_t>(max_lanes, g->tune.iso_lanes);
  const uint64_t wave = std::min<uint64_t>(max_lanes, (n + lq - 1) & ~(uint64_t)(lq - 1));
  const uint32_t Kp = (uint32_t)((wave + lq - 1) & ~(uint64_t)(lq - 1));
  if ((s = ensure_slab(g, c, (size_t)rows * Kp * lb))) return s;
  BF_CUDA(cudaMemsetAsync(d_counts, 0, n * 8, st));
  const unsigned tpb = std::min<uint32_t>(128, ((Kp / lq + 31) / 32) * 32);
  const unsigned lane_blocks = (Kp / lq + tpb - 1) / tpb;
  uint16_t* slab16 = reinterpret_cast<uint16_t*>(c.d_slab);
  uint64_t launches = 0;
  float t_up = 0, t_dn = 0, t_ex = 0;
  if (stats) {  // algorithmic-byte counters of the sweeps (k_iso_count)
    if (!c.d_count) {
      BF_CUDA(cudaMalloc(&c.d_count, 16));
      g->device_bytes += 16;
    }
    BF_CUDA(cudaMemsetAsync(c.d_count, 0, 16, st));
  }
  for (uint64_t s0 = 0; s0 < n; s0 += wave) {
    const uint64_t kw = std::min<uint64_t>(wave, n - s0);
    if (stats) BF_CUDA(cudaEventRecord(c.ev[0], st));
    BF_CUDA(cudaMemsetAsync(d_active, 0, 2 * aw * 4, st));  // active + seeded bitmaps
    launch_mark_paths(g, p_orig + s0, kw, sc.d_cidx, d_seeded, st);
    // rows are Kp * lb bytes = Kp * lb / 4 words
    launch_init_rows(d_seeded, sc.d_split, (uint32_t)aw, c.d_slab, Kp * lb / 4, st);
    launches += 2;
    if ((s = launch_upward(g, p_orig + s0, kw, INF, sc.d_cidx, c.d_slab, Kp, d_active, st,
                           p_thr + s0, nullptr, nullptr,
                           half ? UPWARD_OUT_SLAB16 : UPWARD_OUT_SLAB32)))
      return s;
    ++launches;
    if (stats) BF_CUDA(cudaEventRecord(c.ev[1], st));
    if (half && (g->tune.persist & 2u) && Kp <= 4096) {
      if ((s = iso_sweep_persistent(g, c, sc, slab16, Kp, d_active, p_thr + s0, (uint32_t)kw,
                                    d_seeded, st)))
        return s;
      ++launches;
    } else if (half) {
      const bool pdl = g->tune.pdl != 0;
      // runs of consecutive levels of at most two rounds of one block's items
      // go to k_sweep_run16 (one launch per run)
      const uint32_t wpi = (Kp + 255) / 256;
      const uint32_t small = wpi <= 32 ? 2 * (32 / wpi) : 0;
      for (uint32_t l = 0; l < g->n_levels; ++l) {
        const uint32_t i0 = sc.lvl_item[l], i1 = sc.lvl_item[l + 1];
        if (i1 == i0) continue;
        if (i1 - i0 <= small) {
          uint32_t l1 = l + 1;
          while (l1 < g->n_levels && sc.lvl_item[l1 + 1] - sc.lvl_item[l1] <= small) ++l1;
          if (l1 - l >= 2) {
            if (g->tune.staged && sc.lvl_erec_ready)
              BF_CUDA(launch_level(k_sweep_run16_staged, dim3(1), 1024, pdl, st,
                                   (const uint4*)sc.d_item, (const uint32_t*)sc.d_lvl,
                                   (const uint32_t*)sc.d_lvl_erec, l, l1, (const uint2*)sc.d_erec,
                                   slab16, Kp, d_active, (const uint32_t*)(p_thr + s0),
                                   (uint32_t)kw, (const uint32_t*)d_seeded, g->d_err));
            else
              BF_CUDA(launch_level(k_sweep_run16, dim3(1), 1024, pdl, st, (const uint4*)sc.d_item,
                                   (const uint32_t*)sc.d_lvl, l, l1, (const uint2*)sc.d_erec,
                                   slab16, Kp, d_active, (const uint32_t*)(p_thr + s0),
                                   (uint32_t)kw, (const uint32_t*)d_seeded, g->d_err));
            ++launches;
            l = l1 - 1;
            continue;
          }
        }
        if (Kp <= 128) {  // thread groups of Kp / 8 threads per item
          const uint32_t G = Kp <= 8 ? 1 : Kp <= 16 ? 2 : Kp <= 32 ? 4 : Kp <= 64 ? 8 : 16;
          const uint32_t per_block = 128 / G;
          const uint32_t blocks = std::min<uint32_t>((i1 - i0 + per_block - 1) / per_block,
                                                     GATED16_BLOCKS);
          auto kern = G == 1 ? k_sweep_group16<1> : G == 2 ? k_sweep_group16<2>
                    : G == 4 ? k_sweep_group16<4> : G == 8 ? k_sweep_group16<8>
                                                          : k_sweep_group16<16>;
          BF_CUDA(launch_level(kern, dim3(blocks), 128, pdl, st, (const uint4*)sc.d_item, i0, i1,
                               (const uint2*)sc.d_erec, slab16, Kp, d_active,
                               (const uint32_t*)(p_thr + s0), (uint32_t)kw,
                               (const uint32_t*)d_seeded, g->d_err));
          ++launches;
          continue;
        }
        const bool own = Kp <= 256;  // four warps per block with their own items
        const uint32_t blocks = own ? std::min<uint32_t>((i1 - i0 + 3) / 4, 152 * 12)
                                    : std::min<uint32_t>(i1 - i0, GATED16_BLOCKS);
        BF_CUDA(launch_level(own ? k_sweep_gated16<4> : k_sweep_gated16<1>,
                             dim3(blocks, own ? 1 : lane_blocks), own ? 128 : tpb, pdl, st,
                             (const uint4*)sc.d_item, i0, i1, (const uint2*)sc.d_erec, slab16,
                             Kp, d_active, (const uint32_t*)(p_thr + s0), (uint32_t)kw,
                             (const uint32_t*)d_seeded, g->d_err));
        ++launches;
      }
    } else if ((s = sweep_levels_gated(g, sc, c.d_slab, Kp, lane_blocks, tpb, d_active,
                                       p_thr + s0, (uint32_t)kw, st, &launches, d_seeded))) {
      return s;
    }
    if (stats) BF_CUDA(cudaEventRecord(c.ev[2], st));
    dim3 bgrid((unsigned)((g->n + TILE_R - 1) / TILE_R),
               (unsigned)((kw + TILE_L * LANE_TILES_PER_BLOCK - 1) / (TILE_L * LANE_TILES_PER_BLOCK)));
    if (half) {
      dim3 bg16((unsigned)((g->n + BT_RANKS - 1) / BT_RANKS),
                (unsigned)((kw + BT_LANES - 1) / BT_LANES));
      k_bits16<<<bg16, 256, 0, st>>>(slab16, Kp, sc.d_cidx, g->n, (uint32_t)kw,
                                     reinterpret_cast<uint32_t*>(d_bits), 2 * w64,
                                     reinterpret_cast<unsigned long long*>(d_counts), d_active,
                                     p_row + s0);
    } else
      k_bits<<<bgrid, 256, 0, st>>>(c.d_slab, Kp, sc.d_cidx, g->n, p_thr + s0,
                                              (uint32_t)kw, reinterpret_cast<uint32_t*>(d_bits),
                                              2 * w64,
                                              reinterpret_cast<unsigned long long*>(d_counts),
                                              d_active, p_row + s0);
    BF_CUDA(cudaGetLastError());
    ++launches;
    if (sink) {
      const uint32_t* h_rows = pk.data() + 2 * n + s0;
      const uint32_t* bits32 = reinterpret_cast<const uint32_t*>(d_bits);
      bf_status es = half ? emit_settled(slab16, Kp, g, sc, bits32, 2 * w64, p_row + s0, h_rows,
                                         (uint32_t)kw, d_counts, n, sink, st)
                          : emit_settled(c.d_slab, Kp, g, sc, bits32, 2 * w64, p_row + s0, h_rows,
                                         (uint32_t)kw, d_counts, n, sink, st);
      if (es) return es;
      launches += 2;
    }
    if (stats) {
      BF_CUDA(cudaEventRecord(c.ev[3], st));
      // outside the timed phases: count the wave's algorithmic sweep bytes
      k_iso_count<<<(unsigned)std::min<uint64_t>((sc.n_items + 255) / 256, 152 * 8), 256, 0, st>>>(
          (const uint4*)sc.d_item, sc.n_items, (const uint2*)sc.d_erec, d_active, Kp * lb,
          reinterpret_cast<unsigned long long*>(c.d_count));
      BF_CUDA(cudaGetLastError());
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
  BF_CUDA(cudaStreamSynchronize(st));  // pk / perm host vectors die on return
  if (stats) {
    const uint64_t waves = (n + wave - 1) / wave;
    stats->n_batches += waves;
    stats->waves += waves;
    stats->kernel_launches += launches;
    stats->upward_ms += t_up;
    stats->downward_ms += t_dn;
    stats->extract_ms += t_ex;
    stats->swept_nodes = sc.n_r;
    stats->swept_edges = sc.n_edges;
    stats->lanes = Kp;
    uint64_t cnt[2] = {0, 0};
    BF_CUDA(cudaMemcpyAsync(cnt, c.d_count, 16, cudaMemcpyDeviceToHost, st));
    BF_CUDA(cudaStreamSynchronize(st));
    // + every wave scans the schedule: 16 B per item and 8 B per edge record
    stats->sweep_bytes += cnt[0] + waves * (16 * sc.n_items + 8 * sc.n_edges);
    stats->active_rows += cnt[1];
  }
  return BF_OK;
}

}  // namespace bf
