// Matrix tile emission on the device: the four UInt32 columns of a matrix
// RecordBatch (source_idx, target_idx, duration_ms, distance_m) from a
// row-major block of durations, as build_matrix_batch and
// build_matrix_tile_batch build them on the host
// (route/src/server/flight.rs:432-500, :509-589):
//   * cells in row-major order; a cell is pruned when the source's sorted
//     radius list (indexed by the source's original index) lacks the
//     destination's original index (:452-456, :528-532);
//   * a pruned cell reads u32::MAX, any other the matrix value, u32::MAX
//     above the time bound (:459, :534-539);
//   * sparse output drops cells whose duration is u32::MAX (:465, :542);
//   * duration_ms = d.saturating_mul(1000); distance_m = the lat matrix's
//     cell or u32::MAX; both u32::MAX on a sentinel cell (:470-483, :548-566).
// The columns come out as plain u32 arrays: Arrow's layout of a UInt32 array
// without nulls, so the caller wraps them without a copy.
//
// Dense: one thread per cell, or per four cells with 16-byte accesses when
// rows are a multiple of four cells (2D grid: columns x rows), reads and the
// four column writes coalesced. Sparse: an order-preserving compaction - a
// count and the kept-cell ballots per block (a row segment of up to 16384
// cells for rows of 2048 cells or more, its radius list read once and
// searched in shared memory when it fits; else 2048 consecutive cells), a
// device-wide scan of the counts, then an ordered write of the kept cells.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.cuh"
#include "scan.cuh"

using namespace bf;

namespace {

constexpr uint32_t MAXV = 0xFFFFFFFFu;
constexpr uint32_t TPB = 256, ITEMS = 8, CELLS = TPB * ITEMS;
constexpr uint32_t ERR_NO_LIST = 1u, ERR_BAD_LIST = 2u;

struct TileIn {
  const uint32_t* m;
  const uint32_t* lat;  // may be null
  uint32_t n_src, n_dst;
  const uint32_t* src_orig;
  const uint32_t* dst_orig;
  uint32_t threshold;
  const uint64_t* mask_off;  // null: no radius mask
  const uint32_t* mask;
  uint32_t n_mask_src;
  uint64_t n_mask;
  uint32_t sparse;
};

struct TileOut {
  uint32_t *s, *t, *du, *di;
};

// (row, column) of a flat cell index; 32-bit division when the block allows.
__device__ __forceinline__ void split(uint64_t i, uint32_t n_dst, bool narrow, uint32_t* si,
                                      uint32_t* di) {
  if (narrow) {
    const uint32_t q = (uint32_t)i / n_dst;
    *si = q;
    *di = (uint32_t)i - q * n_dst;
  } else {
    *si = (uint32_t)(i / n_dst);
    *di = (uint32_t)(i % n_dst);
  }
}

// binary_search's answer (present or not) on a sorted list: halving steps on
// 32-bit offsets, one comparison at the end.
__device__ __forceinline__ bool in_list(const uint32_t* __restrict__ v, uint32_t len, uint32_t x) {
  if (len == 0) return false;
  while (len > 1) {
    const uint32_t half = len >> 1;
    if (v[half] <= x) v += half;
    len -= half;
  }
  return *v == x;
}

// The cell's duration d (already loaded) after pruning and the time bound
// (both give u32::MAX, so the bound is tested first and only cells within
// it search the radius list); os, od: the original indices.
__device__ __forceinline__ uint32_t decide(const TileIn& a, uint32_t d, uint32_t os, uint32_t od,
                                           uint32_t* err) {
  if (a.mask_off && os >= a.n_mask_src) {  // the reference indexes every row's list
    atomicOr(err, ERR_NO_LIST);
    return MAXV;
  }
  if (d > a.threshold) return MAXV;
  if (a.mask_off) {
    const uint64_t lo = a.mask_off[os], hi = a.mask_off[os + 1];
    if (hi < lo || hi > a.n_mask || hi - lo > 0xFFFFFFFFull) {
      atomicOr(err, ERR_BAD_LIST);
      return MAXV;
    }
    if (!in_list(a.mask + lo, (uint32_t)(hi - lo), od)) return MAXV;
  }
  return d;
}

__device__ __forceinline__ uint32_t cell_value(const TileIn& a, uint32_t si, uint32_t di,
                                               uint64_t cell, uint32_t* os, uint32_t* od,
                                               uint32_t* err) {
  *os = a.src_orig[si];
  *od = a.dst_orig[di];
  return decide(a, a.m[cell], *os, *od, err);
}

__device__ __forceinline__ void put(const TileIn& a, const TileOut& o, uint64_t k, uint64_t cell,
                                    uint32_t os, uint32_t od, uint32_t d) {
  o.s[k] = os;
  o.t[k] = od;
  if (d == MAXV) {
    o.du[k] = MAXV;
    o.di[k] = MAXV;
  } else {
    const uint64_t ms = (uint64_t)d * 1000u;
    o.du[k] = ms > MAXV ? MAXV : (uint32_t)ms;
    o.di[k] = a.lat ? a.lat[cell] : MAXV;
  }
}


__global__ void __launch_bounds__(TPB) k_tile_dense(TileIn a, TileOut o, uint32_t* err) {
  for (uint32_t si = blockIdx.y; si < a.n_src; si += gridDim.y)
    for (uint32_t di = blockIdx.x * TPB + threadIdx.x; di < a.n_dst; di += gridDim.x * TPB) {
      const uint64_t cell = (uint64_t)si * a.n_dst + di;
      uint32_t os, od;
      const uint32_t d = cell_value(a, si, di, cell, &os, &od, err);
      put(a, o, cell, cell, os, od, d);
    }
}

// Dense with four cells per thread (n_dst a multiple of 4, arrays 16-byte
// aligned): one 16-byte load of durations (and lat) and one 16-byte store
// per column.
__global__ void __launch_bounds__(TPB) k_tile_dense4(TileIn a, TileOut o, uint32_t* err) {
  const uint32_t q4 = a.n_dst >> 2;
  for (uint32_t si = blockIdx.y; si < a.n_src; si += gridDim.y) {
    const uint32_t os = a.src_orig[si];
    const bool no_list = a.mask_off && os >= a.n_mask_src;
    if (no_list && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ERR_NO_LIST);
    for (uint32_t q = blockIdx.x * TPB + threadIdx.x; q < q4; q += gridDim.x * TPB) {
      const uint64_t cell = (uint64_t)si * a.n_dst + 4ull * q;
      const uint4 m4 = *reinterpret_cast<const uint4*>(a.m + cell);
      const uint4 l4 = a.lat ? *reinterpret_cast<const uint4*>(a.lat + cell)
                             : make_uint4(MAXV, MAXV, MAXV, MAXV);
      const uint4 od = *reinterpret_cast<const uint4*>(a.dst_orig + 4ull * q);
      const uint32_t dv[4] = {m4.x, m4.y, m4.z, m4.w}, lv[4] = {l4.x, l4.y, l4.z, l4.w};
      const uint32_t ov[4] = {od.x, od.y, od.z, od.w};
      uint32_t du[4], di[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        uint32_t d = no_list || dv[k] > a.threshold ? MAXV : dv[k];
        if (d != MAXV && a.mask_off) d = decide(a, d, os, ov[k], err);
        if (d == MAXV) {
          du[k] = MAXV;
          di[k] = MAXV;
        } else {
          const uint64_t ms = (uint64_t)d * 1000u;
          du[k] = ms > MAXV ? MAXV : (uint32_t)ms;
          di[k] = lv[k];
        }
      }
      *reinterpret_cast<uint4*>(o.s + cell) = make_uint4(os, os, os, os);
      *reinterpret_cast<uint4*>(o.t + cell) = od;
      *reinterpret_cast<uint4*>(o.du + cell) = make_uint4(du[0], du[1], du[2], du[3]);
      *reinterpret_cast<uint4*>(o.di + cell) = make_uint4(di[0], di[1], di[2], di[3]);
    }
  }
}

// Sparse pass 1: per block the kept cells, per (step, warp) the ballot of
// kept cells (bit lane of word (cell / 32)); rows and columns advance by
// TPB cells a step instead of a division per cell.
__global__ void __launch_bounds__(TPB)
    k_tile_count(TileIn a, uint64_t n, bool narrow, unsigned long long* __restrict__ cnt,
                 uint32_t* __restrict__ keep_bits, uint32_t* err) {
  __shared__ uint32_t red[TPB / 32];
  const uint64_t base = (uint64_t)blockIdx.x * CELLS;
  uint32_t c = 0, si = 0, di = 0;
  split(base + threadIdx.x, a.n_dst, narrow, &si, &di);
  uint32_t dur[ITEMS];  // the block's durations, all loads in flight before any decision
#pragma unroll
  for (uint32_t j = 0; j < ITEMS; ++j) {
    const uint64_t i = base + (uint64_t)j * TPB + threadIdx.x;
    dur[j] = i < n ? a.m[i] : MAXV;
  }
#pragma unroll
  for (uint32_t j = 0; j < ITEMS; ++j) {
    const uint64_t i = base + (uint64_t)j * TPB + threadIdx.x;
    if (base + (uint64_t)j * TPB >= n) break;  // uniform across the block
    if (j) {
      if (a.n_dst >= TPB) {
        di += TPB;
        if (di >= a.n_dst) {
          di -= a.n_dst;
          ++si;
        }
      } else {
        split(i, a.n_dst, narrow, &si, &di);
      }
    }
    bool keep = false;
    if (i < n) keep = decide(a, dur[j], a.src_orig[si], a.dst_orig[di], err) != MAXV;
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, keep);
    if ((threadIdx.x & 31) == 0) keep_bits[(base + (uint64_t)j * TPB) / 32 + (threadIdx.x >> 5)] = bal;
    c += keep;
  }
  for (int s = 16; s > 0; s >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (uint32_t w = 0; w < TPB / 32; ++w) t += red[w];
    cnt[blockIdx.x] = t;
  }
}

// Wide rows (n_dst >= ROW_MIN): a block per row segment of up to SEG cells,
// so a row's radius list is read once per segment: staged in shared memory
// when it holds at most LIST_STAGE entries, else searched in place. Ballot
// words are per row (wpr = ceil(n_dst / 32) words each), counts per
// segment, in cell order.
constexpr uint32_t ROW_MIN = 2048, SEG = 16384, SEG_WORDS = SEG / 32, LIST_STAGE = 4096;
enum : uint32_t { RL_NONE = 0, RL_SMEM = 1, RL_GLOBAL = 2, RL_BAD = 3, RL_MISSING = 4 };
// A staged list is also set into a bitmap of original indices below
// BITMAP_BITS, so a destination id below it is one shared-memory word test
// (ids at or above it are searched in the staged list).
constexpr uint32_t BITMAP_BITS = 1u << 17, BITMAP_WORDS = BITMAP_BITS / 32;

struct RowList {
  uint32_t v[LIST_STAGE];
  uint32_t bmp[BITMAP_WORDS];
};

// Stages len list entries (block-uniform call) and sets the bitmap's first
// nbw words (ids below 32 nbw: the destination ids' range, capped).
__device__ __forceinline__ void stage_row_list(RowList& rl, const uint32_t* __restrict__ src,
                                               uint32_t len, uint32_t nbw) {
  for (uint32_t k = threadIdx.x; k < nbw; k += TPB) rl.bmp[k] = 0;
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < len; k += TPB) {
    const uint32_t x = src[k];
    rl.v[k] = x;
    if (x < nbw * 32) atomicOr(&rl.bmp[x >> 5], 1u << (x & 31));
  }
  __syncthreads();
}

__device__ __forceinline__ bool in_row_list(const RowList& rl, uint32_t len, uint32_t nbw,
                                            uint32_t x) {
  if (x < nbw * 32) return (rl.bmp[x >> 5] >> (x & 31)) & 1u;
  return in_list(rl.v, len, x);
}

// Per wide row, once per call: how its radius list is read ({mode, len, list
// offset low and high words}, decide()'s rules), and into bound[0] the
// largest destination id (the bitmap's range).
__global__ void __launch_bounds__(TPB) k_tile_rowinfo(TileIn a, uint4* __restrict__ info,
                                                      uint32_t* __restrict__ bound) {
  const uint32_t stride = gridDim.x * TPB;
  for (uint32_t si = blockIdx.x * TPB + threadIdx.x; si < a.n_src; si += stride) {
    uint32_t mode = RL_NONE, len = 0;
    uint64_t lo = 0;
    if (a.mask_off) {
      const uint32_t os = a.src_orig[si];
      if (os >= a.n_mask_src) {
        mode = RL_MISSING;
      } else {
        lo = a.mask_off[os];
        const uint64_t hi = a.mask_off[os + 1];
        if (hi < lo || hi > a.n_mask || hi - lo > 0xFFFFFFFFull) {
          mode = RL_BAD;
          lo = 0;
        } else {
          len = (uint32_t)(hi - lo);
          mode = len <= LIST_STAGE ? RL_SMEM : RL_GLOBAL;
        }
      }
    }
    info[si] = make_uint4(mode, len, (uint32_t)lo, (uint32_t)(lo >> 32));
  }
  uint32_t mx = 0;
  for (uint32_t c = blockIdx.x * TPB + threadIdx.x; c < a.n_dst; c += stride)
    mx = max(mx, a.dst_orig[c]);
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(bound, mx);
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* red) {
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t t = 0;
  for (uint32_t w = 0; w < TPB / 32; ++w) t += red[w];
  return t;
}

// Sparse pass 1 for wide rows: the segment's kept cells and ballots, with
// decide()'s rules: a row without a list keeps nothing (ERR_NO_LIST), a bad
// list keeps nothing and is an error once a cell is within the bound.
__global__ void __launch_bounds__(TPB)
    k_tile_count_rows(TileIn a, uint32_t segs, uint32_t wpr, const uint4* __restrict__ info,
                      const uint32_t* __restrict__ bound, unsigned long long* __restrict__ cnt,
                      uint32_t* __restrict__ keep_bits, uint32_t* err) {
  __shared__ RowList rl;
  __shared__ uint32_t red[TPB / 32];
  const uint32_t si = blockIdx.x / segs, sg = blockIdx.x % segs;
  const uint32_t c_begin = sg * SEG, c_end = min(c_begin + SEG, a.n_dst);
  const uint32_t lane = threadIdx.x & 31;
  // the first step's durations load while the row's list is looked up
  const uint32_t* row = a.m + (uint64_t)si * a.n_dst;
  uint32_t dur[ITEMS];
#pragma unroll
  for (uint32_t j = 0; j < ITEMS; ++j) {
    const uint32_t col = c_begin + j * TPB + threadIdx.x;
    dur[j] = col < c_end ? row[col] : MAXV;
  }
  const uint4 ri = info[si];  // {mode, len, list offset (lo, hi words)}
  const uint32_t nbw = min(BITMAP_WORDS, (*bound >> 5) + 1);
  const uint32_t mode = ri.x, len = ri.y;
  const uint64_t lo = ri.z | ((uint64_t)ri.w << 32);
  if (mode == RL_MISSING && threadIdx.x == 0) atomicOr(err, ERR_NO_LIST);
  // uniform: every thread read the same row record
  if (mode == RL_SMEM) stage_row_list(rl, a.mask + lo, len, nbw);
  const uint32_t* lg = a.mask + lo;
  uint32_t* bits = keep_bits + (uint64_t)si * wpr;
  const bool listed = mode == RL_SMEM || mode == RL_GLOBAL;
  uint32_t c = 0;
  bool bad_hit = false;
  for (uint32_t b0 = c_begin; b0 < c_end; b0 += CELLS) {
    // the next step's durations are in flight while this step decides
    uint32_t nxt[ITEMS];
#pragma unroll
    for (uint32_t j = 0; j < ITEMS; ++j) {
      const uint32_t col = b0 + CELLS + j * TPB + threadIdx.x;
      nxt[j] = col < c_end ? row[col] : MAXV;
    }
    // in-bound cells' destination ids, all loads issued before any search
    bool inb[ITEMS];
    uint32_t od[ITEMS];
#pragma unroll
    for (uint32_t j = 0; j < ITEMS; ++j) {
      const uint32_t col = b0 + j * TPB + threadIdx.x;
      inb[j] = col < c_end && dur[j] <= a.threshold && dur[j] != MAXV;
      od[j] = inb[j] && listed ? a.dst_orig[col] : 0u;
    }
#pragma unroll
    for (uint32_t j = 0; j < ITEMS; ++j) {
      bool keep = false;
      if (inb[j]) {
        if (mode == RL_NONE) keep = true;
        else if (mode == RL_SMEM) keep = in_row_list(rl, len, nbw, od[j]);
        else if (mode == RL_GLOBAL) keep = in_list(lg, len, od[j]);
        else if (mode == RL_BAD) bad_hit = true;
      }
      const unsigned bal = __ballot_sync(0xFFFFFFFFu, keep);
      const uint32_t wcell = b0 + j * TPB + (threadIdx.x & ~31u);
      if (lane == 0 && wcell < c_end) bits[wcell / 32] = bal;
      c += keep;
      dur[j] = nxt[j];
    }
  }
  if (bad_hit) atomicOr(err, ERR_BAD_LIST);
  const uint32_t t = block_sum(c, red);
  if (threadIdx.x == 0) cnt[blockIdx.x] = t;
}

// k_tile_count_rows with 16-byte accesses (rows a multiple of 4 cells, the
// matrix and the destination ids 16-byte aligned): a thread takes 4
// consecutive cells per load and VEC loads per step, so each SM keeps twice
// the bytes in flight; the 4-cell keep bits of 8 lanes are OR-combined by
// shuffles into one ballot word.
constexpr uint32_t VEC = 4, CELLS4 = TPB * 4 * VEC;

__global__ void __launch_bounds__(TPB)
    k_tile_count_rows4(TileIn a, uint32_t segs, uint32_t wpr, const uint4* __restrict__ info,
                       const uint32_t* __restrict__ bound, unsigned long long* __restrict__ cnt,
                       uint32_t* __restrict__ keep_bits, uint32_t* err) {
  __shared__ RowList rl;
  __shared__ uint32_t red[TPB / 32];
  const uint32_t si = blockIdx.x / segs, sg = blockIdx.x % segs;
  const uint32_t c_begin = sg * SEG, c_end = min(c_begin + SEG, a.n_dst);
  const uint32_t lane = threadIdx.x & 31;
  const uint4* row4 = reinterpret_cast<const uint4*>(a.m + (uint64_t)si * a.n_dst);
  const uint4* od4 = reinterpret_cast<const uint4*>(a.dst_orig);
  // the first step's durations load while the row's list is looked up
  uint4 dur[VEC];
#pragma unroll
  for (uint32_t u = 0; u < VEC; ++u) {
    const uint32_t col = c_begin + (u * TPB + threadIdx.x) * 4;
    dur[u] = col < c_end ? row4[col / 4] : make_uint4(MAXV, MAXV, MAXV, MAXV);
  }
  const uint4 ri = info[si];  // {mode, len, list offset (lo, hi words)}
  const uint32_t nbw = min(BITMAP_WORDS, (*bound >> 5) + 1);
  const uint32_t mode = ri.x, len = ri.y;
  const uint64_t lo = ri.z | ((uint64_t)ri.w << 32);
  if (mode == RL_MISSING && threadIdx.x == 0) atomicOr(err, ERR_NO_LIST);
  // uniform: every thread read the same row record
  if (mode == RL_SMEM) stage_row_list(rl, a.mask + lo, len, nbw);
  const uint32_t* lg = a.mask + lo;
  uint32_t* bits = keep_bits + (uint64_t)si * wpr;
  // a cell is within the bound iff d <= thr1 (the u32::MAX sentinel never
  // is); cells past the segment read as the sentinel, so no column test
  const uint32_t thr1 = min(a.threshold, MAXV - 1);
  const bool listed = mode == RL_SMEM || mode == RL_GLOBAL;
  // staged lists whose ids all fall in the bitmap are tested branch-free
  const bool bitmap_only = mode == RL_SMEM && (*bound >> 5) < BITMAP_WORDS;
  const uint32_t lim = nbw * 32;
  uint32_t c = 0;
  bool bad_hit = false;
  for (uint32_t b0 = c_begin; b0 < c_end; b0 += CELLS4) {
    uint4 nxt[VEC];
#pragma unroll
    for (uint32_t u = 0; u < VEC; ++u) {
      const uint32_t col = b0 + CELLS4 + (u * TPB + threadIdx.x) * 4;
      nxt[u] = col < c_end ? row4[col / 4] : make_uint4(MAXV, MAXV, MAXV, MAXV);
    }
#pragma unroll
    for (uint32_t u = 0; u < VEC; ++u) {
      const uint32_t col = b0 + (u * TPB + threadIdx.x) * 4;  // < c_end or all four out
      const uint4 d = dur[u];
      const uint32_t inb = (uint32_t)(d.x <= thr1) | ((uint32_t)(d.y <= thr1) << 1) |
                           ((uint32_t)(d.z <= thr1) << 2) | ((uint32_t)(d.w <= thr1) << 3);
      uint32_t k4 = 0;
      if (mode == RL_NONE) {
        k4 = inb;
      } else if (bitmap_only) {
        // every destination id is below lim: one shared word per cell
        const uint4 o = col < c_end ? od4[col / 4] : make_uint4(0, 0, 0, 0);
        const uint32_t m4 = ((rl.bmp[o.x >> 5] >> (o.x & 31)) & 1u) |
                            (((rl.bmp[o.y >> 5] >> (o.y & 31)) & 1u) << 1) |
                            (((rl.bmp[o.z >> 5] >> (o.z & 31)) & 1u) << 2) |
                            (((rl.bmp[o.w >> 5] >> (o.w & 31)) & 1u) << 3);
        k4 = inb & m4;
      } else if (inb) {
        if (listed) {
          const uint4 o = od4[col / 4];
          const uint32_t ov[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
          for (uint32_t k = 0; k < 4; ++k)
            if (((inb >> k) & 1u) &&
                (mode == RL_SMEM ? (ov[k] < lim ? ((rl.bmp[ov[k] >> 5] >> (ov[k] & 31)) & 1u) != 0
                                                : in_list(rl.v, len, ov[k]))
                                 : in_list(lg, len, ov[k])))
              k4 |= 1u << k;
        } else if (mode == RL_BAD) {
          bad_hit = true;
        }
      }
      // lanes 8q .. 8q + 7 hold the 32 cells of ballot word q of this warp's 128
      uint32_t word = k4 << ((lane & 7) * 4);
      word |= __shfl_xor_sync(0xFFFFFFFFu, word, 1);
      word |= __shfl_xor_sync(0xFFFFFFFFu, word, 2);
      word |= __shfl_xor_sync(0xFFFFFFFFu, word, 4);
      const uint32_t wcell = b0 + (u * TPB + (threadIdx.x & ~31u)) * 4 + (lane >> 3) * 32;
      if ((lane & 7) == 0 && wcell < c_end) bits[wcell / 32] = word;
      c += __popc(k4);
      dur[u] = nxt[u];
    }
  }
  if (bad_hit) atomicOr(err, ERR_BAD_LIST);
  const uint32_t t = block_sum(c, red);
  if (threadIdx.x == 0) cnt[blockIdx.x] = t;
}

// Sparse pass 2 for wide rows: the segment's kept cells in order, a warp
// per row segment (no block barrier): 32 ballot words at a time (the next
// 32 loading meanwhile), a shuffle scan of their popcounts for each word's
// offset, then the kept cells word by word with a lane per cell (words
// without kept cells are skipped by ballot).
__global__ void __launch_bounds__(TPB)
    k_tile_write_rows(TileIn a, TileOut o, uint64_t nseg, uint32_t segs, uint32_t wpr,
                      const unsigned long long* __restrict__ pre,
                      const uint32_t* __restrict__ keep_bits) {
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t seg = (uint64_t)blockIdx.x * (TPB / 32) + wid;
  if (seg >= nseg) return;
  const unsigned long long k0 = pre[seg];
  if (pre[seg + 1] == k0) return;  // nothing kept in this segment (uniform per warp)
  const uint32_t si = (uint32_t)(seg / segs), sg = (uint32_t)(seg % segs);
  const uint32_t w_begin = sg * SEG_WORDS, w_end = min(w_begin + SEG_WORDS, wpr);
  const uint32_t* bits_row = keep_bits + (uint64_t)si * wpr;
  const uint32_t os = a.src_orig[si];
  const uint64_t row0 = (uint64_t)si * a.n_dst;
  uint32_t carry = 0;
  uint32_t bits = w_begin + lane < w_end ? bits_row[w_begin + lane] : 0u;
  for (uint32_t w0 = w_begin; w0 < w_end; w0 += 32) {
    const uint32_t wn = w0 + 32 + lane;
    const uint32_t nbits = wn < w_end ? bits_row[wn] : 0u;
    const uint32_t cn = __popc(bits);
    uint32_t inc = cn;
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, d);
      if (lane >= d) inc += y;
    }
    const uint32_t ex = carry + inc - cn;
    carry += __shfl_sync(0xFFFFFFFFu, inc, 31);
    uint32_t nz = __ballot_sync(0xFFFFFFFFu, bits != 0u);
    while (nz) {
      const uint32_t q = __ffs(nz) - 1;
      nz &= nz - 1;
      const uint32_t b = __shfl_sync(0xFFFFFFFFu, bits, q);
      const uint32_t off = __shfl_sync(0xFFFFFFFFu, ex, q);
      if ((b >> lane) & 1u) {
        const uint32_t col = (w0 + q) * 32 + lane;
        const uint64_t cell = row0 + col;
        put(a, o, k0 + off + __popc(b & ((1u << lane) - 1u)), cell, os, a.dst_orig[col],
            a.m[cell]);
      }
    }
    bits = nbits;
  }
}

// Sparse pass 2: the block's kept cells, in order, from pass 1's ballots:
// a thread's output slot is the block's offset plus the kept cells of the
// earlier words of the block (a two-warp shuffle scan of the word counts)
// and the lower lanes of its own word. A kept cell passed the bound and its
// radius list in pass 1, so its duration is written as read.
__global__ void __launch_bounds__(TPB)
    k_tile_write(TileIn a, TileOut o, uint64_t n, bool narrow,
                 const unsigned long long* __restrict__ pre,
                 const uint32_t* __restrict__ keep_bits) {
  constexpr uint32_t WORDS = CELLS / 32;
  static_assert(WORDS == 64 && TPB >= 64, "two warps scan the block's 64 ballot words");
  __shared__ uint32_t wpre[WORDS];
  __shared__ uint32_t half;
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned long long k0 = pre[blockIdx.x];
  if (pre[blockIdx.x + 1] == k0) return;  // nothing kept in this block (uniform)
  const uint64_t base = (uint64_t)blockIdx.x * CELLS;
  const uint64_t w0 = base / 32, nw = (n + 31) / 32;
  if (wid < 2) {
    const uint32_t w = wid * 32 + lane;
    const uint32_t c = w0 + w < nw ? __popc(keep_bits[w0 + w]) : 0;
    uint32_t inc = c;
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, d);
      if (lane >= d) inc += y;
    }
    wpre[w] = inc - c;
    if (wid == 0 && lane == 31) half = inc;
  }
  __syncthreads();
  for (uint32_t w = wid; w < WORDS; w += TPB / 32) {
    if (w0 + w >= nw) break;
    const uint32_t bits = keep_bits[w0 + w];
    if (!((bits >> lane) & 1u)) continue;
    const uint64_t i = (w0 + w) * 32 + lane;
    uint32_t si, di;
    split(i, a.n_dst, narrow, &si, &di);
    const uint32_t slot = wpre[w] + (w >= 32 ? half : 0u) + __popc(bits & ((1u << lane) - 1u));
    put(a, o, k0 + slot, i, a.src_orig[si], a.dst_orig[di], a.m[i]);
  }
}

// Scratch of the device variant and the host variant's copies, per device.
struct TileWs {
  std::mutex mu;
  cudaStream_t st = nullptr;
  void* buf[12] = {};
  size_t cap[12] = {};
};
TileWs& tile_ws(int device) {
  static TileWs ws[64];
  return ws[device];
}

template <class T>
cudaError_t ws_get(TileWs& ws, int i, size_t bytes, T** p) {
  bytes = std::max<size_t>(bytes, 16);
  if (ws.cap[i] < bytes) {
    if (ws.buf[i]) cudaFree(ws.buf[i]);
    ws.buf[i] = nullptr;
    ws.cap[i] = 0;
    const cudaError_t e = cudaMalloc(&ws.buf[i], bytes);
    if (e != cudaSuccess) return e;
    ws.cap[i] = bytes;
  }
  *p = reinterpret_cast<T*>(ws.buf[i]);
  return cudaSuccess;
}

bf_status check_args(uint32_t n_src, uint32_t n_dst, const void* m, const void* so,
                     const void* dor, const bf_tile_columns* out, uint64_t* n_rows,
                     const void* mask_off, const void* mask, uint64_t n_mask) {
  const bool cells = (uint64_t)n_src * n_dst != 0;
  if (!out || !n_rows || (cells && (!m || !so || !dor)) ||
      (cells && (!out->source_idx || !out->target_idx || !out->duration_ms || !out->distance_m)) ||
      (mask_off && n_mask && !mask)) {
    set_error("bf_tile_emit: null argument");
    return BF_ERR_INVALID;
  }
  return BF_OK;
}

// Emission from device inputs into device columns on `st`; *n_rows after a
// synchronisation of the stream.
bf_status emit_device(TileWs& ws, const TileIn& a, const TileOut& o, cudaStream_t st,
                      uint64_t* n_rows) {
  const uint64_t n = (uint64_t)a.n_src * a.n_dst;
  uint32_t* d_err = nullptr;
  BF_CUDA(ws_get(ws, 0, 4, &d_err));
  BF_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  uint64_t rows = 0;
  if (n && !a.sparse) {
    auto al = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
    const bool v4 = a.n_dst % 4 == 0 && al(a.m) && (!a.lat || al(a.lat)) && al(a.dst_orig) &&
                    al(o.s) && al(o.t) && al(o.du) && al(o.di);
    const uint32_t per_row = v4 ? a.n_dst / 4 : a.n_dst;
    const unsigned gx = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((per_row + TPB - 1) / TPB, 64));
    const unsigned gy = (unsigned)std::min<uint64_t>(a.n_src, 65535);
    if (v4)
      k_tile_dense4<<<dim3(gx, gy), TPB, 0, st>>>(a, o, d_err);
    else
      k_tile_dense<<<dim3(gx, gy), TPB, 0, st>>>(a, o, d_err);
    BF_CUDA(cudaGetLastError());
    rows = n;
  } else if (n && a.n_dst >= ROW_MIN &&
             (uint64_t)a.n_src * ((a.n_dst + SEG - 1) / SEG) <= 0x7FFFFFFFull) {
    const uint32_t segs = (a.n_dst + SEG - 1) / SEG, wpr = (a.n_dst + 31) / 32;
    const uint64_t nb = (uint64_t)a.n_src * segs;
    unsigned long long* d_cnt = nullptr;
    uint32_t* d_bits = nullptr;
    uint64_t* d_bsum = nullptr;
    const uint64_t nsb = (nb + SCAN_BLOCK - 1) / SCAN_BLOCK;
    BF_CUDA(ws_get(ws, 1, (2 * nb + 1) * 8, &d_cnt));
    BF_CUDA(ws_get(ws, 9, (uint64_t)a.n_src * wpr * 4, &d_bits));
    BF_CUDA(ws_get(ws, 10, (nsb + 2) * 8, &d_bsum));
    // per-row list records and the destination ids' range (bound[0], from
    // which the count blocks size their bitmaps)
    uint4* d_info = nullptr;
    BF_CUDA(ws_get(ws, 11, (uint64_t)a.n_src * 16 + 16, &d_info));
    uint32_t* d_bound = reinterpret_cast<uint32_t*>(d_info + a.n_src);
    BF_CUDA(cudaMemsetAsync(d_bound, 0, 4, st));
    const unsigned gi = (unsigned)std::min<uint64_t>(
        (std::max(a.n_src, a.n_dst) + TPB - 1) / TPB, 152 * 8);
    k_tile_rowinfo<<<gi, TPB, 0, st>>>(a, d_info, d_bound);
    auto al = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
    if (a.n_dst % 4 == 0 && al(a.m) && al(a.dst_orig))
      k_tile_count_rows4<<<(unsigned)nb, TPB, 0, st>>>(a, segs, wpr, d_info, d_bound, d_cnt, d_bits,
                                                       d_err);
    else
      k_tile_count_rows<<<(unsigned)nb, TPB, 0, st>>>(a, segs, wpr, d_info, d_bound, d_cnt, d_bits,
                                                      d_err);
    uint64_t* pre = reinterpret_cast<uint64_t*>(d_cnt + nb);
    k_scan_sums<uint64_t><<<(unsigned)nsb, SCAN_TPB, 0, st>>>(
        U64Val{reinterpret_cast<const uint64_t*>(d_cnt)}, nb, nullptr, d_bsum);
    k_scan_top<uint64_t><<<1, SCAN_TPB, 0, st>>>(d_bsum, (uint32_t)nsb);
    k_scan_out<uint64_t><<<(unsigned)nsb, SCAN_TPB, 0, st>>>(
        U64Val{reinterpret_cast<const uint64_t*>(d_cnt)}, nb, nullptr, d_bsum, (uint32_t)nsb,
        pre);
    k_tile_write_rows<<<(unsigned)((nb + TPB / 32 - 1) / (TPB / 32)), TPB, 0, st>>>(
        a, o, nb, segs, wpr, d_cnt + nb, d_bits);
    BF_CUDA(cudaGetLastError());
    BF_CUDA(cudaMemcpyAsync(&rows, d_cnt + 2 * nb, 8, cudaMemcpyDeviceToHost, st));
  } else if (n) {
    const uint64_t nb = (n + CELLS - 1) / CELLS;
    if (nb > 0x7FFFFFFFull) {
      set_error("bf_tile_emit: block too large");
      return BF_ERR_INVALID;
    }
    unsigned long long* d_cnt = nullptr;
    uint32_t* d_bits = nullptr;
    uint64_t* d_bsum = nullptr;
    const uint64_t nsb = (nb + SCAN_BLOCK - 1) / SCAN_BLOCK;
    BF_CUDA(ws_get(ws, 1, (2 * nb + 1) * 8, &d_cnt));
    BF_CUDA(ws_get(ws, 9, nb * (CELLS / 32) * 4, &d_bits));
    BF_CUDA(ws_get(ws, 10, (nsb + 2) * 8, &d_bsum));
    const bool narrow = n <= 0xFFFFFFFFull;
    k_tile_count<<<(unsigned)nb, TPB, 0, st>>>(a, n, narrow, d_cnt, d_bits, d_err);
    // exclusive scan of the block counts (total at [2 nb])
    uint64_t* pre = reinterpret_cast<uint64_t*>(d_cnt + nb);
    k_scan_sums<uint64_t><<<(unsigned)nsb, SCAN_TPB, 0, st>>>(
        U64Val{reinterpret_cast<const uint64_t*>(d_cnt)}, nb, nullptr, d_bsum);
    k_scan_top<uint64_t><<<1, SCAN_TPB, 0, st>>>(d_bsum, (uint32_t)nsb);
    k_scan_out<uint64_t><<<(unsigned)nsb, SCAN_TPB, 0, st>>>(
        U64Val{reinterpret_cast<const uint64_t*>(d_cnt)}, nb, nullptr, d_bsum, (uint32_t)nsb,
        pre);
    k_tile_write<<<(unsigned)nb, TPB, 0, st>>>(a, o, n, narrow, d_cnt + nb, d_bits);
    BF_CUDA(cudaGetLastError());
    BF_CUDA(cudaMemcpyAsync(&rows, d_cnt + 2 * nb, 8, cudaMemcpyDeviceToHost, st));
  }
  uint32_t err = 0;
  BF_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  if (err & ERR_NO_LIST) {
    set_error("bf_tile_emit: a source's original index has no radius list");
    return BF_ERR_INVALID;
  }
  if (err & ERR_BAD_LIST) {
    set_error("bf_tile_emit: a radius list's offsets decrease or run past the list array");
    return BF_ERR_INVALID;
  }
  *n_rows = rows;
  return BF_OK;
}

bf_status set_device(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || device >= 64) {
    cudaGetLastError();
    set_error("bf_tile_emit: no such device");
    return BF_ERR_INVALID;
  }
  if (cudaSetDevice(device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  return BF_OK;
}

}  // namespace

extern "C" {

bf_status bf_tile_emit_device(const uint32_t* d_matrix, const uint32_t* d_lat, uint32_t n_src,
                              uint32_t n_dst, const uint32_t* d_src_orig,
                              const uint32_t* d_dst_orig, uint32_t threshold,
                              const uint64_t* d_mask_off, const uint32_t* d_mask,
                              uint32_t n_mask_src, uint64_t n_mask, uint32_t sparse, int device,
                              void* stream, const bf_tile_columns* d_out, uint64_t* n_rows) {
  bf_status rc;
  if ((rc = check_args(n_src, n_dst, d_matrix, d_src_orig, d_dst_orig, d_out, n_rows, d_mask_off,
                       d_mask, n_mask)))
    return rc;
  if ((rc = set_device(device))) return rc;
  TileWs& ws = tile_ws(device);
  std::lock_guard<std::mutex> lk(ws.mu);
  if (!ws.st) BF_CUDA(cudaStreamCreateWithFlags(&ws.st, cudaStreamNonBlocking));
  cudaStream_t st = stream ? (cudaStream_t)stream : ws.st;
  const TileIn a{d_matrix, d_lat, n_src, n_dst, d_src_orig, d_dst_orig, threshold,
                 d_mask_off, d_mask, n_mask_src, n_mask, sparse};
  const TileOut o{d_out->source_idx, d_out->target_idx, d_out->duration_ms, d_out->distance_m};
  return emit_device(ws, a, o, st, n_rows);
}

bf_status bf_tile_emit(const uint32_t* matrix, const uint32_t* lat, uint32_t n_src,
                       uint32_t n_dst, const uint32_t* src_orig, const uint32_t* dst_orig,
                       uint32_t threshold, const uint64_t* mask_off, const uint32_t* mask,
                       uint32_t n_mask_src, uint32_t sparse, int device,
                       const bf_tile_columns* out, uint64_t* n_rows) {
  const uint64_t n_mask = mask_off ? mask_off[n_mask_src] : 0;
  bf_status rc;
  if ((rc = check_args(n_src, n_dst, matrix, src_orig, dst_orig, out, n_rows, mask_off, mask,
                       n_mask)))
    return rc;
  if (mask_off)
    for (uint32_t s = 0; s < n_mask_src; ++s)
      if (mask_off[s + 1] < mask_off[s]) {
        set_error("bf_tile_emit: radius list offsets must be non-decreasing");
        return BF_ERR_INVALID;
      }
  if ((rc = set_device(device))) return rc;
  TileWs& ws = tile_ws(device);
  std::lock_guard<std::mutex> lk(ws.mu);
  if (!ws.st) BF_CUDA(cudaStreamCreateWithFlags(&ws.st, cudaStreamNonBlocking));
  cudaStream_t st = ws.st;
  const uint64_t n = (uint64_t)n_src * n_dst;
  uint32_t *dm = nullptr, *dl = nullptr, *ds = nullptr, *dd = nullptr, *dmask = nullptr;
  uint64_t* dmoff = nullptr;
  uint32_t* dcol = nullptr;
  cudaError_t e = ws_get(ws, 2, n * 4, &dm);
  if (e == cudaSuccess && lat) e = ws_get(ws, 3, n * 4, &dl);
  if (e == cudaSuccess) e = ws_get(ws, 4, (uint64_t)n_src * 4, &ds);
  if (e == cudaSuccess) e = ws_get(ws, 5, (uint64_t)n_dst * 4, &dd);
  if (e == cudaSuccess && mask_off) e = ws_get(ws, 6, ((uint64_t)n_mask_src + 1) * 8, &dmoff);
  if (e == cudaSuccess && mask_off) e = ws_get(ws, 7, n_mask * 4, &dmask);
  if (e == cudaSuccess) e = ws_get(ws, 8, n * 16, &dcol);
  if (e != cudaSuccess) return cuda_status(e, "bf_tile_emit: device memory");
  auto up = [&](void* d, const void* h, uint64_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
  };
  up(dm, matrix, n * 4);
  if (lat) up(dl, lat, n * 4);
  up(ds, src_orig, (uint64_t)n_src * 4);
  up(dd, dst_orig, (uint64_t)n_dst * 4);
  if (mask_off) {
    up(dmoff, mask_off, ((uint64_t)n_mask_src + 1) * 8);
    up(dmask, mask, n_mask * 4);
  }
  if (e != cudaSuccess) return cuda_status(e, "bf_tile_emit: upload");
  const TileIn a{dm, lat ? dl : nullptr, n_src, n_dst, ds, dd, threshold,
                 mask_off ? dmoff : nullptr, dmask, n_mask_src, n_mask, sparse};
  const TileOut o{dcol, dcol + n, dcol + 2 * n, dcol + 3 * n};
  uint64_t rows = 0;
  if ((rc = emit_device(ws, a, o, st, &rows))) return rc;
  uint32_t* dst_cols[4] = {out->source_idx, out->target_idx, out->duration_ms, out->distance_m};
  for (int c = 0; c < 4 && rows; ++c)
    BF_CUDA(cudaMemcpyAsync(dst_cols[c], dcol + (uint64_t)c * n, rows * 4, cudaMemcpyDeviceToHost,
                            st));
  BF_CUDA(cudaStreamSynchronize(st));
  *n_rows = rows;
  return BF_OK;
}

void bf_tile_release(int device) {
  if (device < 0 || device >= 64) return;
  TileWs& ws = tile_ws(device);
  std::lock_guard<std::mutex> lk(ws.mu);
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (ws.st) cudaStreamSynchronize(ws.st);
  for (int i = 0; i < 12; ++i) {
    if (ws.buf[i]) cudaFree(ws.buf[i]);
    ws.buf[i] = nullptr;
    ws.cap[i] = 0;
  }
  if (ws.st) cudaStreamDestroy(ws.st);
  ws.st = nullptr;
}

}  // extern "C"
