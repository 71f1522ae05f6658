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
// four column writes coalesced. Sparse: an order-preserving compaction - per
// block of 2048 cells a count and the kept-cell ballots (radius lists of the
// block's rows searched in shared memory), a device-wide scan of the counts,
// then an ordered write of the kept cells only.
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

// Radius lists of the (at most two) rows a count block spans, staged in
// shared memory when each holds at most LIST_STAGE entries: the in-bound
// cells then search them there instead of through a chain of global loads.
constexpr uint32_t LIST_STAGE = 4096;
struct ListStage {
  uint32_t v[2][LIST_STAGE];
  uint32_t len[2];
  uint32_t row0;
  int ok;
};

// Stages the lists of rows [si0, si1] (si1 - si0 <= 1) when both are valid
// and short enough; a row with a bad or missing list is left to decide()
// (which reports it). Returns true when the block searches shared memory.
__device__ __forceinline__ bool stage_lists(const TileIn& a, uint32_t si0, uint32_t si1,
                                            ListStage& ls) {
  if (threadIdx.x == 0) {
    int ok = si1 - si0 <= 1;
    for (uint32_t r = 0; ok && r <= si1 - si0; ++r) {
      const uint32_t os = a.src_orig[si0 + r];
      if (os >= a.n_mask_src) {
        ok = 0;
        break;
      }
      const uint64_t lo = a.mask_off[os], hi = a.mask_off[os + 1];
      if (hi < lo || hi > a.n_mask || hi - lo > LIST_STAGE) {
        ok = 0;
        break;
      }
      ls.len[r] = (uint32_t)(hi - lo);
    }
    ls.row0 = si0;
    ls.ok = ok;
  }
  __syncthreads();
  if (!ls.ok) return false;
  for (uint32_t r = 0; r <= si1 - si0; ++r) {
    const uint32_t* src = a.mask + a.mask_off[a.src_orig[si0 + r]];
    for (uint32_t k = threadIdx.x; k < ls.len[r]; k += blockDim.x) ls.v[r][k] = src[k];
  }
  __syncthreads();
  return true;
}

// Sparse pass 1: per block the kept cells, per (step, warp) the ballot of
// kept cells (bit lane of word (cell / 32)); rows and columns advance by
// TPB cells a step instead of a division per cell. With a radius mask, the
// lists of the block's rows are searched in shared memory when they fit.
__global__ void __launch_bounds__(TPB)
    k_tile_count(TileIn a, uint64_t n, bool narrow, unsigned long long* __restrict__ cnt,
                 uint32_t* __restrict__ keep_bits, uint32_t* err) {
  __shared__ uint32_t red[TPB / 32];
  __shared__ ListStage ls;
  const uint64_t base = (uint64_t)blockIdx.x * CELLS;
  uint32_t c = 0, si = 0, di = 0;
  split(base + threadIdx.x, a.n_dst, narrow, &si, &di);
  uint32_t dur[ITEMS];  // the block's durations, all loads in flight before any decision
#pragma unroll
  for (uint32_t j = 0; j < ITEMS; ++j) {
    const uint64_t i = base + (uint64_t)j * TPB + threadIdx.x;
    dur[j] = i < n ? a.m[i] : MAXV;
  }
  bool staged = false;
  if (a.mask_off && a.n_dst >= TPB) {
    uint32_t s0, s1, d0, d1;
    split(base, a.n_dst, narrow, &s0, &d0);
    split(min(base + CELLS, n) - 1, a.n_dst, narrow, &s1, &d1);
    staged = stage_lists(a, s0, s1, ls);
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
    if (i < n) {
      if (staged) {
        // decide() with the row's list read from shared memory
        const uint32_t d = dur[j];
        if (d <= a.threshold && d != MAXV) {
          const uint32_t r = si - ls.row0;
          keep = in_list(ls.v[r], ls.len[r], a.dst_orig[di]);
        }
      } else {
        keep = decide(a, dur[j], a.src_orig[si], a.dst_orig[di], err) != MAXV;
      }
    }
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
