// contour.cu — isochrone contour rasters on the GPU: steps 1-3 of the
// reference's sparse contour pipeline (route/src/range/sparse_contour.rs:
// 650-770) for a batch of isochrones: stamp the reachable segments
// (Bresenham between the cells of consecutive points, then every point),
// stamp the anchor's 3x3 disk, then 3x3 dilations and erosions.
//
// The reference keeps a sparse map of 64x64-cell tiles; here each isochrone
// owns one dense bit raster (rows of 64-cell words) covering its stamped
// cells plus one more cell than the dilations can grow. Outside cells read
// as zero, exactly like the reference's absent tiles, and the 3x3 operators
// are translation invariant, so the closed cell sets are identical. Cell
// indices are floor((x - origin) / cell) from the same doubles as the
// reference (a subtraction and a division, no contraction), so they agree
// bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "engine.cuh"

using namespace bf;

namespace {

struct IsoDev {
  double ox, oy, cell;
  int32_t col0, row0;
  uint32_t wpr, height;  // words per row, rows
  uint64_t woff;         // first word
};

__device__ __forceinline__ void cell_of(const IsoDev& g, double x, double y, int32_t* c,
                                        int32_t* r) {
  *c = (int32_t)floor(__ddiv_rn(__dsub_rn(x, g.ox), g.cell));
  *r = (int32_t)floor(__ddiv_rn(__dsub_rn(y, g.oy), g.cell));
}

__device__ __forceinline__ void set_cell(const IsoDev& g, int32_t c, int32_t r,
                                         unsigned long long* words, uint32_t* err) {
  const int64_t lc = (int64_t)c - g.col0, lr = (int64_t)r - g.row0;
  if (lc < 0 || lr < 0 || lc >= (int64_t)g.wpr * 64 || lr >= (int64_t)g.height) {
    atomicOr(err, 1u);  // outside the raster the layout computed: a bug, never a write
    return;
  }
  atomicOr(words + g.woff + (uint64_t)lr * g.wpr + (uint64_t)(lc >> 6), 1ull << (lc & 63));
}

// stamp_line (sparse_contour.rs:112-144) over every consecutive point pair
// of a segment, then every point of it: one thread per segment.
__global__ void k_stamp(uint64_t n_seg, const double2* __restrict__ xy,
                        const uint64_t* __restrict__ seg_pt, const uint32_t* __restrict__ seg_iso,
                        const IsoDev* __restrict__ iso, unsigned long long* __restrict__ words,
                        uint32_t* err) {
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n_seg;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const IsoDev g = iso[seg_iso[s]];
    const uint64_t p0 = seg_pt[s], p1 = seg_pt[s + 1];
    for (uint64_t p = p0; p + 1 < p1; ++p) {
      int32_t c0, r0, c1, r1;
      const double2 a = xy[p], b = xy[p + 1];
      cell_of(g, a.x, a.y, &c0, &r0);
      cell_of(g, b.x, b.y, &c1, &r1);
      const int32_t dx = abs(c1 - c0), dy = abs(r1 - r0);
      const int32_t sx = c0 < c1 ? 1 : -1, sy = r0 < r1 ? 1 : -1;
      int32_t e = dx - dy, c = c0, r = r0;
      for (int64_t guard = 0; guard <= (int64_t)dx + dy; ++guard) {  // dx + dy + 1 cells at most
        set_cell(g, c, r, words, err);
        if (c == c1 && r == r1) break;
        const int32_t e2 = 2 * e;
        if (e2 > -dy) {
          e -= dy;
          c += sx;
        }
        if (e2 < dx) {
          e += dx;
          r += sy;
        }
      }
    }
    for (uint64_t p = p0; p < p1; ++p) {
      int32_t c, r;
      cell_of(g, xy[p].x, xy[p].y, &c, &r);
      set_cell(g, c, r, words, err);
    }
  }
}

// The anchor's 3x3 disk (sparse_contour.rs:732-745).
__global__ void k_anchor(uint32_t n_iso, const IsoDev* __restrict__ iso,
                         const uint8_t* __restrict__ has_anchor, const double2* __restrict__ anchor,
                         unsigned long long* __restrict__ words, uint32_t* err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_iso || !has_anchor[k]) return;
  const IsoDev g = iso[k];
  if (g.height == 0) return;  // no segments: the reference returns no contour
  int32_t c, r;
  cell_of(g, anchor[k].x, anchor[k].y, &c, &r);
  for (int dc = -1; dc <= 1; ++dc)
    for (int dr = -1; dr <= 1; ++dr) set_cell(g, c + dc, r + dr, words, err);
}

// One 3x3 dilation (OR) or erosion (AND) over every raster word
// (dilate_sparse / erode_sparse, sparse_contour.rs:184-431): a word's
// horizontal pass takes the edge bits from its left and right words, the
// vertical pass combines the rows above and below; outside reads zero.
template <bool DILATE>
__global__ void k_morph(uint32_t n_iso, const IsoDev* __restrict__ iso, uint64_t total,
                        const unsigned long long* __restrict__ in,
                        unsigned long long* __restrict__ out) {
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < total;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = n_iso;  // isochrone owning word w
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (iso[mid].woff <= w)
        lo = mid;
      else
        hi = mid;
    }
    const IsoDev g = iso[lo];
    const uint64_t local = w - g.woff;
    const uint32_t r = (uint32_t)(local / g.wpr), j = (uint32_t)(local % g.wpr);
    auto at = [&](int64_t rr, int64_t jj) -> uint64_t {
      if (rr < 0 || rr >= g.height || jj < 0 || jj >= g.wpr) return 0;
      return in[g.woff + (uint64_t)rr * g.wpr + (uint64_t)jj];
    };
    auto horiz = [&](int64_t rr) -> uint64_t {
      const uint64_t row = at(rr, j), lb = (at(rr, (int64_t)j - 1) >> 63) & 1,
                     rb = (at(rr, (int64_t)j + 1) & 1) << 63;
      return DILATE ? (row | (row << 1) | (row >> 1) | lb | rb)
                    : (row & ((row << 1) | lb) & ((row >> 1) | rb));
    };
    const uint64_t a = horiz((int64_t)r - 1), c = horiz(r), b = horiz((int64_t)r + 1);
    out[w] = DILATE ? (a | c | b) : (a & c & b);
  }
}

unsigned grid_of(uint64_t n) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 152ull * 16));
}

// Host layout: grid origin and raster extent per isochrone (the same
// doubles and operation order as the reference's bounding box and margin).
bool layout(const double* xy, const uint64_t* seg_pt, const uint64_t* iso_seg, uint32_t n_iso,
            const double* cell_m, const uint8_t* has_anchor, const double* anchor_xy,
            uint32_t dilation, bf_raster* ras, std::vector<IsoDev>& dev, uint64_t* total) {
  uint64_t woff = 0;
  dev.resize(n_iso);
  for (uint32_t k = 0; k < n_iso; ++k) {
    const double cell = cell_m[k];
    double mnx = INFINITY, mny = INFINITY;
    for (uint64_t s = iso_seg[k]; s < iso_seg[k + 1]; ++s)
      for (uint64_t p = seg_pt[s]; p < seg_pt[s + 1]; ++p) {
        mnx = std::min(mnx, xy[2 * p]);
        mny = std::min(mny, xy[2 * p + 1]);
      }
    bf_raster& R = ras[k];
    R = bf_raster{};
    IsoDev& g = dev[k];
    g = IsoDev{};
    if (std::isinf(mnx)) {  // no points: an empty raster
      g.woff = woff;
      R.word_offset = woff;
      continue;
    }
    const double margin = cell * 3.0;
    g.ox = mnx - margin;
    g.oy = mny - margin;
    g.cell = cell;
    int64_t c0 = INT64_MAX, r0 = INT64_MAX, c1 = INT64_MIN, r1 = INT64_MIN;
    auto take = [&](double x, double y, int d) {
      const int64_t c = (int64_t)(int32_t)std::floor((x - g.ox) / cell);
      const int64_t r = (int64_t)(int32_t)std::floor((y - g.oy) / cell);
      c0 = std::min(c0, c - d);
      r0 = std::min(r0, r - d);
      c1 = std::max(c1, c + d);
      r1 = std::max(r1, r + d);
    };
    for (uint64_t s = iso_seg[k]; s < iso_seg[k + 1]; ++s)
      for (uint64_t p = seg_pt[s]; p < seg_pt[s + 1]; ++p) take(xy[2 * p], xy[2 * p + 1], 0);
    if (has_anchor && has_anchor[k]) take(anchor_xy[2 * k], anchor_xy[2 * k + 1], 1);
    const int64_t grow = (int64_t)dilation + 1;
    c0 -= grow;
    r0 -= grow;
    c1 += grow;
    r1 += grow;
    if (c0 < INT32_MIN || r0 < INT32_MIN || c1 > INT32_MAX || r1 > INT32_MAX) return false;
    g.col0 = (int32_t)c0;
    g.row0 = (int32_t)r0;
    g.wpr = (uint32_t)((c1 - c0 + 1 + 63) / 64);
    g.height = (uint32_t)(r1 - r0 + 1);
    g.woff = woff;
    R.col0 = g.col0;
    R.row0 = g.row0;
    R.width_words = g.wpr;
    R.height = g.height;
    R.word_offset = woff;
    R.origin_x = g.ox;
    R.origin_y = g.oy;
    woff += (uint64_t)g.wpr * g.height;
  }
  *total = woff;
  return true;
}

}  // namespace

extern "C" {

bf_status bf_contour_rasters(const double* xy, const uint64_t* seg_pt, const uint64_t* iso_seg,
                             uint32_t n_iso, const double* cell_m, const uint8_t* has_anchor,
                             const double* anchor_xy, uint32_t dilation, uint32_t erosion,
                             int device, bf_raster* rasters, uint64_t* words, uint64_t cap_words,
                             uint64_t* n_words) {
  if (!seg_pt || !iso_seg || !cell_m || !rasters || !n_words || (n_iso && !xy) ||
      (has_anchor && !anchor_xy)) {
    set_error("bf_contour_rasters: null argument");
    return BF_ERR_INVALID;
  }
  for (uint32_t k = 0; k < n_iso; ++k)
    if (iso_seg[k + 1] < iso_seg[k] || !(cell_m[k] > 0) || std::isinf(cell_m[k])) {
      set_error("bf_contour_rasters: iso_seg must be non-decreasing and cell sizes positive");
      return BF_ERR_INVALID;
    }
  const uint64_t n_seg = iso_seg[n_iso];
  for (uint64_t s = 0; s < n_seg; ++s)
    if (seg_pt[s + 1] < seg_pt[s]) {
      set_error("bf_contour_rasters: seg_pt must be non-decreasing");
      return BF_ERR_INVALID;
    }
  std::vector<IsoDev> iso;
  uint64_t total = 0;
  if (!layout(xy, seg_pt, iso_seg, n_iso, cell_m, has_anchor, anchor_xy, dilation, rasters, iso,
              &total)) {
    set_error("bf_contour_rasters: a raster extends beyond 32-bit cell coordinates");
    return BF_ERR_INVALID;
  }
  *n_words = total;
  if (!words || cap_words < total || total == 0) {
    if (words && total) std::fill(words, words + std::min(cap_words, total), 0ull);
    return BF_OK;  // layout only: call again with room for *n_words words
  }
  if (cudaSetDevice(device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  const uint64_t n_pts = seg_pt[n_seg];
  std::vector<uint32_t> seg_iso(n_seg);
  for (uint32_t k = 0; k < n_iso; ++k)
    for (uint64_t s = iso_seg[k]; s < iso_seg[k + 1]; ++s) seg_iso[s] = k;
  cudaStream_t st = nullptr;
  BF_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  void* buf[8] = {};
  auto cleanup = [&]() {
    for (void* p : buf)
      if (p) cudaFree(p);
    cudaStreamDestroy(st);
  };
  double2* d_xy = nullptr;
  uint64_t* d_seg = nullptr;
  uint32_t *d_siso = nullptr, *d_err = nullptr;
  IsoDev* d_iso = nullptr;
  uint8_t* d_has = nullptr;
  double2* d_anchor = nullptr;
  unsigned long long *d_a = nullptr, *d_b = nullptr;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes, int slot) {
    if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess) buf[slot] = *p;
  };
  alloc((void**)&d_xy, n_pts * sizeof(double2), 0);
  alloc((void**)&d_seg, (n_seg + 1) * 8, 1);
  alloc((void**)&d_siso, n_seg * 4 + 4, 2);
  alloc((void**)&d_iso, n_iso * sizeof(IsoDev), 3);
  alloc((void**)&d_a, total * 8, 4);
  alloc((void**)&d_b, total * 8, 5);
  alloc((void**)&d_err, 4, 6);
  if (has_anchor) {
    alloc((void**)&d_has, n_iso, 7);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_anchor, std::max<size_t>(n_iso * 16, 16));
  }
  if (e != cudaSuccess) {
    if (d_anchor) cudaFree(d_anchor);
    cleanup();
    return cuda_status(e, "bf_contour_rasters: device memory");
  }
  auto run = [&]() -> cudaError_t {
    cudaError_t r;
    if ((r = cudaMemcpyAsync(d_xy, xy, n_pts * 16, cudaMemcpyHostToDevice, st))) return r;
    if ((r = cudaMemcpyAsync(d_seg, seg_pt, (n_seg + 1) * 8, cudaMemcpyHostToDevice, st))) return r;
    if (n_seg && (r = cudaMemcpyAsync(d_siso, seg_iso.data(), n_seg * 4, cudaMemcpyHostToDevice, st)))
      return r;
    if ((r = cudaMemcpyAsync(d_iso, iso.data(), n_iso * sizeof(IsoDev), cudaMemcpyHostToDevice, st)))
      return r;
    if ((r = cudaMemsetAsync(d_a, 0, total * 8, st))) return r;
    if ((r = cudaMemsetAsync(d_err, 0, 4, st))) return r;
    if (n_seg) k_stamp<<<grid_of(n_seg), 256, 0, st>>>(n_seg, d_xy, d_seg, d_siso, d_iso, d_a, d_err);
    if (has_anchor) {
      if ((r = cudaMemcpyAsync(d_has, has_anchor, n_iso, cudaMemcpyHostToDevice, st))) return r;
      if ((r = cudaMemcpyAsync(d_anchor, anchor_xy, n_iso * 16, cudaMemcpyHostToDevice, st))) return r;
      k_anchor<<<(n_iso + 127) / 128, 128, 0, st>>>(n_iso, d_iso, d_has, d_anchor, d_a, d_err);
    }
    unsigned long long *cur = d_a, *nxt = d_b;
    for (uint32_t i = 0; i < dilation; ++i) {
      k_morph<true><<<grid_of(total), 256, 0, st>>>(n_iso, d_iso, total, cur, nxt);
      std::swap(cur, nxt);
    }
    for (uint32_t i = 0; i < erosion; ++i) {
      k_morph<false><<<grid_of(total), 256, 0, st>>>(n_iso, d_iso, total, cur, nxt);
      std::swap(cur, nxt);
    }
    if ((r = cudaGetLastError())) return r;
    if ((r = cudaMemcpyAsync(words, cur, total * 8, cudaMemcpyDeviceToHost, st))) return r;
    return cudaStreamSynchronize(st);
  };
  e = run();
  uint32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&err, d_err, 4, cudaMemcpyDeviceToHost);
  if (d_anchor) cudaFree(d_anchor);
  cleanup();
  if (e != cudaSuccess) return cuda_status(e, "bf_contour_rasters");
  if (err) {
    set_error("bf_contour_rasters: a stamped cell fell outside its raster");
    return BF_ERR_DEVICE;
  }
  return BF_OK;
}

}  // extern "C"
