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
#include <climits>
#include <cstdlib>
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

// Per isochrone (one block each): the minimum point corner, then the grid
// origin (minimum less three cells, as the reference) and the extreme cells
// of its points and anchor disk; also tags every segment with its isochrone.
struct Extent {
  double ox, oy;
  int32_t c0, r0, c1, r1;
  uint32_t has_points, pad;
};

__device__ __forceinline__ double block_min(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : INFINITY;
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ int block_minmax_i(int v, bool is_max, int* red) {
  for (int o = 16; o > 0; o >>= 1) {
    const int w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = is_max ? max(v, w) : min(v, w);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : (is_max ? INT_MIN : INT_MAX);
    for (int o = 16; o > 0; o >>= 1) {
      const int w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
      v = is_max ? max(v, w) : min(v, w);
    }
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const int r = red[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(256) k_extent(const double2* __restrict__ xy,
                                                const uint64_t* __restrict__ seg_pt,
                                                const uint64_t* __restrict__ iso_seg,
                                                const double* __restrict__ cell_m,
                                                const uint8_t* __restrict__ has_anchor,
                                                const double2* __restrict__ anchor,
                                                uint32_t* __restrict__ seg_iso,
                                                Extent* __restrict__ ext) {
  __shared__ double dred[8];
  __shared__ int ired[8];
  const uint32_t k = blockIdx.x;
  const uint64_t s0 = iso_seg[k], s1 = iso_seg[k + 1];
  for (uint64_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) seg_iso[s] = k;
  const uint64_t p0 = seg_pt[s0], p1 = seg_pt[s1];
  double mx = INFINITY, my = INFINITY;
  for (uint64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    mx = fmin(mx, xy[p].x);
    my = fmin(my, xy[p].y);
  }
  mx = block_min(mx, dred);
  my = block_min(my, dred);
  Extent e{};
  if (p1 == p0) {
    if (threadIdx.x == 0) ext[k] = e;
    return;
  }
  const double cell = cell_m[k];
  IsoDev g{};
  g.ox = __dsub_rn(mx, __dmul_rn(cell, 3.0));
  g.oy = __dsub_rn(my, __dmul_rn(cell, 3.0));
  g.cell = cell;
  int c0 = INT_MAX, r0 = INT_MAX, c1 = INT_MIN, r1 = INT_MIN;
  for (uint64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    int32_t c, r;
    cell_of(g, xy[p].x, xy[p].y, &c, &r);
    c0 = min(c0, c);
    r0 = min(r0, r);
    c1 = max(c1, c);
    r1 = max(r1, r);
  }
  if (threadIdx.x == 0 && has_anchor && has_anchor[k]) {
    int32_t c, r;
    cell_of(g, anchor[k].x, anchor[k].y, &c, &r);
    c0 = min(c0, c - 1);
    r0 = min(r0, r - 1);
    c1 = max(c1, c + 1);
    r1 = max(r1, r + 1);
  }
  c0 = block_minmax_i(c0, false, ired);
  r0 = block_minmax_i(r0, false, ired);
  c1 = block_minmax_i(c1, true, ired);
  r1 = block_minmax_i(r1, true, ired);
  if (threadIdx.x == 0) ext[k] = Extent{g.ox, g.oy, c0, r0, c1, r1, 1u, 0u};
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

// Raster layout from the per-isochrone extents: one more cell than the
// dilations can grow on every side; word offsets in isochrone order.
bool place(uint32_t n_iso, const Extent* ext, const double* cell_m, uint32_t dilation,
           bf_raster* ras, std::vector<IsoDev>& dev, uint64_t* total) {
  uint64_t woff = 0;
  dev.assign(n_iso, IsoDev{});
  for (uint32_t k = 0; k < n_iso; ++k) {
    bf_raster& R = ras[k];
    R = bf_raster{};
    IsoDev& g = dev[k];
    g.woff = woff;
    R.word_offset = woff;
    if (!ext[k].has_points) continue;
    const int64_t grow = (int64_t)dilation + 1;
    const int64_t c0 = (int64_t)ext[k].c0 - grow, r0 = (int64_t)ext[k].r0 - grow;
    const int64_t c1 = (int64_t)ext[k].c1 + grow, r1 = (int64_t)ext[k].r1 + grow;
    if (c0 < INT32_MIN || r0 < INT32_MIN || c1 > INT32_MAX || r1 > INT32_MAX) return false;
    g.ox = ext[k].ox;
    g.oy = ext[k].oy;
    g.cell = cell_m[k];
    g.col0 = (int32_t)c0;
    g.row0 = (int32_t)r0;
    g.wpr = (uint32_t)((c1 - c0 + 1 + 63) / 64);
    g.height = (uint32_t)(r1 - r0 + 1);
    R.col0 = g.col0;
    R.row0 = g.row0;
    R.width_words = g.wpr;
    R.height = g.height;
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
                             int device, bf_raster* rasters, uint64_t** words,
                             uint64_t* n_words) {
  if (words) *words = nullptr;
  if (!seg_pt || !iso_seg || !cell_m || !rasters || !n_words || (has_anchor && !anchor_xy)) {
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
  const uint64_t n_pts = seg_pt[n_seg];
  if (n_pts && !xy) {
    set_error("bf_contour_rasters: null points");
    return BF_ERR_INVALID;
  }
  std::vector<IsoDev> iso;
  uint64_t total = 0;
  if (!words) {  // layout only, on the host
    if (!layout(xy, seg_pt, iso_seg, n_iso, cell_m, has_anchor, anchor_xy, dilation, rasters, iso,
                &total)) {
      set_error("bf_contour_rasters: a raster extends beyond 32-bit cell coordinates");
      return BF_ERR_INVALID;
    }
    *n_words = total;
    return BF_OK;
  }
  if (cudaSetDevice(device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t st = nullptr;
  BF_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  std::vector<void*> bufs;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](auto** p, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc((void**)p, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess) bufs.push_back(*p);
  };
  auto done = [&](bf_status rc) {
    for (void* p : bufs) cudaFree(p);
    cudaStreamDestroy(st);
    return rc;
  };
  double2 *d_xy = nullptr, *d_anchor = nullptr;
  uint64_t *d_seg = nullptr, *d_iseg = nullptr;
  uint32_t *d_siso = nullptr, *d_err = nullptr;
  double* d_cell = nullptr;
  uint8_t* d_has = nullptr;
  Extent* d_ext = nullptr;
  IsoDev* d_iso = nullptr;
  alloc(&d_xy, n_pts * sizeof(double2));
  alloc(&d_seg, (n_seg + 1) * 8);
  alloc(&d_iseg, ((uint64_t)n_iso + 1) * 8);
  alloc(&d_siso, n_seg * 4);
  alloc(&d_cell, (uint64_t)n_iso * 8);
  alloc(&d_ext, (uint64_t)n_iso * sizeof(Extent));
  alloc(&d_iso, (uint64_t)n_iso * sizeof(IsoDev));
  alloc(&d_err, 4);
  if (has_anchor) {
    alloc(&d_has, n_iso);
    alloc(&d_anchor, (uint64_t)n_iso * 16);
  }
  if (e != cudaSuccess) return done(cuda_status(e, "bf_contour_rasters: device memory"));
  std::vector<Extent> ext(n_iso);
  auto stage1 = [&]() -> cudaError_t {
    cudaError_t r;
    if (n_pts && (r = cudaMemcpyAsync(d_xy, xy, n_pts * 16, cudaMemcpyHostToDevice, st))) return r;
    if ((r = cudaMemcpyAsync(d_seg, seg_pt, (n_seg + 1) * 8, cudaMemcpyHostToDevice, st))) return r;
    if ((r = cudaMemcpyAsync(d_iseg, iso_seg, ((uint64_t)n_iso + 1) * 8, cudaMemcpyHostToDevice, st)))
      return r;
    if (n_iso && (r = cudaMemcpyAsync(d_cell, cell_m, (uint64_t)n_iso * 8, cudaMemcpyHostToDevice, st)))
      return r;
    if (has_anchor && n_iso) {
      if ((r = cudaMemcpyAsync(d_has, has_anchor, n_iso, cudaMemcpyHostToDevice, st))) return r;
      if ((r = cudaMemcpyAsync(d_anchor, anchor_xy, (uint64_t)n_iso * 16, cudaMemcpyHostToDevice, st)))
        return r;
    }
    if (n_iso)
      k_extent<<<n_iso, 256, 0, st>>>(d_xy, d_seg, d_iseg, d_cell, d_has, d_anchor, d_siso, d_ext);
    if ((r = cudaGetLastError())) return r;
    if (n_iso && (r = cudaMemcpyAsync(ext.data(), d_ext, (uint64_t)n_iso * sizeof(Extent),
                                      cudaMemcpyDeviceToHost, st)))
      return r;
    return cudaStreamSynchronize(st);
  };
  if ((e = stage1()) != cudaSuccess) return done(cuda_status(e, "bf_contour_rasters: extents"));
  if (!place(n_iso, ext.data(), cell_m, dilation, rasters, iso, &total)) {
    set_error("bf_contour_rasters: a raster extends beyond 32-bit cell coordinates");
    return done(BF_ERR_INVALID);
  }
  *n_words = total;
  uint64_t* h_words = (uint64_t*)std::malloc(std::max<uint64_t>(total, 1) * 8);
  if (!h_words) {
    set_error("out of host memory");
    return done(BF_ERR_OOM);
  }
  unsigned long long *d_a = nullptr, *d_b = nullptr;
  alloc(&d_a, total * 8);
  alloc(&d_b, total * 8);
  if (e != cudaSuccess) {
    std::free(h_words);
    return done(cuda_status(e, "bf_contour_rasters: raster memory"));
  }
  auto stage2 = [&]() -> cudaError_t {
    cudaError_t r;
    if (n_iso && (r = cudaMemcpyAsync(d_iso, iso.data(), (uint64_t)n_iso * sizeof(IsoDev),
                                      cudaMemcpyHostToDevice, st)))
      return r;
    if ((r = cudaMemsetAsync(d_a, 0, std::max<uint64_t>(total, 1) * 8, st))) return r;
    if ((r = cudaMemsetAsync(d_err, 0, 4, st))) return r;
    if (n_seg) k_stamp<<<grid_of(n_seg), 256, 0, st>>>(n_seg, d_xy, d_seg, d_siso, d_iso, d_a, d_err);
    if (has_anchor && n_iso)
      k_anchor<<<(n_iso + 127) / 128, 128, 0, st>>>(n_iso, d_iso, d_has, d_anchor, d_a, d_err);
    unsigned long long *cur = d_a, *nxt = d_b;
    for (uint32_t i = 0; i < dilation && total; ++i) {
      k_morph<true><<<grid_of(total), 256, 0, st>>>(n_iso, d_iso, total, cur, nxt);
      std::swap(cur, nxt);
    }
    for (uint32_t i = 0; i < erosion && total; ++i) {
      k_morph<false><<<grid_of(total), 256, 0, st>>>(n_iso, d_iso, total, cur, nxt);
      std::swap(cur, nxt);
    }
    if ((r = cudaGetLastError())) return r;
    if (total && (r = cudaMemcpyAsync(h_words, cur, total * 8, cudaMemcpyDeviceToHost, st))) return r;
    return cudaStreamSynchronize(st);
  };
  e = stage2();
  uint32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&err, d_err, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess || err) {
    std::free(h_words);
    if (e != cudaSuccess) return done(cuda_status(e, "bf_contour_rasters"));
    set_error("bf_contour_rasters: a stamped cell fell outside its raster");
    return done(BF_ERR_DEVICE);
  }
  *words = h_words;
  return done(BF_OK);
}

void bf_contour_free(uint64_t* words) { std::free(words); }

}  // extern "C"
