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
#include <tuple>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <mutex>
#include <string>
#include <type_traits>
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
// of a segment, and every point of it: one thread per segment, each point's
// cell computed once (two IEEE double divisions), the line drawn from the
// previous point's cell. Point ranges are clamped to the points given.
__global__ void k_stamp(uint64_t n_seg, uint64_t n_pts, const double2* __restrict__ xy,
                        const uint64_t* __restrict__ seg_pt, const uint32_t* __restrict__ seg_iso,
                        const IsoDev* __restrict__ iso, unsigned long long* __restrict__ words,
                        uint32_t* err) {
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n_seg;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const IsoDev g = iso[seg_iso[s]];
    const uint64_t p1 = min(seg_pt[s + 1], n_pts), p0 = min(seg_pt[s], p1);
    int32_t pc = 0, pr = 0;
    for (uint64_t p = p0; p < p1; ++p) {
      int32_t c1, r1;
      const double2 q = xy[p];
      cell_of(g, q.x, q.y, &c1, &r1);
      set_cell(g, c1, r1, words, err);
      if (p > p0) {
        const int32_t c0 = pc, r0 = pr;
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
      pc = c1;
      pr = r1;
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

// Extents: the grid origin is each isochrone's minimum corner less three
// cells (as the reference); cell indices floor((x - origin) / cell) are
// monotone in x and y, so the extreme cells are those of the extreme
// coordinates. Chunked min / max partials first (EXT_CHUNKS blocks per
// isochrone, which also tag segments with their isochrone and check the
// segment offsets), then one thread per isochrone.
constexpr uint32_t EXT_CHUNKS = 32;

struct MinMax {
  double x0, y0, x1, y1;  // minimum and maximum coordinates
};

struct Extent {
  double ox, oy;
  int32_t c0, r0, c1, r1;
  uint32_t has_points, pad;
};

__device__ __forceinline__ double warp_min(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}

__global__ void __launch_bounds__(256) k_minmax(uint64_t n_pts, const double2* __restrict__ xy,
                                                const uint64_t* __restrict__ seg_pt,
                                                const uint64_t* __restrict__ iso_seg,
                                                uint32_t* __restrict__ seg_iso,
                                                MinMax* __restrict__ part, uint32_t* err) {
  __shared__ MinMax red[8];
  const uint32_t k = blockIdx.x / EXT_CHUNKS, ch = blockIdx.x % EXT_CHUNKS;
  const uint64_t s0 = iso_seg[k], s1 = iso_seg[k + 1];
  const uint64_t sa = s0 + (s1 - s0) * ch / EXT_CHUNKS, sb = s0 + (s1 - s0) * (ch + 1) / EXT_CHUNKS;
  for (uint64_t s = sa + threadIdx.x; s < sb; s += blockDim.x) {
    seg_iso[s] = k;
    if (seg_pt[s + 1] < seg_pt[s] || seg_pt[s + 1] > n_pts) atomicOr(err, 2u);
  }
  const uint64_t q1 = min(seg_pt[s1], n_pts), q0 = min(seg_pt[s0], q1);
  const uint64_t pa = q0 + (q1 - q0) * ch / EXT_CHUNKS, pb = q0 + (q1 - q0) * (ch + 1) / EXT_CHUNKS;
  double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  for (uint64_t p = pa + threadIdx.x; p < pb; p += blockDim.x) {
    const double2 q = xy[p];
    mnx = fmin(mnx, q.x);
    mny = fmin(mny, q.y);
    mxx = fmax(mxx, q.x);
    mxy = fmax(mxy, q.y);
  }
  mnx = warp_min(mnx);
  mny = warp_min(mny);
  mxx = warp_max(mxx);
  mxy = warp_max(mxy);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = MinMax{mnx, mny, mxx, mxy};
  __syncthreads();
  if (threadIdx.x == 0) {
    MinMax r = red[0];
    for (uint32_t w = 1; w < (blockDim.x >> 5); ++w) {
      r.x0 = fmin(r.x0, red[w].x0);
      r.y0 = fmin(r.y0, red[w].y0);
      r.x1 = fmax(r.x1, red[w].x1);
      r.y1 = fmax(r.y1, red[w].y1);
    }
    part[blockIdx.x] = r;
  }
}

__global__ void k_extent(uint32_t n_iso, const MinMax* __restrict__ part,
                         const double* __restrict__ cell_m, const uint8_t* __restrict__ has_anchor,
                         const double2* __restrict__ anchor, Extent* __restrict__ ext) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_iso) return;
  MinMax m = part[(uint64_t)k * EXT_CHUNKS];
  for (uint32_t c = 1; c < EXT_CHUNKS; ++c) {
    const MinMax q = part[(uint64_t)k * EXT_CHUNKS + c];
    m.x0 = fmin(m.x0, q.x0);
    m.y0 = fmin(m.y0, q.y0);
    m.x1 = fmax(m.x1, q.x1);
    m.y1 = fmax(m.y1, q.y1);
  }
  Extent e{};
  if (isinf(m.x0)) {
    ext[k] = e;
    return;
  }
  IsoDev g{};
  g.cell = cell_m[k];
  g.ox = __dsub_rn(m.x0, __dmul_rn(g.cell, 3.0));
  g.oy = __dsub_rn(m.y0, __dmul_rn(g.cell, 3.0));
  int32_t c0, r0, c1, r1;
  cell_of(g, m.x0, m.y0, &c0, &r0);
  cell_of(g, m.x1, m.y1, &c1, &r1);
  if (has_anchor && has_anchor[k]) {
    int32_t c, r;
    cell_of(g, anchor[k].x, anchor[k].y, &c, &r);
    c0 = min(c0, c - 1);
    r0 = min(r0, r - 1);
    c1 = max(c1, c + 1);
    r1 = max(r1, r + 1);
  }
  ext[k] = Extent{g.ox, g.oy, c0, r0, c1, r1, 1u, 0u};
}

// Device buffers and stream of bf_contour_rasters, kept per device across
// calls (grow-only; calls on one device are serialised by the mutex).
enum Slot {
  S_XY, S_SEG, S_ISEG, S_SISO, S_CELL, S_EXT, S_PART, S_ISO, S_ERR, S_HAS, S_ANCH, S_A, S_B,
  S_BLK, S_LANE, S_CUT, S_CUTXY, S_THR, N_SLOTS
};
struct Workspace {
  std::mutex mu;
  cudaStream_t st = nullptr;
  void* buf[N_SLOTS] = {};
  size_t cap[N_SLOTS] = {};
};
Workspace& workspace(int device) {
  static Workspace ws[64];
  return ws[device];
}

// Slot i of the workspace with room for `bytes` (grown by a quarter when it
// has to grow).
template <class T>
cudaError_t ws_get(Workspace& ws, int i, size_t bytes, T** p) {
  bytes = std::max<size_t>(bytes, 16);
  if (ws.cap[i] < bytes) {
    if (ws.buf[i]) cudaFree(ws.buf[i]);
    ws.buf[i] = nullptr;
    ws.cap[i] = 0;
    const size_t want = bytes + bytes / 4;
    const cudaError_t e = cudaMalloc(&ws.buf[i], want);
    if (e != cudaSuccess) return e;
    ws.cap[i] = want;
  }
  *p = reinterpret_cast<T*>(ws.buf[i]);
  return cudaSuccess;
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

namespace {

// Extents, layout, stamping, closing and download for a batch whose points,
// segment offsets and per-isochrone segment offsets are on the device
// (d_xy, d_seg, d_iseg); host arrays for the rest. The caller holds the
// workspace's lock; everything runs on `st`.
bf_status rasters_core(Workspace& ws, cudaStream_t st, const double2* d_xy, const uint64_t* d_seg,
                       const uint64_t* d_iseg, uint64_t n_seg, uint64_t n_pts, uint32_t n_iso,
                       const double* cell_m, const uint8_t* has_anchor, const double* anchor_xy,
                       uint32_t dilation, uint32_t erosion, bf_raster* rasters, uint64_t** words,
                       uint64_t* n_words, const uint64_t** d_words_out = nullptr) {
  cudaError_t e = cudaSuccess;
  uint32_t *d_siso = nullptr, *d_err = nullptr;
  double* d_cell = nullptr;
  uint8_t* d_has = nullptr;
  double2* d_anchor = nullptr;
  Extent* d_ext = nullptr;
  IsoDev* d_iso = nullptr;
  MinMax* d_part = nullptr;
  auto get = [&](int i, size_t bytes, auto** p) {
    if (e == cudaSuccess) e = ws_get(ws, i, bytes, p);
  };
  get(S_SISO, n_seg * 4, &d_siso);
  get(S_CELL, (uint64_t)n_iso * 8, &d_cell);
  get(S_EXT, (uint64_t)n_iso * sizeof(Extent), &d_ext);
  get(S_PART, (uint64_t)n_iso * EXT_CHUNKS * sizeof(MinMax), &d_part);
  get(S_ISO, (uint64_t)n_iso * sizeof(IsoDev), &d_iso);
  get(S_ERR, 4, &d_err);
  get(S_HAS, n_iso, &d_has);
  get(S_ANCH, (uint64_t)n_iso * 16, &d_anchor);
  if (e != cudaSuccess) return cuda_status(e, "bf_contour_rasters: device memory");
  std::vector<Extent> ext(n_iso);
  auto stage1 = [&]() -> cudaError_t {
    cudaError_t r;
    if (n_iso && (r = cudaMemcpyAsync(d_cell, cell_m, (uint64_t)n_iso * 8, cudaMemcpyHostToDevice, st)))
      return r;
    if (has_anchor && n_iso) {
      if ((r = cudaMemcpyAsync(d_has, has_anchor, n_iso, cudaMemcpyHostToDevice, st))) return r;
      if ((r = cudaMemcpyAsync(d_anchor, anchor_xy, (uint64_t)n_iso * 16, cudaMemcpyHostToDevice, st)))
        return r;
    }
    if ((r = cudaMemsetAsync(d_err, 0, 4, st))) return r;
    if (n_iso) {
      k_minmax<<<n_iso * EXT_CHUNKS, 256, 0, st>>>(n_pts, d_xy, d_seg, d_iseg, d_siso, d_part, d_err);
      k_extent<<<(n_iso + 127) / 128, 128, 0, st>>>(n_iso, d_part, d_cell,
                                                     has_anchor ? d_has : nullptr, d_anchor, d_ext);
    }
    if ((r = cudaGetLastError())) return r;
    if (n_iso && (r = cudaMemcpyAsync(ext.data(), d_ext, (uint64_t)n_iso * sizeof(Extent),
                                      cudaMemcpyDeviceToHost, st)))
      return r;
    return cudaStreamSynchronize(st);
  };
  if ((e = stage1()) != cudaSuccess) return cuda_status(e, "bf_contour_rasters: extents");
  {
    uint32_t verr = 0;
    if ((e = cudaMemcpy(&verr, d_err, 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
      return cuda_status(e, "bf_contour_rasters: extents");
    if (verr & 2u) {
      set_error("bf_contour_rasters: seg_pt must be non-decreasing");
      return BF_ERR_INVALID;
    }
  }
  std::vector<IsoDev> iso;
  uint64_t total = 0;
  if (!place(n_iso, ext.data(), cell_m, dilation, rasters, iso, &total)) {
    set_error("bf_contour_rasters: a raster extends beyond 32-bit cell coordinates");
    return BF_ERR_INVALID;
  }
  *n_words = total;
  // with d_words_out the closed rasters stay on the device (in the
  // workspace, valid until its next use) and nothing is downloaded
  uint64_t* h_words =
      d_words_out ? nullptr : (uint64_t*)std::malloc(std::max<uint64_t>(total, 1) * 8);
  if (!h_words && !d_words_out) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  unsigned long long *d_a = nullptr, *d_b = nullptr;
  get(S_A, total * 8, &d_a);
  get(S_B, total * 8, &d_b);
  if (e != cudaSuccess) {
    std::free(h_words);
    return cuda_status(e, "bf_contour_rasters: raster memory");
  }
  auto stage2 = [&]() -> cudaError_t {
    cudaError_t r;
    if (n_iso && (r = cudaMemcpyAsync(d_iso, iso.data(), (uint64_t)n_iso * sizeof(IsoDev),
                                      cudaMemcpyHostToDevice, st)))
      return r;
    if ((r = cudaMemsetAsync(d_a, 0, std::max<uint64_t>(total, 1) * 8, st))) return r;
    if ((r = cudaMemsetAsync(d_err, 0, 4, st))) return r;
    if (n_seg)
      k_stamp<<<grid_of(n_seg), 256, 0, st>>>(n_seg, n_pts, d_xy, d_seg, d_siso, d_iso, d_a, d_err);
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
    if (d_words_out) {
      *d_words_out = reinterpret_cast<const uint64_t*>(cur);
    } else if (total && (r = cudaMemcpyAsync(h_words, cur, total * 8, cudaMemcpyDeviceToHost, st))) {
      return r;
    }
    return cudaStreamSynchronize(st);
  };
  e = stage2();
  uint32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&err, d_err, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess || err) {
    std::free(h_words);
    if (e != cudaSuccess) return cuda_status(e, "bf_contour_rasters");
    set_error("bf_contour_rasters: a stamped cell fell outside its raster");
    return BF_ERR_DEVICE;
  }
  if (words) *words = h_words;
  return BF_OK;
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
  const uint64_t n_pts = seg_pt[n_seg];  // segment offsets are checked with the extents
  if (n_pts && !xy) {
    set_error("bf_contour_rasters: null points");
    return BF_ERR_INVALID;
  }
  if (!words) {  // layout only, on the host
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
    return BF_OK;
  }
  if (cudaSetDevice(device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || device >= 64) {
    cudaGetLastError();
    set_error("bf_contour_rasters: no such device");
    return BF_ERR_INVALID;
  }
  // per-device workspace kept across calls: one stream, grow-only buffers
  Workspace& ws = workspace(device);
  std::lock_guard<std::mutex> lk(ws.mu);
  if (!ws.st) BF_CUDA(cudaStreamCreateWithFlags(&ws.st, cudaStreamNonBlocking));
  cudaStream_t st = ws.st;
  double2* d_xy = nullptr;
  uint64_t *d_seg = nullptr, *d_iseg = nullptr;
  cudaError_t e = ws_get(ws, S_XY, n_pts * sizeof(double2), &d_xy);
  if (e == cudaSuccess) e = ws_get(ws, S_SEG, (n_seg + 1) * 8, &d_seg);
  if (e == cudaSuccess) e = ws_get(ws, S_ISEG, ((uint64_t)n_iso + 1) * 8, &d_iseg);
  if (e == cudaSuccess && n_pts) e = cudaMemcpyAsync(d_xy, xy, n_pts * 16, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_seg, seg_pt, (n_seg + 1) * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_iseg, iso_seg, ((uint64_t)n_iso + 1) * 8, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "bf_contour_rasters: upload");
  return rasters_core(ws, st, d_xy, d_seg, d_iseg, n_seg, n_pts, n_iso, cell_m, has_anchor,
                      anchor_xy, dilation, erosion, rasters, words, n_words);
}

void bf_contour_free(uint64_t* words) { std::free(words); }

void bf_contour_release(int device) {
  if (device < 0 || device >= 64) return;
  Workspace& ws = workspace(device);
  std::lock_guard<std::mutex> lk(ws.mu);
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (ws.st) cudaStreamSynchronize(ws.st);
  for (int i = 0; i < N_SLOTS; ++i) {
    if (ws.buf[i]) cudaFree(ws.buf[i]);
    ws.buf[i] = nullptr;
    ws.cap[i] = 0;
  }
  if (ws.st) cudaStreamDestroy(ws.st);
  ws.st = nullptr;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Steps 4-5 (sparse_contour.rs:770-1183): boundary tracing with cell-centre
// vertices, the ring containing the anchor (else the largest, the last of
// equal length), back-projection and Douglas-Peucker, on the GPU
// (csrc/trace.cu) for rasters the caller holds on the host.

namespace {

constexpr double EARTH_R = 6378137.0;
constexpr double PI_D = 3.14159265358979323846264338;

}  // namespace

extern "C" {

bf_status bf_contour_polygons(const bf_raster* rasters, const uint64_t* words, uint32_t n_iso,
                              const double* cell_m, const double* simplify_m,
                              const uint8_t* has_anchor, const double* anchor_xy,
                              uint64_t* ring_off, double** lonlat) {
  if (lonlat) *lonlat = nullptr;
  if (!rasters || !cell_m || !simplify_m || !ring_off || !lonlat || (has_anchor && !anchor_xy)) {
    set_error("bf_contour_polygons: null argument");
    return BF_ERR_INVALID;
  }
  uint64_t total = 0;
  for (uint32_t k = 0; k < n_iso; ++k)
    total = std::max<uint64_t>(total, rasters[k].word_offset +
                                          (uint64_t)rasters[k].width_words * rasters[k].height);
  if (total && !words) {
    set_error("bf_contour_polygons: null words");
    return BF_ERR_INVALID;
  }
  int dev = 0;
  BF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("bf_contour_polygons: device ordinal out of range");
    return BF_ERR_INVALID;
  }
  Workspace& ws = workspace(dev);
  std::lock_guard<std::mutex> lk(ws.mu);
  if (!ws.st) BF_CUDA(cudaStreamCreateWithFlags(&ws.st, cudaStreamNonBlocking));
  uint64_t* d_words = nullptr;
  BF_CUDA(ws_get(ws, S_A, std::max<uint64_t>(total, 1) * 8, &d_words));
  if (total) BF_CUDA(cudaMemcpyAsync(d_words, words, total * 8, cudaMemcpyHostToDevice, ws.st));
  std::vector<uint64_t> off;
  std::vector<double> ll;
  bf_status rc = trace_rings_device(d_words, rasters, n_iso, cell_m, simplify_m, has_anchor,
                                    anchor_xy, ws.st, off, ll);
  if (rc) return rc;
  double* out = (double*)std::malloc(std::max<size_t>(ll.size(), 2) * 8);
  if (!out) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  if (!ll.empty()) std::memcpy(out, ll.data(), ll.size() * 8);
  for (uint32_t k = 0; k <= n_iso; ++k) ring_off[k] = off[k];
  *lonlat = out;
  return BF_OK;
}

void bf_contour_free_polygons(double* lonlat) { std::free(lonlat); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Isochrone polygons end to end: settled sets of every origin (bulk waves),
// the reachable road segments of each (whole, or cut at the threshold, as
// build_isochrone_geometry_sparse does, server/geometry.rs:281-418), the
// contour rasters on the GPU, tracing and simplification on host threads.

#include <chrono>

// Device copy of a geometry (uploaded on first use on that device).
struct GeoDev {
  bool ready = false;
  uint64_t* off = nullptr;
  uint32_t* w = nullptr;
  double2* xy = nullptr;
  int2* e7 = nullptr;
};

struct bf_geometry {
  uint32_t n = 0;
  std::vector<uint64_t> off;   // polyline of rank r: points [off[r], off[r + 1])
  std::vector<int32_t> e7;     // (lat_e7, lon_e7) per point
  std::vector<double> xy;      // Web-Mercator (x, y) per point
  std::vector<uint32_t> w;     // traversal weight per rank
  mutable std::mutex mu;
  mutable GeoDev dev[64];
};

namespace {

// to_mercator (sparse_contour.rs:441-445): to_radians is x * (PI / 180).
void mercator_e7(int32_t lat_e7, int32_t lon_e7, double* x, double* y) {
  const double lat = (double)lat_e7 / 1e7, lon = (double)lon_e7 / 1e7;
  *x = lon * (PI_D / 180.0) * EARTH_R;
  *y = std::log(std::tan(lat * (PI_D / 180.0) / 2.0 + PI_D / 4.0)) * EARTH_R;
}

// ---- reachable road segments of a wave of isochrones, on the device ----
//
// build_isochrone_geometry_sparse (server/geometry.rs:281-418): every settled
// rank whose road is stamped contributes its polyline whole, or, on the
// frontier (distance + weight beyond the threshold), cut with the
// reference's f32 arithmetic: frac = (T - d) / w, the first floor(frac * n)
// + 1 points and an interpolated cut point. The anchor is the first vertex
// of the first settled road (ranks ascending) of minimum distance.
// Entry i of the wave is settled (rank, dist) pair i; lane l owns entries
// [lane_off[l], lane_off[l + 1]). Counting, a one-block scan of the block
// totals and an ordered write give each segment its offsets; the cut
// points go to the host for projection (host libm, as the reference) and
// come back by a scatter.
struct WaveIn {
  const uint32_t* ranks;
  const uint32_t* dists;
  const uint64_t* lane_off;
  uint32_t kw;
  const uint32_t* thr;  // per lane
  const uint64_t* g_off;
  const uint32_t* g_w;
  const double2* g_xy;
  const int2* g_e7;
  uint32_t g_n;
  uint64_t n;  // entries
};

struct Road {
  uint64_t p0, take;
  uint32_t rank, dist;
  int32_t clat, clon;
  uint32_t seg, cut;  // 0 or 1
  bool anchor;        // a stamped road: an anchor candidate
};

constexpr uint32_t SEG_TPB = 256, SEG_ITEMS = 8, SEG_BLOCK = SEG_TPB * SEG_ITEMS;

__device__ __forceinline__ uint32_t lane_at(const uint64_t* __restrict__ off, uint32_t kw,
                                            uint64_t i) {
  uint32_t lo = 0, hi = kw;  // off[lo] <= i < off[hi]
  while (hi - lo > 1) {
    const uint32_t m = (lo + hi) >> 1;
    if (off[m] <= i)
      lo = m;
    else
      hi = m;
  }
  return lo;
}

__device__ __forceinline__ Road road_of(const WaveIn& a, uint64_t i, uint32_t l, uint32_t* err) {
  Road R{};
  const uint32_t r = a.ranks[i], d = a.dists[i], T = a.thr[l];
  R.rank = r;
  R.dist = d;
  if (r >= a.g_n) {
    atomicOr(err, 4u);
    return R;
  }
  if (d > T) return R;
  const uint32_t w = a.g_w[r];
  if (w == 0 || w == 0xFFFFFFFFu) return R;
  const uint64_t p0 = a.g_off[r], np = a.g_off[r + 1] - p0;
  if (np == 0) return R;
  R.anchor = true;
  R.p0 = p0;
  const uint32_t d_end = (d + w < d) ? 0xFFFFFFFFu : d + w;
  uint64_t take = np;
  if (d_end > T) {
    const float frac = __fdiv_rn(__uint2float_rn(T - d), __uint2float_rn(w));
    if (frac <= 0.0f) return R;
    if (np > 1 && frac < 1.0f) {
      const uint64_t nsg = np - 1;
      const float sf = __fmul_rn(frac, __ull2float_rn(nsg));
      const uint64_t si = min((uint64_t)floorf(sf), nsg - 1);
      const float lf = __fsub_rn(sf, __ull2float_rn(si));
      take = si + 1;
      if (lf > 0.0f && si + 1 < np) {
        const int2 pa = a.g_e7[p0 + si], pb = a.g_e7[p0 + si + 1];
        R.clat = pa.x + __float2int_rz(__fmul_rn(__int2float_rn(pb.x - pa.x), lf));
        R.clon = pa.y + __float2int_rz(__fmul_rn(__int2float_rn(pb.y - pa.y), lf));
        R.cut = 1;
      }
    } else if (np == 1) {
      take = 1;
    }
  }
  R.take = take;
  R.seg = 1;
  return R;
}

// Per block of SEG_BLOCK entries: segment, point and cut totals; per lane:
// segment counts and the anchor key (dist << 32 | rank), aggregated over a
// warp whose entries share a lane.
__global__ void __launch_bounds__(SEG_TPB)
    k_seg_count(WaveIn a, unsigned long long* __restrict__ blk,
                unsigned long long* __restrict__ lane_seg,
                unsigned long long* __restrict__ lane_anchor, uint32_t* err) {
  __shared__ unsigned long long red[3][SEG_TPB / 32];
  const unsigned FULL = 0xFFFFFFFFu;
  const uint64_t base = (uint64_t)blockIdx.x * SEG_BLOCK;
  unsigned long long s = 0, p = 0, c = 0;
  for (uint32_t j = 0; j < SEG_ITEMS; ++j) {
    const uint64_t i = base + (uint64_t)j * SEG_TPB + threadIdx.x;
    const bool in = i < a.n;
    if (!__any_sync(FULL, in)) continue;
    uint32_t l = 0;
    Road R{};
    if (in) {
      l = lane_at(a.lane_off, a.kw, i);
      R = road_of(a, i, l, err);
    }
    s += R.seg;
    p += R.take + R.cut;
    c += R.cut;
    const unsigned long long key =
        R.anchor ? (((unsigned long long)R.dist << 32) | R.rank) : ~0ull;
    const uint32_t l0 = __shfl_sync(FULL, l, 0);  // thread 0 holds the warp's first entry
    if (__all_sync(FULL, !in || l == l0)) {
      const uint32_t cnt = __popc(__ballot_sync(FULL, R.seg != 0));
      unsigned long long k = key;
      for (int o = 16; o > 0; o >>= 1) k = min(k, __shfl_xor_sync(FULL, k, o));
      if ((threadIdx.x & 31) == 0) {
        if (cnt) atomicAdd(lane_seg + l0, (unsigned long long)cnt);
        if (k != ~0ull) atomicMin(lane_anchor + l0, k);
      }
    } else if (in) {
      if (R.seg) atomicAdd(lane_seg + l, 1ull);
      if (key != ~0ull) atomicMin(lane_anchor + l, key);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(FULL, s, o);
    p += __shfl_xor_sync(FULL, p, o);
    c += __shfl_xor_sync(FULL, c, o);
  }
  const uint32_t warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][warp] = s;
    red[1][warp] = p;
    red[2][warp] = c;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    unsigned long long t = 0;
    for (uint32_t w = 0; w < SEG_TPB / 32; ++w) t += red[threadIdx.x][w];
    blk[3 * (uint64_t)blockIdx.x + threadIdx.x] = t;
  }
}

// Exclusive scan of the nb block totals (one block), the wave's totals last.
__global__ void __launch_bounds__(1024)
    k_seg_scan(uint64_t nb, const unsigned long long* __restrict__ blk,
               unsigned long long* __restrict__ bscan, unsigned long long* __restrict__ tot) {
  __shared__ unsigned long long sh[3][32];
  const unsigned FULL = 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long carry[3] = {0, 0, 0};
  for (uint64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    const uint64_t b = b0 + threadIdx.x;
    unsigned long long v[3], x[3];
    for (int q = 0; q < 3; ++q) {
      v[q] = b < nb ? blk[3 * b + q] : 0;
      x[q] = v[q];
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long y = __shfl_up_sync(FULL, x[q], d);
        if (lane >= d) x[q] += y;
      }
      if (lane == 31) sh[q][warp] = x[q];
    }
    __syncthreads();
    if (warp == 0)
      for (int q = 0; q < 3; ++q) {
        unsigned long long t = lane < (blockDim.x >> 5) ? sh[q][lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
          const unsigned long long y = __shfl_up_sync(FULL, t, d);
          if (lane >= d) t += y;
        }
        sh[q][lane] = t;
      }
    __syncthreads();
    for (int q = 0; q < 3; ++q) {
      if (b < nb) bscan[3 * b + q] = carry[q] + (warp ? sh[q][warp - 1] : 0) + x[q] - v[q];
      carry[q] += sh[q][(blockDim.x >> 5) - 1];
    }
    __syncthreads();
  }
  if (threadIdx.x < 3) tot[threadIdx.x] = carry[threadIdx.x];
}

template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T* sh, T* total) {
  const unsigned FULL = 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
  for (int d = 1; d < 32; d <<= 1) {
    const T y = __shfl_up_sync(FULL, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  T pre = 0, t = 0;
  for (uint32_t w = 0; w < SEG_TPB / 32; ++w) {
    const T sv = sh[w];
    if (w < warp) pre += sv;
    t += sv;
  }
  __syncthreads();
  *total = t;
  return pre + x - v;
}

// Ordered write: segment s of the wave ends at seg_pt[s + 1]; its points
// are gathered from the projected geometry, its cut point (if any) is
// recorded as cut c at point cut_pos[c].
__global__ void __launch_bounds__(SEG_TPB)
    k_seg_write(WaveIn a, const unsigned long long* __restrict__ bscan,
                uint64_t* __restrict__ seg_pt, double2* __restrict__ xy,
                int2* __restrict__ cut_e7, uint64_t* __restrict__ cut_pos, uint32_t* err) {
  __shared__ uint32_t sh32[SEG_TPB / 32];
  __shared__ unsigned long long sh64[SEG_TPB / 32];
  const uint64_t base = (uint64_t)blockIdx.x * SEG_BLOCK;
  uint64_t s = bscan[3 * (uint64_t)blockIdx.x], p = bscan[3 * (uint64_t)blockIdx.x + 1],
           c = bscan[3 * (uint64_t)blockIdx.x + 2];
  for (uint32_t j = 0; j < SEG_ITEMS; ++j) {
    const uint64_t i = base + (uint64_t)j * SEG_TPB + threadIdx.x;
    Road R{};
    if (i < a.n) R = road_of(a, i, lane_at(a.lane_off, a.kw, i), err);
    uint32_t sc_tot;
    unsigned long long p_tot;
    const uint32_t sc = block_excl_scan<uint32_t>(R.seg | (R.cut << 16), sh32, &sc_tot);
    const unsigned long long pe =
        block_excl_scan<unsigned long long>(R.take + R.cut, sh64, &p_tot);
    if (R.seg) {
      const uint64_t ms = s + (sc & 0xFFFFu), mp = p + pe, mc = c + (sc >> 16);
      for (uint64_t q = 0; q < R.take; ++q) xy[mp + q] = a.g_xy[R.p0 + q];
      if (R.cut) {
        cut_e7[mc] = make_int2(R.clat, R.clon);
        cut_pos[mc] = mp + R.take;
      }
      seg_pt[ms + 1] = mp + R.take + R.cut;
    }
    s += sc_tot & 0xFFFFu;
    c += sc_tot >> 16;
    p += p_tot;
  }
}

__global__ void k_cut_scatter(uint64_t n_cut, const uint64_t* __restrict__ pos,
                              const double2* __restrict__ cxy, double2* __restrict__ xy) {
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n_cut;
       c += (uint64_t)gridDim.x * blockDim.x)
    xy[pos[c]] = cxy[c];
}

// The geometry's device copy on `device` (uploaded on first use).
bf_status geo_device(const bf_geometry* geo, int device, GeoDev** out) {
  std::lock_guard<std::mutex> lk(geo->mu);
  GeoDev& d = geo->dev[device];
  if (!d.ready) {
    const uint64_t np = geo->off[geo->n];
    cudaError_t e = cudaMalloc(&d.off, ((uint64_t)geo->n + 1) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&d.w, std::max<uint64_t>(geo->n, 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d.xy, std::max<uint64_t>(np, 1) * 16);
    if (e == cudaSuccess) e = cudaMalloc(&d.e7, std::max<uint64_t>(np, 1) * 8);
    if (e == cudaSuccess)
      e = cudaMemcpy(d.off, geo->off.data(), ((uint64_t)geo->n + 1) * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && geo->n)
      e = cudaMemcpy(d.w, geo->w.data(), (uint64_t)geo->n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && np) e = cudaMemcpy(d.xy, geo->xy.data(), np * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && np) e = cudaMemcpy(d.e7, geo->e7.data(), np * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      for (void* q : {(void*)d.off, (void*)d.w, (void*)d.xy, (void*)d.e7})
        if (q) cudaFree(q);
      d = GeoDev{};
      return cuda_status(e, "bf_isochrone_polygons: geometry upload");
    }
    d.ready = true;
  }
  *out = &d;
  return BF_OK;
}

}  // namespace

extern "C" {

// SparseContourConfig::for_mode_name_with_threshold (sparse_contour.rs:476-546).
bf_status bf_contour_config(uint32_t mode, uint32_t threshold_s, double* cell_m,
                            uint32_t* dilation, uint32_t* erosion, double* simplify_m) {
  if (!cell_m || !dilation || !erosion || !simplify_m) {
    set_error("bf_contour_config: null argument");
    return BF_ERR_INVALID;
  }
  double cell = 30.0, simp = 30.0;
  uint32_t d = 2, e = 2;
  if (mode == BF_MODE_BIKE) {
    cell = simp = 40.0;
    d = e = 3;
  } else if (mode == BF_MODE_FOOT) {
    cell = simp = 25.0;
    d = e = 3;
  }
  double cm = 1.0, sm = 1.0;
  if (threshold_s > 3600) {
    cm = 6.67;
    sm = 8.0;
  } else if (threshold_s > 1800) {
    cm = sm = 4.0;
  } else if (threshold_s > 600) {
    cm = sm = 2.0;
  }
  *cell_m = cell * cm;
  *simplify_m = simp * sm;
  *dilation = d;
  *erosion = e;
  return BF_OK;
}

bf_status bf_mercator(uint64_t n, const int32_t* lat_lon_e7, double* xy) {
  if (n && (!lat_lon_e7 || !xy)) {
    set_error("bf_mercator: null argument");
    return BF_ERR_INVALID;
  }
  parallel_for((n + 65535) / 65536, [&](uint64_t b) {
    for (uint64_t i = b * 65536; i < std::min<uint64_t>(n, (b + 1) * 65536); ++i)
      mercator_e7(lat_lon_e7[2 * i], lat_lon_e7[2 * i + 1], xy + 2 * i, xy + 2 * i + 1);
  });
  return BF_OK;
}

bf_status bf_geometry_create(uint32_t n_nodes, const uint64_t* poly_off, const int32_t* poly_e7,
                             const uint32_t* node_w, bf_geometry** out) {
  if (out) *out = nullptr;
  if (!poly_off || !node_w || !out || (poly_off[n_nodes] && !poly_e7)) {
    set_error("bf_geometry_create: null argument");
    return BF_ERR_INVALID;
  }
  for (uint32_t r = 0; r < n_nodes; ++r)
    if (poly_off[r + 1] < poly_off[r]) {
      set_error("bf_geometry_create: polyline offsets must be non-decreasing");
      return BF_ERR_INVALID;
    }
  bf_geometry* geo = new (std::nothrow) bf_geometry();
  if (!geo) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  try {
    const uint64_t np = poly_off[n_nodes];
    geo->n = n_nodes;
    geo->off.assign(poly_off, poly_off + n_nodes + 1);
    geo->e7.assign(poly_e7, poly_e7 + 2 * np);
    geo->w.assign(node_w, node_w + n_nodes);
    geo->xy.resize(2 * np);
    bf_mercator(np, poly_e7, geo->xy.data());  // static vertices: projected once
  } catch (const std::bad_alloc&) {
    delete geo;
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  *out = geo;
  return BF_OK;
}

void bf_geometry_destroy(bf_geometry* geo) {
  if (!geo) return;
  int cur = -1;
  cudaGetDevice(&cur);
  for (int dv = 0; dv < 64; ++dv) {
    GeoDev& d = geo->dev[dv];
    if (!d.ready) continue;
    if (cudaSetDevice(dv) == cudaSuccess)
      for (void* q : {(void*)d.off, (void*)d.w, (void*)d.xy, (void*)d.e7}) cudaFree(q);
    cudaGetLastError();
  }
  if (cur >= 0) cudaSetDevice(cur);
  delete geo;
}

bf_status bf_isochrone_polygons(bf_graph* g, const bf_geometry* geo, const uint32_t* origins,
                                const uint32_t* thresholds, const uint32_t* tier_thresholds,
                                uint64_t n, uint32_t mode, uint64_t* ring_off, double** lonlat,
                                double* phase_ms) {
  if (lonlat) *lonlat = nullptr;
  if (!g || !geo || !ring_off || !lonlat || (n && (!origins || !thresholds))) {
    set_error("bf_isochrone_polygons: null argument");
    return BF_ERR_INVALID;
  }
  Graph* gr = graph_of(g);
  if (geo->n != gr->n) {
    set_error("bf_isochrone_polygons: the geometry has a polyline per rank of another graph");
    return BF_ERR_INVALID;
  }
  if (n > 0xFFFFFFFFull) {
    set_error("bf_isochrone_polygons: too many origins in one call");
    return BF_ERR_INVALID;
  }
  if (gr->device < 0 || gr->device >= 64) {
    set_error("bf_isochrone_polygons: device ordinal out of range");
    return BF_ERR_INVALID;
  }
  using clk = std::chrono::steady_clock;
  auto ms = [](clk::time_point a) {
    return std::chrono::duration<double, std::milli>(clk::now() - a).count();
  };
  double ph[4] = {0, 0, 0, 0};
  auto mark = clk::now();
  std::vector<double> cell(n), simp(n);
  uint32_t dil = 0, ero = 0;
  for (uint64_t k = 0; k < n; ++k)
    bf_contour_config(mode, tier_thresholds ? tier_thresholds[k] : thresholds[k], &cell[k], &dil,
                      &ero, &simp[k]);
  // one ring per origin, gathered wave by wave
  std::vector<uint64_t> r_len(n, 0), r_at(n, 0);
  std::vector<double*> wave_ll;
  auto free_waves = [&]() {
    for (double* q : wave_ll) bf_contour_free_polygons(q);
  };
  std::lock_guard<std::mutex> glk(gr->mu);
  if (cudaSetDevice(gr->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  GeoDev* gd = nullptr;
  bf_status rc = geo_device(geo, gr->device, &gd);
  if (rc) return rc;
  Workspace& ws = workspace(gr->device);
  std::lock_guard<std::mutex> wlk(ws.mu);
  if (ws.st) BF_CUDA(cudaStreamSynchronize(ws.st));
  SettledSink sink;
  sink.on_wave = [&](const uint32_t* d_r, const uint32_t* d_d, const uint64_t* d_off,
                     const std::vector<uint64_t>& off, const std::vector<uint32_t>& rows,
                     cudaStream_t st) -> bf_status {
    ph[0] += ms(mark);
    auto t0 = clk::now();
    const uint32_t kw = (uint32_t)rows.size();
    const uint64_t E = off[kw];
    const uint64_t nb = (E + SEG_BLOCK - 1) / SEG_BLOCK;
    std::vector<uint32_t> thr_l(kw);
    std::vector<double> cell_l(kw), simp_l(kw);
    for (uint32_t l = 0; l < kw; ++l) {
      thr_l[l] = thresholds[rows[l]];
      cell_l[l] = cell[rows[l]];
      simp_l[l] = simp[rows[l]];
    }
    uint32_t *d_thr = nullptr, *d_err = nullptr;
    unsigned long long *d_blk = nullptr, *d_lane = nullptr;
    cudaError_t e = ws_get(ws, S_THR, (uint64_t)kw * 4, &d_thr);
    if (e == cudaSuccess) e = ws_get(ws, S_ERR, 4, &d_err);
    if (e == cudaSuccess) e = ws_get(ws, S_BLK, std::max<uint64_t>(nb, 1) * 6 * 8, &d_blk);
    if (e == cudaSuccess) e = ws_get(ws, S_LANE, (2ull * kw + 3) * 8, &d_lane);
    if (e != cudaSuccess) return cuda_status(e, "bf_isochrone_polygons: device memory");
    unsigned long long *lane_seg = d_lane, *lane_anchor = d_lane + kw, *tot = d_lane + 2 * kw;
    const WaveIn a{d_r, d_d, d_off, kw, d_thr, gd->off, gd->w, gd->xy, gd->e7, geo->n, E};
    BF_CUDA(cudaMemcpyAsync(d_thr, thr_l.data(), (uint64_t)kw * 4, cudaMemcpyHostToDevice, st));
    BF_CUDA(cudaMemsetAsync(lane_seg, 0, (uint64_t)kw * 8, st));
    BF_CUDA(cudaMemsetAsync(lane_anchor, 0xFF, (uint64_t)kw * 8, st));
    BF_CUDA(cudaMemsetAsync(tot, 0, 24, st));
    BF_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
    if (E) {
      k_seg_count<<<(unsigned)nb, SEG_TPB, 0, st>>>(a, d_blk, lane_seg, lane_anchor, d_err);
      k_seg_scan<<<1, 1024, 0, st>>>(nb, d_blk, d_blk + 3 * nb, tot);
      BF_CUDA(cudaGetLastError());
    }
    std::vector<unsigned long long> lane(2ull * kw + 3);
    uint32_t verr = 0;
    BF_CUDA(cudaMemcpyAsync(lane.data(), d_lane, lane.size() * 8, cudaMemcpyDeviceToHost, st));
    BF_CUDA(cudaMemcpyAsync(&verr, d_err, 4, cudaMemcpyDeviceToHost, st));
    BF_CUDA(cudaStreamSynchronize(st));
    if (verr) {
      set_error("bf_isochrone_polygons: a settled rank lies outside the geometry");
      return BF_ERR_DEVICE;
    }
    const uint64_t n_seg = lane[2 * kw], n_pts = lane[2 * kw + 1], n_cut = lane[2 * kw + 2];
    std::vector<uint64_t> iso_seg(kw + 1, 0);
    std::vector<uint8_t> has(kw, 0);
    std::vector<double> anc(2ull * kw, 0.0);
    for (uint32_t l = 0; l < kw; ++l) {
      iso_seg[l + 1] = iso_seg[l] + lane[l];
      const unsigned long long key = lane[kw + l];
      if (key != ~0ull && lane[l]) {  // no segment: the reference returns no contour
        const uint64_t p0 = geo->off[(uint32_t)key];
        has[l] = 1;
        anc[2 * l] = geo->xy[2 * p0];
        anc[2 * l + 1] = geo->xy[2 * p0 + 1];
      }
    }
    if (iso_seg[kw] != n_seg) {
      set_error("bf_isochrone_polygons: segment counts disagree");
      return BF_ERR_DEVICE;
    }
    double2 *d_xy = nullptr, *d_cxy = nullptr;
    uint64_t *d_seg = nullptr, *d_iseg = nullptr, *d_cpos = nullptr;
    int2* d_ce7 = nullptr;
    e = ws_get(ws, S_XY, n_pts * 16, &d_xy);
    if (e == cudaSuccess) e = ws_get(ws, S_SEG, (n_seg + 1) * 8, &d_seg);
    if (e == cudaSuccess) e = ws_get(ws, S_ISEG, ((uint64_t)kw + 1) * 8, &d_iseg);
    if (e == cudaSuccess) e = ws_get(ws, S_CUT, n_cut * 16, &d_cpos);
    if (e == cudaSuccess) e = ws_get(ws, S_CUTXY, n_cut * 16, &d_cxy);
    if (e != cudaSuccess) return cuda_status(e, "bf_isochrone_polygons: device memory");
    d_ce7 = reinterpret_cast<int2*>(d_cpos + n_cut);
    BF_CUDA(cudaMemsetAsync(d_seg, 0, 8, st));
    BF_CUDA(cudaMemcpyAsync(d_iseg, iso_seg.data(), ((uint64_t)kw + 1) * 8, cudaMemcpyHostToDevice,
                            st));
    if (E) {
      k_seg_write<<<(unsigned)nb, SEG_TPB, 0, st>>>(a, d_blk + 3 * nb, d_seg, d_xy, d_ce7, d_cpos,
                                                    d_err);
      BF_CUDA(cudaGetLastError());
    }
    if (n_cut) {
      std::vector<int32_t> ce7(2 * n_cut);
      std::vector<double> cxy(2 * n_cut);
      BF_CUDA(cudaMemcpyAsync(ce7.data(), d_ce7, n_cut * 8, cudaMemcpyDeviceToHost, st));
      BF_CUDA(cudaStreamSynchronize(st));
      if ((rc = bf_mercator(n_cut, ce7.data(), cxy.data()))) return rc;
      BF_CUDA(cudaMemcpyAsync(d_cxy, cxy.data(), n_cut * 16, cudaMemcpyHostToDevice, st));
      k_cut_scatter<<<grid_of(n_cut), 256, 0, st>>>(n_cut, d_cpos, d_cxy, d_xy);
      BF_CUDA(cudaGetLastError());
    }
    ph[1] += ms(t0);
    t0 = clk::now();
    std::vector<bf_raster> ras(std::max<uint32_t>(kw, 1));
    const uint64_t* d_words = nullptr;
    uint64_t n_words = 0;
    if ((rc = rasters_core(ws, st, d_xy, d_seg, d_iseg, n_seg, n_pts, kw, cell_l.data(), has.data(),
                           anc.data(), dil, ero, ras.data(), nullptr, &n_words, &d_words)))
      return rc;
    ph[2] += ms(t0);
    t0 = clk::now();
    std::vector<uint64_t> roff;
    std::vector<double> ll_v;
    if ((rc = trace_rings_device(d_words, ras.data(), kw, cell_l.data(), simp_l.data(), has.data(),
                                 anc.data(), st, roff, ll_v)))
      return rc;
    double* ll = (double*)std::malloc(std::max<size_t>(ll_v.size(), 2) * 8);
    if (!ll) {
      set_error("out of host memory");
      return BF_ERR_OOM;
    }
    if (!ll_v.empty()) std::memcpy(ll, ll_v.data(), ll_v.size() * 8);
    wave_ll.push_back(ll);
    for (uint32_t l = 0; l < kw; ++l) {
      r_len[rows[l]] = roff[l + 1] - roff[l];
      r_at[rows[l]] = (uint64_t)(wave_ll.size() - 1) << 40 | roff[l];  // (wave, point)
    }
    ph[3] += ms(t0);
    mark = clk::now();
    return BF_OK;
  };
  if ((rc = settled_waves(gr, origins, thresholds, n, sink, nullptr))) {
    free_waves();
    return rc;
  }
  ph[0] += ms(mark);
  auto t0 = clk::now();
  ring_off[0] = 0;
  for (uint64_t k = 0; k < n; ++k) ring_off[k + 1] = ring_off[k] + r_len[k];
  double* out = (double*)std::malloc(std::max<uint64_t>(ring_off[n], 1) * 16);
  if (!out) {
    free_waves();
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  parallel_for(n, [&](uint64_t k) {
    if (!r_len[k]) return;
    const double* src = wave_ll[r_at[k] >> 40] + 2 * (r_at[k] & ((1ull << 40) - 1));
    std::memcpy(out + 2 * ring_off[k], src, r_len[k] * 16);
  });
  free_waves();
  *lonlat = out;
  ph[3] += ms(t0);
  if (phase_ms)
    for (int i = 0; i < 4; ++i) phase_ms[i] = ph[i];
  return BF_OK;
}

}  // extern "C"
