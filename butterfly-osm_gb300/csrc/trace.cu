// trace.cu — contour rings on the GPU: boundary tracing, ring choice,
// back-projection and Douglas-Peucker (steps 4-5 of the reference's sparse
// contour pipeline, route/src/range/sparse_contour.rs:770-1183), for a batch
// of closed rasters already on the device.
//
// The reference walks each ring cell by cell: boundary starts in (column,
// row) order, one per boundary cell with its first boundary edge in N, W, E,
// S priority; every start whose edge no earlier ring visited begins a ring,
// which follows next_boundary_edge (sparse_contour.rs:1049-1130) back to its
// start. A walk is a long chain of dependent steps, so here the rings come
// out of data-parallel passes:
//
//   edges     every boundary edge (a set cell's side whose neighbour is
//             unset) gets an index and its successor under the same
//             next_boundary_edge rule; successors form disjoint cycles.
//   cycles    pointer jumping gives every edge the smallest start key
//             (column, row) on its cycle. A cycle holding no start is never
//             traced; a traced cycle's walk begins at that start, which is
//             the first of its starts in (column, row) order (every later one
//             is visited by then), and rings are ordered by that key.
//   order     list ranking from the start gives each edge its step and each
//             emitted vertex (a cell centre, consecutive equal ones once) its
//             index; a last vertex equal to the first is dropped, rings of
//             fewer than three vertices are dropped.
//   choice    the anchor's crossing parity and distance test per ring
//             segment (in_ring || near_ring within one cell); the ring
//             containing the anchor with the most vertices (the first of
//             equal size), else the ring with the most vertices (the last).
//   project   vertex (c + 0.5, r + 0.5) cells from the grid origin to
//             (lon, lat) from per-column and per-row tables computed on the
//             host with the host libm (the reference's back-projection).
//   simplify  Douglas-Peucker level by level: every open range's farthest
//             interior point (the first of equal distances) is kept when its
//             distance exceeds the tolerance, which splits the range; ranges
//             split independently, so the kept set is the recursive form's.
//
// Every floating-point step uses the round-to-nearest intrinsics in the
// reference's operation order (no contraction), so rings are bit-identical.
// The reference caps a walk at (non-empty 64 x 64 tiles) x 16384 steps, more
// than a ring of those tiles can have, so the cap never ends a walk here.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "engine.cuh"
#include "scan.cuh"

namespace bf {

namespace {

constexpr double EARTH_R_T = 6378137.0;
constexpr double PI_T = 3.14159265358979323846264338;
constexpr uint64_t NOKEY = ~0ull;
constexpr uint32_t TPB = 256;

struct TIso {
  int32_t col0, row0;
  uint32_t wpr, height;
  uint64_t woff;     // first word of the raster
  uint64_t lon_off;  // first entry of its per-column longitude table
  uint64_t lat_off;  // first entry of its per-row latitude table
  uint32_t has_anchor, pad;
  double ax, ay;     // anchor in cells from the grid origin
};

unsigned grid(uint64_t n, unsigned cap = 152 * 16) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + TPB - 1) / TPB, cap));
}

__device__ __forceinline__ uint32_t iso_of_word(const TIso* __restrict__ iso, uint32_t n_iso,
                                                uint64_t w) {
  uint32_t lo = 0, hi = n_iso;  // largest k with iso[k].woff <= w
  while (hi - lo > 1) {
    const uint32_t m = (lo + hi) >> 1;
    if (iso[m].woff <= w)
      lo = m;
    else
      hi = m;
  }
  return lo;
}

// std::max / std::min on doubles (the host's clamps), including which of
// two equal operands (-0.0 and 0.0) is returned.
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

struct Nb {
  uint64_t cur, north, south, west, east;
};

__device__ __forceinline__ uint64_t word_at(const uint64_t* __restrict__ words, const TIso& g,
                                            int64_t r, int64_t c) {
  if (r < 0 || r >= (int64_t)g.height || c < 0 || c >= (int64_t)g.wpr) return 0;
  return words[g.woff + (uint64_t)r * g.wpr + (uint64_t)c];
}

// The word at raster row lr, word column j and its four neighbours' bits
// aligned on it (cells outside the raster read as unset).
__device__ __forceinline__ Nb neighbours(const uint64_t* __restrict__ words, const TIso& g,
                                         int64_t lr, int64_t j) {
  Nb n;
  n.cur = word_at(words, g, lr, j);
  n.north = word_at(words, g, lr - 1, j);
  n.south = word_at(words, g, lr + 1, j);
  n.west = (n.cur << 1) | (word_at(words, g, lr, j - 1) >> 63);
  n.east = (n.cur >> 1) | (word_at(words, g, lr, j + 1) << 63);
  return n;
}

__device__ __forceinline__ bool cell_set(const uint64_t* __restrict__ words, const TIso& g,
                                         int64_t lc, int64_t lr) {
  if (lc < 0 || lr < 0 || lr >= (int64_t)g.height || lc >= (int64_t)g.wpr * 64) return false;
  return (words[g.woff + (uint64_t)lr * g.wpr + (uint64_t)(lc >> 6)] >> (lc & 63)) & 1ull;
}

// Rasters may lie anywhere in the caller's word array (in any order, even
// sharing words): each is copied to its own place in a packed array, in
// raster order, which the passes below rely on.
__global__ void __launch_bounds__(TPB)
    k_tr_pack(const uint64_t* __restrict__ words, const TIso* __restrict__ iso, uint32_t n_iso,
              const uint64_t* __restrict__ src_off, uint64_t TW, uint64_t* __restrict__ packed) {
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < TW;
       w += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t k = iso_of_word(iso, n_iso, w);
    packed[w] = words[src_off[k] + (w - iso[k].woff)];
  }
}

// Boundary cells: set cells with an unset neighbour on some side.
__global__ void __launch_bounds__(TPB)
    k_tr_mask(const uint64_t* __restrict__ words, const TIso* __restrict__ iso, uint32_t n_iso,
              uint64_t TW, uint64_t* __restrict__ bmask) {
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < TW;
       w += (uint64_t)gridDim.x * blockDim.x) {
    const TIso g = iso[iso_of_word(iso, n_iso, w)];
    const uint64_t loc = w - g.woff;
    const Nb n = neighbours(words, g, (int64_t)(loc / g.wpr), (int64_t)(loc % g.wpr));
    bmask[w] = n.cur & ~(n.north & n.south & n.west & n.east);
  }
}

struct PopVal64 {
  const uint64_t* a;
  __device__ uint32_t operator()(uint64_t i) const { return __popcll(a[i]); }
};

__device__ __forceinline__ uint32_t bcell_of(const uint64_t* __restrict__ bmask,
                                             const uint32_t* __restrict__ bpre, uint64_t w,
                                             uint32_t b) {
  return bpre[w] + __popcll(bmask[w] & ((1ull << b) - 1ull));
}

// Edge codes as the reference's: 0 = N, 1 = E, 2 = S, 3 = W. Per boundary
// cell: its raster, local (column, row), the mask of its boundary edges and
// (bits 4-5) its first edge in start priority N, W, E, S.
__global__ void __launch_bounds__(TPB)
    k_tr_cells(const uint64_t* __restrict__ words, const TIso* __restrict__ iso, uint32_t n_iso,
               uint64_t TW, const uint64_t* __restrict__ bmask, const uint32_t* __restrict__ bpre,
               uint32_t* __restrict__ c_iso, uint2* __restrict__ c_pos,
               uint32_t* __restrict__ c_code) {
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < TW;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t m = bmask[w];
    if (!m) continue;
    const uint32_t k = iso_of_word(iso, n_iso, w);
    const TIso g = iso[k];
    const uint64_t loc = w - g.woff;
    const int64_t lr = (int64_t)(loc / g.wpr), j = (int64_t)(loc % g.wpr);
    const Nb n = neighbours(words, g, lr, j);
    uint32_t at = bpre[w];
    while (m) {
      const uint32_t b = __ffsll(m) - 1;
      m &= m - 1;
      const uint32_t eN = !((n.north >> b) & 1), eE = !((n.east >> b) & 1);
      const uint32_t eS = !((n.south >> b) & 1), eW = !((n.west >> b) & 1);
      const uint32_t mask = eN | (eE << 1) | (eS << 2) | (eW << 3);
      const uint32_t first = eN ? 0u : eW ? 3u : eE ? 1u : 2u;
      c_iso[at] = k;
      c_pos[at] = make_uint2((uint32_t)(j * 64 + b), (uint32_t)lr);
      c_code[at] = mask | (first << 4);
      ++at;
    }
  }
}

struct EdgeCountVal {
  const uint32_t* code;
  __device__ uint32_t operator()(uint64_t i) const { return __popc(code[i] & 15u); }
};

__device__ __forceinline__ uint32_t edge_index(const uint32_t* __restrict__ ebase,
                                               const uint32_t* __restrict__ c_code, uint32_t cell,
                                               uint32_t e) {
  return ebase[cell] + __popc(c_code[cell] & 15u & ((1u << e) - 1u));
}

// Per edge: successor (next_boundary_edge), cell, and start key (local
// column, row) if it is its cell's first edge. A successor outside the
// boundary edges (which a raster never produces) sets err.
__global__ void __launch_bounds__(TPB)
    k_tr_succ(const uint64_t* __restrict__ words, const TIso* __restrict__ iso, uint32_t BC,
              const uint64_t* __restrict__ bmask, const uint32_t* __restrict__ bpre,
              const uint32_t* __restrict__ c_iso, const uint2* __restrict__ c_pos,
              const uint32_t* __restrict__ c_code, const uint32_t* __restrict__ ebase,
              uint32_t* __restrict__ succ, uint32_t* __restrict__ e_cell,
              uint64_t* __restrict__ key, uint32_t* __restrict__ err) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < BC; c += gridDim.x * blockDim.x) {
    const TIso g = iso[c_iso[c]];
    const int64_t lc = c_pos[c].x, lr = c_pos[c].y;
    const uint32_t code = c_code[c];
    uint32_t ei = ebase[c];
    for (uint32_t e = 0; e < 4; ++e) {
      if (!((code >> e) & 1u)) continue;
      int64_t nc = lc, nr = lr;
      uint32_t ne;
      switch (e) {  // next_boundary_edge, sparse_contour.rs:1049-1130
        case 0:
          if (cell_set(words, g, lc + 1, lr - 1)) { nc = lc + 1; nr = lr - 1; ne = 3; }
          else if (cell_set(words, g, lc + 1, lr)) { nc = lc + 1; ne = 0; }
          else ne = 1;
          break;
        case 1:
          if (cell_set(words, g, lc + 1, lr + 1)) { nc = lc + 1; nr = lr + 1; ne = 0; }
          else if (cell_set(words, g, lc, lr + 1)) { nr = lr + 1; ne = 1; }
          else ne = 2;
          break;
        case 2:
          if (cell_set(words, g, lc - 1, lr + 1)) { nc = lc - 1; nr = lr + 1; ne = 1; }
          else if (cell_set(words, g, lc - 1, lr)) { nc = lc - 1; ne = 2; }
          else ne = 3;
          break;
        default:
          if (cell_set(words, g, lc - 1, lr - 1)) { nc = lc - 1; nr = lr - 1; ne = 2; }
          else if (cell_set(words, g, lc, lr - 1)) { nr = lr - 1; ne = 3; }
          else ne = 0;
      }
      uint32_t s = ei;  // itself on an inconsistency (a one-edge cycle)
      bool ok = false;
      if (nc >= 0 && nr >= 0 && nr < (int64_t)g.height && nc < (int64_t)g.wpr * 64) {
        const uint64_t w2 = g.woff + (uint64_t)nr * g.wpr + (uint64_t)(nc >> 6);
        const uint32_t b2 = (uint32_t)(nc & 63);
        if ((bmask[w2] >> b2) & 1ull) {
          const uint32_t c2 = bcell_of(bmask, bpre, w2, b2);
          if ((c_code[c2] >> ne) & 1u) {
            s = edge_index(ebase, c_code, c2, ne);
            ok = true;
          }
        }
      }
      if (!ok) atomicOr(err, 1u);
      succ[ei] = s;
      e_cell[ei] = c;
      key[ei] = (e == (code >> 4)) ? (((uint64_t)lc << 32) | (uint64_t)lr) : NOKEY;
      ++ei;
    }
  }
}

__global__ void __launch_bounds__(TPB)
    k_tr_pred(uint32_t E, const uint32_t* __restrict__ succ, uint32_t* __restrict__ pred) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x)
    pred[succ[i]] = i;
}

// One pointer-jumping round: m' = min(m, m[p]), p' = p[p].
__global__ void __launch_bounds__(TPB)
    k_tr_jump_min(uint32_t E, const uint64_t* __restrict__ m, const uint32_t* __restrict__ p,
                  uint64_t* __restrict__ m2, uint32_t* __restrict__ p2) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
    const uint32_t q = p[i];
    m2[i] = min(m[i], m[q]);
    p2[i] = p[q];
  }
}

// Start edge of each edge's cycle (NONE: the cycle holds no start) and the
// emit flag: the start, or an edge whose predecessor lies on another cell.
__global__ void __launch_bounds__(TPB)
    k_tr_start(uint32_t E, const uint64_t* __restrict__ cyc, const uint32_t* __restrict__ e_cell,
               const uint32_t* __restrict__ pred, const TIso* __restrict__ iso,
               const uint32_t* __restrict__ c_iso, const uint64_t* __restrict__ bmask,
               const uint32_t* __restrict__ bpre, const uint32_t* __restrict__ c_code,
               const uint32_t* __restrict__ ebase, uint32_t* __restrict__ start,
               uint32_t* __restrict__ emit) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
    const uint64_t kk = cyc[i];
    if (kk == NOKEY) {
      start[i] = NONE;
      emit[i] = 0;
      continue;
    }
    const TIso g = iso[c_iso[e_cell[i]]];
    const uint32_t lc = (uint32_t)(kk >> 32), lr = (uint32_t)kk;
    const uint64_t w = g.woff + (uint64_t)lr * g.wpr + (lc >> 6);
    const uint32_t c = bcell_of(bmask, bpre, w, lc & 63);
    const uint32_t s = edge_index(ebase, c_code, c, (c_code[c] >> 4) & 3u);
    start[i] = s;
    emit[i] = (i == s || e_cell[pred[i]] != e_cell[i]) ? 1u : 0u;
  }
}

// List ranking from the start: dv[i] = (edges, emitted vertices) from i
// (included) to the start (excluded; the start's own dv covers its ring).
// Edges of untraced cycles are done from the outset.
__global__ void __launch_bounds__(TPB)
    k_tr_rank_init(uint32_t E, const uint32_t* __restrict__ succ, const uint32_t* __restrict__ start,
                   const uint32_t* __restrict__ emit, uint32_t* __restrict__ q,
                   uint64_t* __restrict__ dv, uint8_t* __restrict__ done) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
    q[i] = succ[i];
    dv[i] = (1ull << 32) | emit[i];
    done[i] = (start[i] == NONE || succ[i] == start[i]) ? 1 : 0;
  }
}

__global__ void __launch_bounds__(TPB)
    k_tr_rank(uint32_t E, const uint32_t* __restrict__ q, const uint64_t* __restrict__ dv,
              const uint8_t* __restrict__ done, uint32_t* __restrict__ q2,
              uint64_t* __restrict__ dv2, uint8_t* __restrict__ done2) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
    if (done[i]) {
      q2[i] = q[i];
      dv2[i] = dv[i];
      done2[i] = 1;
      continue;
    }
    const uint32_t j = q[i];
    dv2[i] = dv[i] + dv[j];
    done2[i] = done[j];
    q2[i] = q[j];
  }
}

// Rings: one per traced start edge, in edge order (rasters in order).
struct RingHeadVal {
  const uint32_t* start;
  __device__ uint32_t operator()(uint64_t i) const { return start[i] == (uint32_t)i ? 1u : 0u; }
};

struct Ring {
  uint32_t iso, size;  // size: vertices after the trailing duplicate is dropped
  uint32_t V, pad;     // emitted vertices
  uint64_t key;        // (column, row) of the start: the ring's order
};

__global__ void __launch_bounds__(TPB)
    k_tr_rings(uint32_t E, const uint32_t* __restrict__ start, const uint32_t* __restrict__ rpre,
               const uint64_t* __restrict__ dv, const uint32_t* __restrict__ pred,
               const uint32_t* __restrict__ e_cell, const uint32_t* __restrict__ c_iso,
               const uint64_t* __restrict__ cyc, Ring* __restrict__ rings,
               uint32_t* __restrict__ ring_v) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
    if (start[i] != i) continue;
    const uint32_t r = rpre[i];
    const uint32_t V = (uint32_t)dv[i];
    const bool trail = V > 1 && e_cell[pred[i]] == e_cell[i];
    Ring R;
    R.iso = c_iso[e_cell[i]];
    R.V = V;
    R.size = V - (trail ? 1u : 0u);
    R.pad = 0;
    R.key = cyc[i];
    rings[r] = R;
    ring_v[r] = V;
  }
}

struct U32Val {
  const uint32_t* a;
  __device__ uint32_t operator()(uint64_t i) const { return a[i]; }
};

// Vertices of every ring (local cell coordinates), trailing duplicate dropped.
__global__ void __launch_bounds__(TPB)
    k_tr_verts(uint32_t E, const uint32_t* __restrict__ start, const uint32_t* __restrict__ emit,
               const uint32_t* __restrict__ rpre, const uint64_t* __restrict__ dv,
               const uint32_t* __restrict__ e_cell, const uint2* __restrict__ c_pos,
               const Ring* __restrict__ rings, const uint64_t* __restrict__ voff,
               uint2* __restrict__ verts) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
    const uint32_t s = start[i];
    if (s == NONE || !emit[i]) continue;
    const uint32_t r = rpre[s];
    const Ring R = rings[r];
    const uint32_t vi = R.V - (uint32_t)dv[i];
    if (vi < R.size) verts[voff[r] + vi] = c_pos[e_cell[i]];
  }
}

__global__ void k_tr_vring(uint32_t NR, const uint64_t* __restrict__ voff,
                           uint32_t* __restrict__ vring) {
  for (uint32_t r = blockIdx.x; r < NR; r += gridDim.x)
    for (uint64_t v = voff[r] + threadIdx.x; v < voff[r + 1]; v += blockDim.x) vring[v] = r;
}

// The anchor against every ring segment of rasters with an anchor: crossing
// parity (in_ring) and distance within one cell (near_ring), in the
// reference's operation order.
__global__ void __launch_bounds__(TPB)
    k_tr_anchor(uint64_t NV, const uint32_t* __restrict__ vring, const Ring* __restrict__ rings,
                const uint64_t* __restrict__ voff, const uint2* __restrict__ verts,
                const TIso* __restrict__ iso, uint32_t* __restrict__ cross,
                uint32_t* __restrict__ near) {
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < NV;
       v += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = vring[v];
    const Ring R = rings[r];
    const TIso g = iso[R.iso];
    if (!g.has_anchor || R.size < 3) continue;
    const uint64_t k = v - voff[r];
    if (k >= R.size) continue;
    const uint2 A = verts[v], B = verts[voff[r] + (k + 1 == R.size ? 0 : k + 1)];
    const double ax = (double)(g.col0 + (int64_t)A.x) + 0.5;
    const double ay = (double)(g.row0 + (int64_t)A.y) + 0.5;
    const double bx = (double)(g.col0 + (int64_t)B.x) + 0.5;
    const double by = (double)(g.row0 + (int64_t)B.y) + 0.5;
    const double px = g.ax, py = g.ay;
    if ((ay > py) != (by > py) &&
        px < __dadd_rn(__ddiv_rn(__dmul_rn(__dsub_rn(bx, ax), __dsub_rn(py, ay)),
                                 __dsub_rn(by, ay)),
                       ax))
      atomicXor(&cross[r], 1u);
    const double dx = __dsub_rn(bx, ax), dy = __dsub_rn(by, ay);
    const double len2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    double t = 0.0;
    if (len2 > 0.0)
      t = smin(smax(__ddiv_rn(__dadd_rn(__dmul_rn(__dsub_rn(px, ax), dx),
                                        __dmul_rn(__dsub_rn(py, ay), dy)),
                              len2),
                    0.0),
               1.0);
    const double cx = __dadd_rn(ax, __dmul_rn(t, dx)), cy = __dadd_rn(ay, __dmul_rn(t, dy));
    const double ex = __dsub_rn(px, cx), ey = __dsub_rn(py, cy);
    if (__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)) <= 1.0) atomicOr(&near[r], 1u);
  }
}

// The chosen ring of each raster: with an anchor, the ring containing it
// with the most vertices (the first of equal size in ring order), else (or
// when none contains it) the ring with the most vertices (the last of equal
// size). Rings of a raster are contiguous; their order is the start key.
__global__ void k_tr_choose(uint32_t n_iso, uint32_t NR, const Ring* __restrict__ rings,
                            const uint32_t* __restrict__ cross, const uint32_t* __restrict__ near,
                            const TIso* __restrict__ iso, uint32_t* __restrict__ best) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_iso) return;
  uint32_t lo = 0, hi = NR;  // first ring of raster k
  while (lo < hi) {
    const uint32_t m = (lo + hi) >> 1;
    if (rings[m].iso < k)
      lo = m + 1;
    else
      hi = m;
  }
  uint32_t b = NONE;
  if (iso[k].has_anchor)
    for (uint32_t r = lo; r < NR && rings[r].iso == k; ++r) {
      const Ring R = rings[r];
      if (R.size < 3 || !(cross[r] || near[r])) continue;
      if (b == NONE || R.size > rings[b].size ||
          (R.size == rings[b].size && R.key < rings[b].key))
        b = r;
    }
  if (b == NONE)
    for (uint32_t r = lo; r < NR && rings[r].iso == k; ++r) {
      const Ring R = rings[r];
      if (R.size < 3) continue;
      if (b == NONE || R.size > rings[b].size ||
          (R.size == rings[b].size && R.key > rings[b].key))
        b = r;
    }
  best[k] = b;
}

// Points of the chosen rings as (lon, lat) from the host-computed tables.
__global__ void __launch_bounds__(TPB)
    k_tr_project(uint32_t n_iso, const uint32_t* __restrict__ best, const uint64_t* __restrict__ voff,
                 const uint2* __restrict__ verts, const uint64_t* __restrict__ poff,
                 const TIso* __restrict__ iso, const double* __restrict__ lon,
                 const double* __restrict__ lat, double2* __restrict__ pts,
                 uint32_t* __restrict__ pring) {
  for (uint32_t k = blockIdx.x; k < n_iso; k += gridDim.x) {
    const uint32_t r = best[k];
    if (r == NONE) continue;
    const TIso g = iso[k];
    const uint64_t n = poff[k + 1] - poff[k];
    for (uint64_t j = threadIdx.x; j < n; j += blockDim.x) {
      const uint2 v = verts[voff[r] + j];
      pts[poff[k] + j] = make_double2(lon[g.lon_off + v.x], lat[g.lat_off + v.y]);
      pring[poff[k] + j] = k;
    }
  }
}

// seg_dist of the reference's Douglas-Peucker, in its operation order.
__device__ __forceinline__ double seg_dist(double2 p, double2 s, double2 e) {
  const double dx = __dsub_rn(e.x, s.x), dy = __dsub_rn(e.y, s.y);
  const double len_sq = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  if (len_sq < 1e-12) {
    const double pdx = __dsub_rn(p.x, s.x), pdy = __dsub_rn(p.y, s.y);
    return __dsqrt_rn(__dadd_rn(__dmul_rn(pdx, pdx), __dmul_rn(pdy, pdy)));
  }
  double t = __ddiv_rn(__dadd_rn(__dmul_rn(__dsub_rn(p.x, s.x), dx),
                                 __dmul_rn(__dsub_rn(p.y, s.y), dy)),
                       len_sq);
  t = smin(smax(t, 0.0), 1.0);
  const double px = __dadd_rn(s.x, __dmul_rn(t, dx)), py = __dadd_rn(s.y, __dmul_rn(t, dy));
  const double pdx = __dsub_rn(p.x, px), pdy = __dsub_rn(p.y, py);
  return __dsqrt_rn(__dadd_rn(__dmul_rn(pdx, pdx), __dmul_rn(pdy, pdy)));
}

// Douglas-Peucker state per point: keep flag; for a kept point a opening a
// range, rend[a] = its right end b and open[a]; for an interior point its
// range's left end in lend. Per ring [first, last] starts open.
__global__ void __launch_bounds__(TPB)
    k_dp_init(uint64_t P, const uint32_t* __restrict__ pring, const uint64_t* __restrict__ poff,
              uint8_t* __restrict__ keep, uint8_t* __restrict__ open, uint32_t* __restrict__ rend,
              uint32_t* __restrict__ lend) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t k = pring[i];
    const uint64_t a = poff[k], b = poff[k + 1] - 1;
    const bool small = b - a + 1 <= 2;  // rings of at most two points stay whole
    keep[i] = (small || i == a || i == b) ? 1 : 0;
    open[i] = (!small && i == a) ? 1 : 0;
    rend[i] = (uint32_t)b;
    lend[i] = (uint32_t)a;
  }
}

// One level: every interior point of an open range offers its distance to
// the range's chord (the maximum per range, then the first index of it).
__global__ void __launch_bounds__(TPB)
    k_dp_dist(uint64_t P, const double2* __restrict__ pts, const uint8_t* __restrict__ keep,
              const uint8_t* __restrict__ open, const uint32_t* __restrict__ rend,
              const uint32_t* __restrict__ lend, unsigned long long* __restrict__ dmax,
              double* __restrict__ dist) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (keep[i]) continue;
    const uint32_t a = lend[i];
    if (!open[a]) continue;
    const double d = seg_dist(pts[i], pts[a], pts[rend[a]]);
    dist[i] = d;
    // non-negative doubles order like their bit patterns
    atomicMax(&dmax[a], (unsigned long long)__double_as_longlong(d));
  }
}

__global__ void __launch_bounds__(TPB)
    k_dp_arg(uint64_t P, const uint8_t* __restrict__ keep, const uint8_t* __restrict__ open,
             const uint32_t* __restrict__ lend, const unsigned long long* __restrict__ dmax,
             const double* __restrict__ dist, uint32_t* __restrict__ imax) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (keep[i]) continue;
    const uint32_t a = lend[i];
    if (!open[a]) continue;
    if ((unsigned long long)__double_as_longlong(dist[i]) == dmax[a])
      atomicMin(&imax[a], (uint32_t)i);
  }
}

// Decide every open range [a, b]: split at its farthest point m when that
// distance exceeds the tolerance (and 0: the reference's strict comparison
// starts from 0), else close it. Only index a is written here (split_at[a],
// the old right end in rend_old[a], rend[a] = m); k_dp_apply opens [m, b].
// Counts the splits in *n_split.
__global__ void __launch_bounds__(TPB)
    k_dp_split(uint64_t P, const uint32_t* __restrict__ pring, const double* __restrict__ tol,
               uint8_t* __restrict__ open, uint32_t* __restrict__ rend,
               uint32_t* __restrict__ rend_old, unsigned long long* __restrict__ dmax,
               uint32_t* __restrict__ imax, uint32_t* __restrict__ split_at,
               uint32_t* __restrict__ n_split) {
  for (uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; a < P;
       a += (uint64_t)gridDim.x * blockDim.x) {
    split_at[a] = NONE;
    if (!open[a]) continue;
    const double d = __longlong_as_double((long long)dmax[a]);
    const uint32_t m = imax[a];
    dmax[a] = 0;
    imax[a] = NONE;
    if (m != NONE && d > 0.0 && d > tol[pring[a]]) {
      rend_old[a] = rend[a];
      rend[a] = m;
      split_at[a] = m;
      atomicAdd(n_split, 1u);
    } else {
      open[a] = 0;
    }
  }
}

// Open the right halves [m, b] of the splits, and move the interior points
// right of a split point to their new range.
__global__ void __launch_bounds__(TPB)
    k_dp_apply(uint64_t P, uint8_t* __restrict__ keep, uint8_t* __restrict__ open,
               uint32_t* __restrict__ rend, const uint32_t* __restrict__ rend_old,
               const uint32_t* __restrict__ split_at, uint32_t* __restrict__ lend) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t m = split_at[i];
    if (m != NONE) {  // i opened a range that was split at m
      keep[m] = 1;
      open[m] = 1;
      rend[m] = rend_old[i];
    }
    if (!keep[i]) {
      const uint32_t mm = split_at[lend[i]];
      if (mm != NONE && i > mm) lend[i] = mm;
    }
  }
}

struct KeepVal {
  const uint8_t* k;
  __device__ uint32_t operator()(uint64_t i) const { return k[i]; }
};

__global__ void __launch_bounds__(TPB)
    k_dp_out(uint64_t P, const uint8_t* __restrict__ keep, const uint32_t* __restrict__ kpre,
             const double2* __restrict__ pts, double2* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (keep[i]) out[kpre[i]] = pts[i];
}

// Device buffers of the tracer, kept per device (grow-only; calls on one
// device are serialised by the mutex).
enum TSlot {
  T_ISO, T_BMASK, T_BPRE, T_BSUM, T_CISO, T_CPOS, T_CCODE, T_EBASE, T_SUCC, T_PRED, T_CELL,
  T_KEY, T_KEY2, T_P2, T_START, T_EMIT, T_Q, T_Q2, T_DV, T_DV2, T_DONE, T_DONE2, T_RPRE, T_RINGS,
  T_RINGV, T_VOFF, T_VTMP, T_VERTS, T_VRING, T_CROSS, T_NEAR, T_BEST, T_LON, T_LAT, T_POFF,
  T_PTS, T_PRING, T_KEEP, T_OPEN, T_REND, T_ROLD, T_LEND, T_DMAX, T_IMAX, T_DIST, T_SPLIT, T_TOL,
  T_KPRE, T_OUT, T_ERR, T_PACK, T_SRCOFF, T_NS
};
struct TWork {
  std::mutex mu;
  void* buf[T_NS] = {};
  size_t cap[T_NS] = {};
  uint32_t* h_small = nullptr;  // page-locked read-back words
};
TWork& twork(int device) {
  static TWork w[64];
  return w[device];
}
template <class T>
cudaError_t tget(TWork& w, int i, size_t count, T** p) {
  const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
  if (w.cap[i] < bytes) {
    if (w.buf[i]) cudaFree(w.buf[i]);
    w.buf[i] = nullptr;
    w.cap[i] = 0;
    const size_t want = bytes + bytes / 4;
    const cudaError_t e = cudaMalloc(&w.buf[i], want);
    if (e != cudaSuccess) return e;
    w.cap[i] = want;
  }
  *p = reinterpret_cast<T*>(w.buf[i]);
  return cudaSuccess;
}

}  // namespace

bf_status trace_rings_device(const uint64_t* d_words, const bf_raster* ras, uint32_t n_iso,
                             const double* cell_m, const double* simplify_m,
                             const uint8_t* has_anchor, const double* anchor_xy, cudaStream_t st,
                             std::vector<uint64_t>& ring_off, std::vector<double>& lonlat) {
  ring_off.assign((size_t)n_iso + 1, 0);
  lonlat.clear();
  if (!n_iso) return BF_OK;
  int dev = 0;
  BF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("contour tracing: device ordinal out of range");
    return BF_ERR_INVALID;
  }
  TWork& w = twork(dev);
  std::lock_guard<std::mutex> lk(w.mu);
  cudaError_t e = cudaSuccess;
  auto get = [&](int i, size_t count, auto** p) {
    if (e == cudaSuccess) e = tget(w, i, count, p);
  };
  // host: raster table and the back-projection tables (host libm)
  std::vector<TIso> iso(n_iso);
  std::vector<uint64_t> src_off(n_iso);
  uint64_t TW = 0, nlon = 0, nlat = 0;
  for (uint32_t k = 0; k < n_iso; ++k) {
    const bf_raster& R = ras[k];
    TIso& t = iso[k];
    t.col0 = R.col0;
    t.row0 = R.row0;
    t.wpr = R.width_words;
    t.height = R.height;
    t.woff = TW;  // packed, raster after raster
    src_off[k] = R.word_offset;
    t.lon_off = nlon;
    t.lat_off = nlat;
    t.has_anchor = (has_anchor && has_anchor[k]) ? 1u : 0u;
    t.pad = 0;
    t.ax = t.has_anchor ? (anchor_xy[2 * k] - R.origin_x) / cell_m[k] : 0.0;
    t.ay = t.has_anchor ? (anchor_xy[2 * k + 1] - R.origin_y) / cell_m[k] : 0.0;
    nlon += (uint64_t)R.width_words * 64;
    nlat += R.height;
    TW += (uint64_t)R.width_words * R.height;
  }
  std::vector<double> lon(std::max<uint64_t>(nlon, 1)), lat(std::max<uint64_t>(nlat, 1));
  parallel_for(n_iso, [&](uint64_t k) {
    const bf_raster& R = ras[k];
    const double cell = cell_m[k];
    for (uint64_t c = 0; c < (uint64_t)R.width_words * 64; ++c) {
      const double x = R.origin_x + ((double)(R.col0 + (int64_t)c) + 0.5) * cell;
      lon[iso[k].lon_off + c] = (x / EARTH_R_T) * (180.0 / PI_T);
    }
    for (uint64_t r = 0; r < R.height; ++r) {
      const double y = R.origin_y + ((double)(R.row0 + (int64_t)r) + 0.5) * cell;
      lat[iso[k].lat_off + r] =
          (2.0 * std::atan(std::exp(y / EARTH_R_T)) - PI_T / 2.0) * (180.0 / PI_T);
    }
  });
  std::vector<double> tol(n_iso);
  for (uint32_t k = 0; k < n_iso; ++k) tol[k] = simplify_m[k] / 111000.0;
  if (!w.h_small) BF_CUDA(cudaHostAlloc((void**)&w.h_small, 64, cudaHostAllocDefault));
  TIso* d_iso;
  uint64_t* d_bmask;
  uint32_t *d_bpre, *d_bsum, *d_err;
  double *d_lon, *d_lat;
  get(T_ISO, n_iso, &d_iso);
  get(T_BMASK, TW, &d_bmask);
  get(T_BPRE, TW + 1, &d_bpre);
  get(T_BSUM, (TW + 1) / SCAN_BLOCK + 4, &d_bsum);
  get(T_ERR, 2, &d_err);
  get(T_LON, lon.size(), &d_lon);
  get(T_LAT, lat.size(), &d_lat);
  if (e != cudaSuccess) return cuda_status(e, "contour tracing: device memory");
  BF_CUDA(cudaMemcpyAsync(d_iso, iso.data(), n_iso * sizeof(TIso), cudaMemcpyHostToDevice, st));
  BF_CUDA(cudaMemcpyAsync(d_lon, lon.data(), lon.size() * 8, cudaMemcpyHostToDevice, st));
  BF_CUDA(cudaMemcpyAsync(d_lat, lat.data(), lat.size() * 8, cudaMemcpyHostToDevice, st));
  BF_CUDA(cudaMemsetAsync(d_err, 0, 8, st));
  {  // the rasters, packed in raster order
    uint64_t *d_pack, *d_src;
    get(T_PACK, TW, &d_pack);
    get(T_SRCOFF, n_iso, &d_src);
    if (e != cudaSuccess) return cuda_status(e, "contour tracing: device memory");
    BF_CUDA(cudaMemcpyAsync(d_src, src_off.data(), n_iso * 8, cudaMemcpyHostToDevice, st));
    if (TW) k_tr_pack<<<grid(TW), TPB, 0, st>>>(d_words, d_iso, n_iso, d_src, TW, d_pack);
    d_words = d_pack;
  }
  // boundary cells and their edges
  if (TW) k_tr_mask<<<grid(TW), TPB, 0, st>>>(d_words, d_iso, n_iso, TW, d_bmask);
  scan_launch<uint32_t>(PopVal64{d_bmask}, TW, d_bsum, d_bpre, st);
  BF_CUDA(cudaMemcpyAsync(w.h_small, d_bpre + TW, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  const uint32_t BC = w.h_small[0];
  uint32_t *d_ciso, *d_ccode, *d_ebase;
  uint2* d_cpos;
  get(T_CISO, BC, &d_ciso);
  get(T_CPOS, BC, &d_cpos);
  get(T_CCODE, BC, &d_ccode);
  get(T_EBASE, (uint64_t)BC + 1, &d_ebase);
  get(T_BSUM, ((uint64_t)BC + 1) / SCAN_BLOCK + 4, &d_bsum);
  if (e != cudaSuccess) return cuda_status(e, "contour tracing: device memory");
  if (TW)
    k_tr_cells<<<grid(TW), TPB, 0, st>>>(d_words, d_iso, n_iso, TW, d_bmask, d_bpre, d_ciso,
                                         d_cpos, d_ccode);
  scan_launch<uint32_t>(EdgeCountVal{d_ccode}, BC, d_bsum, d_ebase, st);
  BF_CUDA(cudaMemcpyAsync(w.h_small, d_ebase + BC, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  const uint32_t E = w.h_small[0];
  if (!E) return BF_OK;  // no set cell in any raster: no rings
  uint32_t *d_succ, *d_pred, *d_cell, *d_p2, *d_start, *d_emit, *d_q, *d_q2, *d_rpre;
  uint64_t *d_key, *d_key2, *d_dv, *d_dv2;
  uint8_t *d_done, *d_done2;
  get(T_SUCC, E, &d_succ);
  get(T_PRED, E, &d_pred);
  get(T_CELL, E, &d_cell);
  get(T_KEY, E, &d_key);
  get(T_KEY2, E, &d_key2);
  get(T_P2, E, &d_p2);
  get(T_START, E, &d_start);
  get(T_EMIT, E, &d_emit);
  get(T_Q, E, &d_q);
  get(T_Q2, E, &d_q2);
  get(T_DV, E, &d_dv);
  get(T_DV2, E, &d_dv2);
  get(T_DONE, E, &d_done);
  get(T_DONE2, E, &d_done2);
  get(T_RPRE, (uint64_t)E + 1, &d_rpre);
  get(T_BSUM, ((uint64_t)E + 1) / SCAN_BLOCK + 4, &d_bsum);
  if (e != cudaSuccess) return cuda_status(e, "contour tracing: device memory");
  k_tr_succ<<<grid(BC), TPB, 0, st>>>(d_words, d_iso, BC, d_bmask, d_bpre, d_ciso, d_cpos, d_ccode,
                                      d_ebase, d_succ, d_cell, d_key, d_err);
  // predecessors: the successors are a permutation of the edges
  k_tr_pred<<<grid(E), TPB, 0, st>>>(E, d_succ, d_pred);
  // the smallest start key of every cycle by pointer jumping (on d_key /
  // d_key2 and a copy of the successors in d_p2 / d_q2)
  uint32_t rounds = 1;
  while ((1ull << rounds) < E) ++rounds;
  BF_CUDA(cudaMemcpyAsync(d_p2, d_succ, (size_t)E * 4, cudaMemcpyDeviceToDevice, st));
  uint64_t *m = d_key, *m2 = d_key2;
  uint32_t *p = d_p2, *p2 = d_q2;
  for (uint32_t r = 0; r < rounds; ++r) {
    k_tr_jump_min<<<grid(E), TPB, 0, st>>>(E, m, p, m2, p2);
    std::swap(m, m2);
    std::swap(p, p2);
  }
  const uint64_t* d_cyc = m;  // d_key or d_key2, untouched from here on
  k_tr_start<<<grid(E), TPB, 0, st>>>(E, d_cyc, d_cell, d_pred, d_iso, d_ciso, d_bmask, d_bpre,
                                      d_ccode, d_ebase, d_start, d_emit);
  // list ranking from each ring's start
  k_tr_rank_init<<<grid(E), TPB, 0, st>>>(E, d_succ, d_start, d_emit, d_q, d_dv, d_done);
  uint32_t *q = d_q, *q2 = d_q2;
  uint64_t *dv = d_dv, *dv2 = d_dv2;
  uint8_t *dn = d_done, *dn2 = d_done2;
  for (uint32_t r = 0; r < rounds; ++r) {
    k_tr_rank<<<grid(E), TPB, 0, st>>>(E, q, dv, dn, q2, dv2, dn2);
    std::swap(q, q2);
    std::swap(dv, dv2);
    std::swap(dn, dn2);
  }
  scan_launch<uint32_t>(RingHeadVal{d_start}, E, d_bsum, d_rpre, st);
  BF_CUDA(cudaMemcpyAsync(w.h_small, d_rpre + E, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaMemcpyAsync(w.h_small + 1, d_err, 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  if (w.h_small[1]) {
    set_error("contour tracing: a boundary edge's successor is no boundary edge");
    return BF_ERR_DEVICE;
  }
  const uint32_t NR = w.h_small[0];
  Ring* d_rings;
  uint32_t *d_ringv, *d_vtmp, *d_cross, *d_near, *d_best;
  uint64_t* d_voff;
  get(T_RINGS, NR, &d_rings);
  get(T_RINGV, NR, &d_ringv);
  get(T_VTMP, (uint64_t)NR + 1, &d_vtmp);
  get(T_VOFF, (uint64_t)NR + 1, &d_voff);
  get(T_CROSS, NR, &d_cross);
  get(T_NEAR, NR, &d_near);
  get(T_BEST, n_iso, &d_best);
  if (e != cudaSuccess) return cuda_status(e, "contour tracing: device memory");
  if (NR) {
    k_tr_rings<<<grid(E), TPB, 0, st>>>(E, d_start, d_rpre, dv, d_pred, d_cell, d_ciso, d_cyc,
                                        d_rings, d_ringv);
    // vertex offsets from a u32 scan of the emitted counts (fewer than 2^32
    // boundary edges bound every total)
    scan_launch<uint32_t>(U32Val{d_ringv}, NR, d_bsum, d_vtmp, st);
  }
  std::vector<uint32_t> vtmp((size_t)NR + 1, 0);
  if (NR)
    BF_CUDA(cudaMemcpyAsync(vtmp.data(), d_vtmp, ((size_t)NR + 1) * 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  std::vector<uint64_t> voff(vtmp.begin(), vtmp.end());
  const uint64_t NV = voff[NR];
  uint2* d_verts;
  uint32_t* d_vring;
  get(T_VERTS, NV, &d_verts);
  get(T_VRING, NV, &d_vring);
  if (e != cudaSuccess) return cuda_status(e, "contour tracing: device memory");
  if (NR) {
    BF_CUDA(cudaMemcpyAsync(d_voff, voff.data(), voff.size() * 8, cudaMemcpyHostToDevice, st));
    k_tr_verts<<<grid(E), TPB, 0, st>>>(E, d_start, d_emit, d_rpre, dv, d_cell, d_cpos, d_rings,
                                        d_voff, d_verts);
    BF_CUDA(cudaMemsetAsync(d_cross, 0, (size_t)NR * 4, st));
    BF_CUDA(cudaMemsetAsync(d_near, 0, (size_t)NR * 4, st));
    if (has_anchor && NV) {
      k_tr_vring<<<std::min<uint32_t>(NR, 152 * 8), 128, 0, st>>>(NR, d_voff, d_vring);
      k_tr_anchor<<<grid(NV), TPB, 0, st>>>(NV, d_vring, d_rings, d_voff, d_verts, d_iso, d_cross,
                                            d_near);
    }
  }
  k_tr_choose<<<(n_iso + 127) / 128, 128, 0, st>>>(n_iso, NR, d_rings, d_cross, d_near, d_iso,
                                                  d_best);
  BF_CUDA(cudaGetLastError());
  // chosen ring sizes -> point offsets
  std::vector<uint32_t> best(n_iso);
  std::vector<Ring> hr(NR);
  BF_CUDA(cudaMemcpyAsync(best.data(), d_best, n_iso * 4, cudaMemcpyDeviceToHost, st));
  if (NR) BF_CUDA(cudaMemcpyAsync(hr.data(), d_rings, NR * sizeof(Ring), cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  std::vector<uint64_t> poff((size_t)n_iso + 1, 0);
  for (uint32_t k = 0; k < n_iso; ++k)
    poff[k + 1] = poff[k] + (best[k] == NONE ? 0 : hr[best[k]].size);
  const uint64_t P = poff[n_iso];
  if (!P) return BF_OK;
  uint64_t* d_poff;
  double2 *d_pts, *d_out;
  uint32_t *d_pring, *d_rend, *d_rold, *d_lend, *d_imax, *d_split, *d_kpre;
  uint8_t *d_keep, *d_open;
  unsigned long long* d_dmax;
  double *d_dist, *d_tol;
  get(T_POFF, (uint64_t)n_iso + 1, &d_poff);
  get(T_PTS, P, &d_pts);
  get(T_PRING, P, &d_pring);
  get(T_KEEP, P, &d_keep);
  get(T_OPEN, P, &d_open);
  get(T_REND, P, &d_rend);
  get(T_ROLD, P, &d_rold);
  get(T_LEND, P, &d_lend);
  get(T_DMAX, P, &d_dmax);
  get(T_IMAX, P, &d_imax);
  get(T_DIST, P, &d_dist);
  get(T_SPLIT, P, &d_split);
  get(T_TOL, n_iso, &d_tol);
  get(T_KPRE, P + 1, &d_kpre);
  get(T_OUT, P, &d_out);
  get(T_BSUM, (P + 1) / SCAN_BLOCK + 4, &d_bsum);
  if (e != cudaSuccess) return cuda_status(e, "contour tracing: device memory");
  BF_CUDA(cudaMemcpyAsync(d_poff, poff.data(), poff.size() * 8, cudaMemcpyHostToDevice, st));
  BF_CUDA(cudaMemcpyAsync(d_tol, tol.data(), n_iso * 8, cudaMemcpyHostToDevice, st));
  k_tr_project<<<std::min<uint32_t>(n_iso, 152 * 8), TPB, 0, st>>>(
      n_iso, d_best, d_voff, d_verts, d_poff, d_iso, d_lon, d_lat, d_pts, d_pring);
  // Douglas-Peucker: levels until one splits nothing (every open range then
  // closed); the split count is read back every fourth level
  k_dp_init<<<grid(P), TPB, 0, st>>>(P, d_pring, d_poff, d_keep, d_open, d_rend, d_lend);
  BF_CUDA(cudaMemsetAsync(d_dmax, 0, P * 8, st));
  BF_CUDA(cudaMemsetAsync(d_imax, 0xFF, P * 4, st));
  for (uint32_t level = 0;; ++level) {
    BF_CUDA(cudaMemsetAsync(d_err + 1, 0, 4, st));
    k_dp_dist<<<grid(P), TPB, 0, st>>>(P, d_pts, d_keep, d_open, d_rend, d_lend, d_dmax, d_dist);
    k_dp_arg<<<grid(P), TPB, 0, st>>>(P, d_keep, d_open, d_lend, d_dmax, d_dist, d_imax);
    k_dp_split<<<grid(P), TPB, 0, st>>>(P, d_pring, d_tol, d_open, d_rend, d_rold, d_dmax, d_imax,
                                        d_split, d_err + 1);
    k_dp_apply<<<grid(P), TPB, 0, st>>>(P, d_keep, d_open, d_rend, d_rold, d_split, d_lend);
    BF_CUDA(cudaGetLastError());
    if (level % 4 == 3) {
      BF_CUDA(cudaMemcpyAsync(w.h_small, d_err + 1, 4, cudaMemcpyDeviceToHost, st));
      BF_CUDA(cudaStreamSynchronize(st));
      if (w.h_small[0] == 0) break;
      if (level > (uint32_t)P) {  // every split keeps a new point: cannot happen
        set_error("contour tracing: simplification did not converge");
        return BF_ERR_DEVICE;
      }
    }
  }
  scan_launch<uint32_t>(KeepVal{d_keep}, P, d_bsum, d_kpre, st);
  k_dp_out<<<grid(P), TPB, 0, st>>>(P, d_keep, d_kpre, d_pts, d_out);
  std::vector<uint32_t> kpre(P + 1);
  BF_CUDA(cudaMemcpyAsync(kpre.data(), d_kpre, (P + 1) * 4, cudaMemcpyDeviceToHost, st));
  BF_CUDA(cudaStreamSynchronize(st));
  const uint64_t K = kpre[P];
  lonlat.resize(2 * K);
  if (K) BF_CUDA(cudaMemcpyAsync(lonlat.data(), d_out, K * 16, cudaMemcpyDeviceToHost, st));
  for (uint32_t k = 0; k <= n_iso; ++k) ring_off[k] = kpre[poff[k]];
  BF_CUDA(cudaStreamSynchronize(st));
  return BF_OK;
}

}  // namespace bf
