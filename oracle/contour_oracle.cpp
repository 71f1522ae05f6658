// contour_oracle.cpp — CPU restatement of the reference's isochrone geometry
// (test infrastructure, never part of the product): the reachable segments of
// a settled set (route/src/server/geometry.rs:281-418) and the sparse-tile
// contour (route/src/range/sparse_contour.rs:17-1185): Mercator projection,
// 64x64-cell tiles, Bresenham stamping, 3x3 dilation / erosion, Moore
// boundary tracing with cell-centre vertices, anchored ring selection and
// Douglas-Peucker simplification. Built with -ffp-contract=off so every
// floating-point step rounds as written.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace {

constexpr int TILE = 64;
constexpr double EARTH_R = 6378137.0;               // sparse_contour.rs:439
constexpr double PI_ = 3.14159265358979323846264338;  // std::f64::consts::PI

using Tile = std::array<uint64_t, TILE>;

struct Merc {
  double x, y;
};

// to_mercator / from_mercator (sparse_contour.rs:441-451); to_radians is
// x * (PI / 180), to_degrees x * (180 / PI), as in Rust's f64.
Merc to_merc(double lat, double lon) {
  const double x = lon * (PI_ / 180.0) * EARTH_R;
  const double y = std::log(std::tan(lat * (PI_ / 180.0) / 2.0 + PI_ / 4.0)) * EARTH_R;
  return {x, y};
}
void from_merc(double x, double y, double* lon, double* lat) {
  *lon = (x / EARTH_R) * (180.0 / PI_);
  *lat = (2.0 * std::atan(std::exp(y / EARTH_R)) - PI_ / 2.0) * (180.0 / PI_);
}

uint64_t tkey(int32_t tx, int32_t ty) { return ((uint64_t)(uint32_t)tx << 32) | (uint32_t)ty; }
int32_t tx_of(uint64_t k) { return (int32_t)(uint32_t)(k >> 32); }
int32_t ty_of(uint64_t k) { return (int32_t)(uint32_t)k; }

// SparseTileMap (sparse_contour.rs:60-170): tiles of 64 rows x 64 columns,
// bit c of row r = cell (c, r); tile and local coordinates by Euclidean
// division (arithmetic shift and mask on two's complement).
struct TileMap {
  std::unordered_map<uint64_t, Tile> tiles;
  double cell = 1, ox = 0, oy = 0;

  void cell_of(double x, double y, int32_t* c, int32_t* r) const {
    *c = (int32_t)std::floor((x - ox) / cell);
    *r = (int32_t)std::floor((y - oy) / cell);
  }
  void set(int32_t c, int32_t r) {
    auto it = tiles.find(tkey(c >> 6, r >> 6));
    if (it == tiles.end()) it = tiles.emplace(tkey(c >> 6, r >> 6), Tile{}).first;
    it->second[r & 63] |= 1ull << (c & 63);
  }
  bool get(int32_t c, int32_t r) const {
    auto it = tiles.find(tkey(c >> 6, r >> 6));
    return it != tiles.end() && ((it->second[r & 63] >> (c & 63)) & 1);
  }
  const Tile& bits(int32_t tx, int32_t ty) const {
    static const Tile empty{};
    auto it = tiles.find(tkey(tx, ty));
    return it == tiles.end() ? empty : it->second;
  }
  // stamp_line (sparse_contour.rs:112-144): Bresenham between the two cells
  void stamp_line(double x0, double y0, double x1, double y1) {
    int32_t c0, r0, c1, r1;
    cell_of(x0, y0, &c0, &r0);
    cell_of(x1, y1, &c1, &r1);
    const int32_t dx = std::abs(c1 - c0), dy = std::abs(r1 - r0);
    const int32_t sx = c0 < c1 ? 1 : -1, sy = r0 < r1 ? 1 : -1;
    int32_t err = dx - dy, c = c0, r = r0;
    for (;;) {
      set(c, r);
      if (c == c1 && r == r1) break;
      const int32_t e2 = 2 * err;
      if (e2 > -dy) {
        err -= dy;
        c += sx;
      }
      if (e2 < dx) {
        err += dx;
        r += sy;
      }
    }
  }
};

// dilate_sparse / erode_sparse (sparse_contour.rs:184-431): 3x3 OR / AND,
// neighbour tiles supplying the edge bits, absent tiles reading as zero.
template <bool DILATE>
Tile morph_tile(const TileMap& m, int32_t tx, int32_t ty) {
  const Tile& C = m.bits(tx, ty);
  const Tile& A = m.bits(tx, ty - 1);
  const Tile& B = m.bits(tx, ty + 1);
  const Tile& L = m.bits(tx - 1, ty);
  const Tile& R = m.bits(tx + 1, ty);
  const Tile& AL = m.bits(tx - 1, ty - 1);
  const Tile& AR = m.bits(tx + 1, ty - 1);
  const Tile& BL = m.bits(tx - 1, ty + 1);
  const Tile& BR = m.bits(tx + 1, ty + 1);
  auto horiz = [](uint64_t row, uint64_t left_row, uint64_t right_row) {
    const uint64_t lb = (left_row >> 63) & 1, rb = (right_row & 1) << 63;
    return DILATE ? (row | (row << 1) | (row >> 1) | lb | rb)
                  : (row & ((row << 1) | lb) & ((row >> 1) | rb));
  };
  Tile out{};
  for (int r = 0; r < TILE; ++r) {
    const uint64_t cur = horiz(C[r], L[r], R[r]);
    const uint64_t up = r == 0 ? horiz(A[TILE - 1], AL[TILE - 1], AR[TILE - 1])
                               : horiz(C[r - 1], L[r - 1], R[r - 1]);
    const uint64_t dn = r == TILE - 1 ? horiz(B[0], BL[0], BR[0]) : horiz(C[r + 1], L[r + 1], R[r + 1]);
    out[r] = DILATE ? (cur | up | dn) : (cur & up & dn);
  }
  return out;
}

bool tile_empty(const Tile& t) {
  for (uint64_t w : t)
    if (w) return false;
  return true;
}

TileMap dilate(const TileMap& m) {
  TileMap out;
  out.cell = m.cell;
  out.ox = m.ox;
  out.oy = m.oy;
  std::unordered_set<uint64_t> halo;
  for (const auto& kv : m.tiles)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) halo.insert(tkey(tx_of(kv.first) + dx, ty_of(kv.first) + dy));
  for (uint64_t k : halo) {
    Tile t = morph_tile<true>(m, tx_of(k), ty_of(k));
    if (!tile_empty(t)) out.tiles.emplace(k, t);
  }
  return out;
}

TileMap erode(const TileMap& m) {
  TileMap out;
  out.cell = m.cell;
  out.ox = m.ox;
  out.oy = m.oy;
  for (const auto& kv : m.tiles) {
    Tile t = morph_tile<false>(m, tx_of(kv.first), ty_of(kv.first));
    if (!tile_empty(t)) out.tiles.emplace(kv.first, t);
  }
  return out;
}

using Pt = std::pair<double, double>;
using Ring = std::vector<Pt>;

// next_boundary_edge (sparse_contour.rs:1049-1130): clockwise walk, filled on
// the right; edges N = 0, E = 1, S = 2, W = 3.
std::tuple<int32_t, int32_t, uint8_t> next_edge(const TileMap& m, int32_t c, int32_t r, uint8_t e) {
  switch (e) {
    case 0:
      if (m.get(c + 1, r - 1)) return {c + 1, r - 1, 3};
      if (m.get(c + 1, r)) return {c + 1, r, 0};
      return {c, r, 1};
    case 1:
      if (m.get(c + 1, r + 1)) return {c + 1, r + 1, 0};
      if (m.get(c, r + 1)) return {c, r + 1, 1};
      return {c, r, 2};
    case 2:
      if (m.get(c - 1, r + 1)) return {c - 1, r + 1, 1};
      if (m.get(c - 1, r)) return {c - 1, r, 2};
      return {c, r, 3};
    default:
      if (m.get(c - 1, r - 1)) return {c - 1, r - 1, 2};
      if (m.get(c, r - 1)) return {c, r - 1, 3};
      return {c, r, 0};
  }
}

uint64_t ekey(int32_t c, int32_t r, uint8_t e) {
  return ((uint64_t)(uint32_t)c << 34) ^ ((uint64_t)(uint32_t)r << 2) ^ e;
}

struct EdgeKeyHash {
  size_t operator()(const std::tuple<int32_t, int32_t, uint8_t>& t) const {
    return std::hash<uint64_t>()(ekey(std::get<0>(t), std::get<1>(t), std::get<2>(t)));
  }
};
using Visited = std::unordered_set<std::tuple<int32_t, int32_t, uint8_t>, EdgeKeyHash>;

// trace_boundary_edges_with_visited (sparse_contour.rs:976-1046)
Ring trace(const TileMap& m, int32_t sc, int32_t sr, uint8_t se, Visited& visited) {
  Ring ring;
  int32_t c = sc, r = sr;
  uint8_t e = se;
  const size_t max_iter = m.tiles.size() * TILE * TILE * 4;
  size_t iter = 0;
  for (;;) {
    if (++iter > max_iter) break;
    visited.insert({c, r, e});
    const Pt v{(double)c + 0.5, (double)r + 0.5};
    if (ring.empty() || ring.back() != v) ring.push_back(v);
    const auto nx = next_edge(m, c, r, e);
    if (std::get<0>(nx) == sc && std::get<1>(nx) == sr && std::get<2>(nx) == se) break;
    std::tie(c, r, e) = nx;
  }
  while (ring.size() > 1 && ring.back() == ring.front()) ring.pop_back();
  return ring;
}

bool ring_near(Pt p, const Ring& ring, double tol) {  // sparse_contour.rs:898-918
  const size_t n = ring.size();
  for (size_t i = 0; i < n; ++i) {
    const Pt a = ring[i], b = ring[(i + 1) % n];
    const double dx = b.first - a.first, dy = b.second - a.second;
    const double len2 = dx * dx + dy * dy;
    double t = 0.0;
    if (len2 > 0.0) t = std::clamp(((p.first - a.first) * dx + (p.second - a.second) * dy) / len2, 0.0, 1.0);
    const double cx = a.first + t * dx, cy = a.second + t * dy;
    if ((p.first - cx) * (p.first - cx) + (p.second - cy) * (p.second - cy) <= tol * tol) return true;
  }
  return false;
}

bool point_in_ring(Pt p, const Ring& ring) {  // sparse_contour.rs:920-933
  bool inside = false;
  const size_t n = ring.size();
  for (size_t i = 0; i < n; ++i) {
    const Pt a = ring[i], b = ring[(i + 1) % n];
    if ((a.second > p.second) != (b.second > p.second) &&
        p.first < (b.first - a.first) * (p.second - a.second) / (b.second - a.second) + a.first)
      inside = !inside;
  }
  return inside;
}

// extract_contour_sparse + find_all_boundary_starts (sparse_contour.rs:831-974)
Ring extract(const TileMap& m, const Pt* anchor) {
  if (m.tiles.empty()) return {};
  std::vector<std::tuple<int32_t, int32_t, uint8_t>> starts;
  for (const auto& kv : m.tiles) {
    const int32_t bc = tx_of(kv.first) * TILE, br = ty_of(kv.first) * TILE;
    for (int lr = 0; lr < TILE; ++lr) {
      const uint64_t bits = kv.second[lr];
      if (!bits) continue;
      for (int lc = 0; lc < TILE; ++lc) {
        if (!((bits >> lc) & 1)) continue;
        const int32_t c = bc + lc, r = br + lr;
        if (!m.get(c, r - 1))
          starts.emplace_back(c, r, 0);
        else if (!m.get(c - 1, r))
          starts.emplace_back(c, r, 3);
        else if (!m.get(c + 1, r))
          starts.emplace_back(c, r, 1);
        else if (!m.get(c, r + 1))
          starts.emplace_back(c, r, 2);
      }
    }
  }
  std::sort(starts.begin(), starts.end());
  Visited visited;
  std::vector<Ring> all;
  for (const auto& s : starts) {
    if (visited.count(s)) continue;
    Ring ring = trace(m, std::get<0>(s), std::get<1>(s), std::get<2>(s), visited);
    if (ring.size() >= 3) all.push_back(std::move(ring));
  }
  if (anchor) {
    const Ring* best = nullptr;
    for (const Ring& c : all)
      if ((point_in_ring(*anchor, c) || ring_near(*anchor, c, 1.0)) &&
          (!best || c.size() > best->size()))
        best = &c;
    if (best) return *best;
  }
  const Ring* best = nullptr;  // Iterator::max_by_key: the LAST maximum
  for (const Ring& c : all)
    if (!best || c.size() >= best->size()) best = &c;
  return best ? *best : Ring{};
}

double perp_dist(Pt p, Pt s, Pt e) {  // sparse_contour.rs:1161-1183
  const double dx = e.first - s.first, dy = e.second - s.second;
  const double len_sq = dx * dx + dy * dy;
  if (len_sq < 1e-12) {
    const double pdx = p.first - s.first, pdy = p.second - s.second;
    return std::sqrt(pdx * pdx + pdy * pdy);
  }
  double t = ((p.first - s.first) * dx + (p.second - s.second) * dy) / len_sq;
  t = std::clamp(t, 0.0, 1.0);
  const double px = s.first + t * dx, py = s.second + t * dy;
  const double pdx = p.first - px, pdy = p.second - py;
  return std::sqrt(pdx * pdx + pdy * pdy);
}

Ring douglas_peucker(const Ring& pts, double tol) {  // sparse_contour.rs:1132-1159
  if (pts.size() <= 2) return pts;
  double max_d = 0.0;
  size_t max_i = 0;
  for (size_t i = 1; i + 1 < pts.size(); ++i) {
    const double d = perp_dist(pts[i], pts.front(), pts.back());
    if (d > max_d) {
      max_d = d;
      max_i = i;
    }
  }
  if (max_d > tol) {
    Ring left = douglas_peucker(Ring(pts.begin(), pts.begin() + max_i + 1), tol);
    Ring right = douglas_peucker(Ring(pts.begin() + max_i, pts.end()), tol);
    left.pop_back();
    left.insert(left.end(), right.begin(), right.end());
    return left;
  }
  return {pts.front(), pts.back()};
}

struct Config {
  double cell;
  int dil, ero;
  double simplify_m;
};

// SparseContourConfig::for_mode_name_with_threshold (sparse_contour.rs:476-546)
Config config_for(int mode, uint32_t threshold_s) {
  Config b = mode == 1 ? Config{40.0, 3, 3, 40.0} : mode == 2 ? Config{25.0, 3, 3, 25.0}
                                                                : Config{30.0, 2, 2, 30.0};
  double cm, sm;
  if (threshold_s <= 600) {
    cm = 1.0;
    sm = 1.0;
  } else if (threshold_s <= 1800) {
    cm = 2.0;
    sm = 2.0;
  } else if (threshold_s <= 3600) {
    cm = 4.0;
    sm = 4.0;
  } else {
    cm = 6.67;
    sm = 8.0;
  }
  return Config{b.cell * cm, b.dil, b.ero, b.simplify_m * sm};
}

struct Closed {
  TileMap map;
  double min_x, min_y;
  bool has_anchor;
  Pt anchor_cell;
};

// Steps 1-3 of generate_sparse_contour_anchored (sparse_contour.rs:650-770):
// project, stamp lines and points, stamp the anchor's 3x3 disk, close.
Closed stamp_and_close(const std::vector<std::vector<std::pair<int32_t, int32_t>>>& segs,
                       const Config& cfg, const std::pair<int32_t, int32_t>* anchor) {
  double min_x = INFINITY, min_y = INFINITY;
  std::vector<std::vector<Merc>> ms(segs.size());
  for (size_t i = 0; i < segs.size(); ++i)
    for (const auto& p : segs[i]) {
      const Merc q = to_merc((double)p.first / 1e7, (double)p.second / 1e7);
      min_x = std::min(min_x, q.x);
      min_y = std::min(min_y, q.y);
      ms[i].push_back(q);
    }
  const double margin = cfg.cell * 3.0;
  min_x -= margin;
  min_y -= margin;
  Closed out;
  TileMap& m = out.map;
  m.cell = cfg.cell;
  m.ox = min_x;
  m.oy = min_y;
  for (const auto& s : ms) {
    for (size_t k = 0; k + 1 < s.size(); ++k) m.stamp_line(s[k].x, s[k].y, s[k + 1].x, s[k + 1].y);
    for (const auto& q : s) {
      int32_t c, r;
      m.cell_of(q.x, q.y, &c, &r);
      m.set(c, r);
    }
  }
  out.has_anchor = anchor != nullptr;
  if (anchor) {
    const Merc q = to_merc((double)anchor->first / 1e7, (double)anchor->second / 1e7);
    int32_t c, r;
    m.cell_of(q.x, q.y, &c, &r);
    for (int dc = -1; dc <= 1; ++dc)
      for (int dr = -1; dr <= 1; ++dr) m.set(c + dc, r + dr);
    out.anchor_cell = {(q.x - min_x) / cfg.cell, (q.y - min_y) / cfg.cell};
  }
  for (int i = 0; i < cfg.dil; ++i) m = dilate(m);
  for (int i = 0; i < cfg.ero; ++i) m = erode(m);
  out.min_x = min_x;
  out.min_y = min_y;
  return out;
}

// Steps 4-5: trace, back to WGS84 (lon, lat), simplify.
Ring contour_of(const Closed& cl, const Config& cfg) {
  const Ring cells = extract(cl.map, cl.has_anchor ? &cl.anchor_cell : nullptr);
  if (cells.empty()) return {};
  Ring wgs;
  wgs.reserve(cells.size());
  for (const Pt& p : cells) {
    double lon, lat;
    from_merc(cl.min_x + p.first * cfg.cell, cl.min_y + p.second * cfg.cell, &lon, &lat);
    wgs.emplace_back(lon, lat);
  }
  return douglas_peucker(wgs, cfg.simplify_m / 111000.0);
}

using Segs = std::vector<std::vector<std::pair<int32_t, int32_t>>>;

Segs read_segs(uint32_t n_seg, const uint64_t* off, const int32_t* pts) {
  Segs s(n_seg);
  for (uint32_t i = 0; i < n_seg; ++i)
    for (uint64_t k = off[i]; k < off[i + 1]; ++k) s[i].emplace_back(pts[2 * k], pts[2 * k + 1]);
  return s;
}

uint64_t emit(const Ring& r, double* out, uint64_t cap) {
  for (uint64_t i = 0; i < r.size() && i < cap; ++i) {
    out[2 * i] = r[i].first;
    out[2 * i + 1] = r[i].second;
  }
  return r.size();
}

}  // namespace

extern "C" {

// extract_contour_sparse on the cells (col, row) of a unit-cell map; the
// anchor (in cell units) when has_anchor. Writes up to cap (x, y) vertices,
// returns the ring's length.
uint64_t orc_contour_cells(uint64_t n_cells, const int32_t* cells, int has_anchor, double ax,
                           double ay, double* out, uint64_t cap) {
  TileMap m;
  for (uint64_t i = 0; i < n_cells; ++i) m.set(cells[2 * i], cells[2 * i + 1]);
  const Pt a{ax, ay};
  return emit(extract(m, has_anchor ? &a : nullptr), out, cap);
}

// generate_sparse_contour_anchored: segments of (lat_e7, lon_e7) points
// (segment i = points [off[i], off[i + 1])), explicit morphology and
// simplification; the outer ring as (lon, lat) pairs.
uint64_t orc_sparse_contour(uint32_t n_seg, const uint64_t* off, const int32_t* pts,
                            double cell_m, int dil, int ero, double simplify_m, int has_anchor,
                            int32_t a_lat, int32_t a_lon, double* out, uint64_t cap) {
  if (n_seg == 0) return 0;
  const Config cfg{cell_m, dil, ero, simplify_m};
  const std::pair<int32_t, int32_t> a{a_lat, a_lon};
  const Closed cl = stamp_and_close(read_segs(n_seg, off, pts), cfg, has_anchor ? &a : nullptr);
  return emit(contour_of(cl, cfg), out, cap);
}

// Steps 1-3 of generate_sparse_contour_anchored only: the closed cell set of
// the segments, (col, row) pairs ascending by row then column (up to
// cell_cap), and the grid origin (min_x, min_y) in Mercator metres. Returns
// the number of closed cells.
uint64_t orc_sparse_closed(uint32_t n_seg, const uint64_t* off, const int32_t* pts,
                           double cell_m, int dil, int ero, int has_anchor, int32_t a_lat,
                           int32_t a_lon, int32_t* cells, uint64_t cell_cap,
                           double* grid_origin) {
  if (n_seg == 0) return 0;
  const Config cfg{cell_m, dil, ero, 0.0};
  const std::pair<int32_t, int32_t> a{a_lat, a_lon};
  const Closed cl = stamp_and_close(read_segs(n_seg, off, pts), cfg, has_anchor ? &a : nullptr);
  grid_origin[0] = cl.min_x;
  grid_origin[1] = cl.min_y;
  std::vector<std::pair<int32_t, int32_t>> set;
  for (const auto& kv : cl.map.tiles)
    for (int lr = 0; lr < TILE; ++lr)
      for (int lc = 0; lc < TILE; ++lc)
        if ((kv.second[lr] >> lc) & 1)
          set.emplace_back(ty_of(kv.first) * TILE + lr, tx_of(kv.first) * TILE + lc);
  std::sort(set.begin(), set.end());
  for (uint64_t i = 0; i < set.size() && i < cell_cap; ++i) {
    cells[2 * i] = set[i].second;
    cells[2 * i + 1] = set[i].first;
  }
  return set.size();
}

// SparseContourConfig::for_mode_name_with_threshold: mode 0 car, 1 bike,
// 2 foot (anything else: car).
void orc_contour_config(int mode, uint32_t threshold_s, double* cell_m, int* dil, int* ero,
                        double* simplify_m) {
  const Config c = config_for(mode, threshold_s);
  *cell_m = c.cell;
  *dil = c.dil;
  *ero = c.ero;
  *simplify_m = c.simplify_m;
}

// to_mercator / from_mercator on n points.
void orc_mercator(uint64_t n, const double* lat, const double* lon, double* x, double* y) {
  for (uint64_t i = 0; i < n; ++i) {
    const Merc q = to_merc(lat[i], lon[i]);
    x[i] = q.x;
    y[i] = q.y;
  }
}
void orc_inverse_mercator(uint64_t n, const double* x, const double* y, double* lon, double* lat) {
  for (uint64_t i = 0; i < n; ++i) from_merc(x[i], y[i], lon + i, lat + i);
}

// build_isochrone_geometry_sparse (server/geometry.rs:281-368) with
// extract_partial_polyline_view (:372-411): settled (node, dist) pairs, the
// threshold, per-node weights and (lat_e7, lon_e7) polylines
// (node i = points [poly_off[i], poly_off[i + 1])), the travel mode and an
// optional snapped origin (lon, lat). Also returns the closed cell set
// (col, row pairs, ascending by row then column, up to cell_cap) with the
// grid origin, for checking the rasterisation stage on its own. `tier` is
// the threshold that selects the contour configuration.
uint64_t orc_isochrone_geometry(uint64_t n_settled, const uint32_t* node, const uint32_t* dist,
                                uint32_t max_t, uint32_t n_nodes, const uint32_t* node_w,
                                const uint64_t* poly_off, const int32_t* poly, int mode,
                                int has_origin, double o_lon, double o_lat, double* out,
                                uint64_t cap, int32_t* cells, uint64_t cell_cap,
                                uint64_t* n_cells, double* grid_origin, uint32_t tier) {
  // the contour tier of `tier` (the reference passes its threshold; a
  // caller whose distances are not in seconds passes the seconds here)
  const Config cfg = config_for(mode, tier);
  Segs segs;
  bool have_anchor = false;
  std::pair<int32_t, int32_t> anchor{0, 0};
  uint32_t anchor_dist = 0xFFFFFFFFu;
  for (uint64_t i = 0; i < n_settled; ++i) {
    const uint32_t id = node[i], d = dist[i];
    if (d > max_t || id >= n_nodes) continue;
    const uint32_t w = node_w[id];
    if (w == 0 || w == 0xFFFFFFFFu) continue;
    const uint32_t d_end = (d + w < d) ? 0xFFFFFFFFu : d + w;
    const uint64_t p0 = poly_off[id], p1 = poly_off[id + 1];
    const uint64_t np = p1 - p0;
    if (np == 0) continue;
    auto pt = [&](uint64_t k) { return std::make_pair(poly[2 * (p0 + k)], poly[2 * (p0 + k) + 1]); };
    if (d < anchor_dist) {
      anchor_dist = d;
      anchor = pt(0);
      have_anchor = true;
    }
    std::vector<std::pair<int32_t, int32_t>> s;
    if (d_end <= max_t) {
      for (uint64_t k = 0; k < np; ++k) s.push_back(pt(k));
    } else {
      const float frac = (float)(max_t - d) / (float)w;
      if (frac <= 0.0f) continue;
      if (np == 1) {
        s.push_back(pt(0));
      } else if (frac >= 1.0f) {
        for (uint64_t k = 0; k < np; ++k) s.push_back(pt(k));
      } else {
        const uint64_t nseg = np - 1;
        const float sf = frac * (float)nseg;
        const uint64_t si = std::min<uint64_t>((uint64_t)std::floor(sf), nseg - 1);
        const float lf = sf - (float)si;
        for (uint64_t k = 0; k <= si; ++k) s.push_back(pt(k));
        if (lf > 0.0f && si + 1 < np) {
          const auto a = pt(si), b = pt(si + 1);
          const int32_t lat = a.first + (int32_t)((float)(b.first - a.first) * lf);
          const int32_t lon = a.second + (int32_t)((float)(b.second - a.second) * lf);
          s.emplace_back(lat, lon);
        }
      }
    }
    if (!s.empty()) segs.push_back(std::move(s));
  }
  *n_cells = 0;
  if (segs.empty()) return 0;
  if (has_origin) {
    anchor = {(int32_t)(o_lat * 1e7), (int32_t)(o_lon * 1e7)};
    have_anchor = true;
  }
  const Closed cl = stamp_and_close(segs, cfg, have_anchor ? &anchor : nullptr);
  grid_origin[0] = cl.min_x;
  grid_origin[1] = cl.min_y;
  std::vector<std::pair<int32_t, int32_t>> set;
  for (const auto& kv : cl.map.tiles)
    for (int lr = 0; lr < TILE; ++lr)
      for (int lc = 0; lc < TILE; ++lc)
        if ((kv.second[lr] >> lc) & 1)
          set.emplace_back(ty_of(kv.first) * TILE + lr, tx_of(kv.first) * TILE + lc);
  std::sort(set.begin(), set.end());
  *n_cells = set.size();
  for (uint64_t i = 0; i < set.size() && i < cell_cap; ++i) {
    cells[2 * i] = set[i].second;
    cells[2 * i + 1] = set[i].first;
  }
  return emit(contour_of(cl, cfg), out, cap);
}

}  // extern "C"
