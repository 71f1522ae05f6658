// CPU oracle of the matrix tile emission (test infrastructure: only the
// tests, the smoke check and the bench's CPU-baseline leg load it).
//
// Restates build_matrix_batch and build_matrix_tile_batch
// (route/src/server/flight.rs:432-500 and :509-589), which turn a row-major
// block of durations into the four UInt32 columns of a matrix RecordBatch
// (source_idx, target_idx, duration_ms, distance_m):
//   * cells are visited row-major (flight.rs:450-451, :526-527);
//   * a cell is pruned when the source's sorted radius list does not contain
//     the destination's original index (binary_search, :452-456, :528-532);
//   * a pruned cell reads u32::MAX, otherwise the matrix value, set to
//     u32::MAX above the time bound (:459, :534-539; build_matrix_batch has no
//     bound, i.e. threshold u32::MAX);
//   * sparse output drops cells whose duration is u32::MAX (:465, :542);
//   * duration_ms = d.saturating_mul(1000), distance_m = the lat matrix's cell
//     or u32::MAX; both u32::MAX for a sentinel cell (:470-483, :548-566).
#include <cstdint>

namespace {

constexpr uint32_t MAX = 0xFFFFFFFFu;

bool contains(const uint32_t* a, uint64_t n, uint32_t v) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t m = lo + (hi - lo) / 2;
    if (a[m] < v)
      lo = m + 1;
    else if (a[m] > v)
      hi = m;
    else
      return true;
  }
  return false;
}

}  // namespace

extern "C" {

// Returns the number of rows written, or UINT64_MAX when a source's original
// index has no radius list (the reference indexes neighbor_mask[orig_src]).
uint64_t orc_tile_emit(const uint32_t* m, const uint32_t* lat, uint32_t n_src, uint32_t n_dst,
                       const uint32_t* src_orig, const uint32_t* dst_orig, uint32_t threshold,
                       const uint64_t* mask_off, const uint32_t* mask, uint32_t n_mask_src,
                       int sparse, uint32_t* s_out, uint32_t* t_out, uint32_t* dur_out,
                       uint32_t* dist_out) {
  uint64_t k = 0;
  for (uint32_t si = 0; si < n_src; ++si) {
    const uint32_t os = src_orig[si];
    if (mask_off && os >= n_mask_src) return UINT64_MAX;
    for (uint32_t di = 0; di < n_dst; ++di) {
      const uint32_t od = dst_orig[di];
      const uint64_t cell = (uint64_t)si * n_dst + di;
      const bool pruned =
          mask_off && !contains(mask + mask_off[os], mask_off[os + 1] - mask_off[os], od);
      uint32_t d = MAX;
      if (!pruned) {
        d = m[cell];
        if (d > threshold) d = MAX;
      }
      if (sparse && d == MAX) continue;
      s_out[k] = os;
      t_out[k] = od;
      if (d == MAX) {
        dur_out[k] = MAX;
        dist_out[k] = MAX;
      } else {
        const uint64_t ms = (uint64_t)d * 1000u;
        dur_out[k] = ms > MAX ? MAX : (uint32_t)ms;
        dist_out[k] = lat ? lat[cell] : MAX;
      }
      ++k;
    }
  }
  return k;
}

}  // extern "C"
