// graph.cu — device layout of a rank-aligned CCH.
//
// Input is the CchTopo + CchWeights pair of the reference
// (route/src/formats/cch_topo.rs:250-284, cch_weights.rs:359). INF weights are
// dropped exactly as UpAdjFlat::build_with / DownAdjFlat::build /
// DownReverseAdjFlat::build_with do (route/src/matrix/bucket_ch.rs:191-418).
//
// Layout built here:
//   * elimination tree of the undirected union of finite edges (Liu's
//     algorithm); every finite edge joins a node and one of its ancestors, so
//     a source's upward search space lies on its ancestor path.
//   * per node: parent, depth, and run_end (last rank of the run r, r+1, ...
//     along which parent(x) == x + 1) so a warp emits a whole run of the
//     ancestor path with one dependent load.
//   * UP records {depth(src) - depth(dst), w}: the upward kernel indexes the
//     ancestor path by depth difference and never needs the target id.
//   * levels of the downward pull DAG (level(v) = 1 + max level of the
//     sources of v's DOWN in-edges) and a slab position per node, ordered by
//     (level, rank), so every level is a contiguous position range.
//   * the pull CSR (DownReverseAdjFlat) re-indexed by slab position.

#include <algorithm>
#include <cstring>
#include <numeric>

#include "engine.cuh"

namespace bf {

namespace {

template <class T>
bf_status dev_upload(T** dptr, const T* src, size_t count, Graph* g) {
  *dptr = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)dptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *dptr = nullptr;
    set_error("cudaMalloc of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    return BF_ERR_OOM;
  }
  g->device_bytes += bytes;
  if (count) BF_CUDA(cudaMemcpy(*dptr, src, count * sizeof(T), cudaMemcpyHostToDevice));
  return BF_OK;
}

}  // namespace

static bf_status build_graph_impl(const bf_cch_csr* csr, const bf_config* cfg, Graph* g,
                                  bool two, const uint32_t* up_len, const uint32_t* down_len);

// The CCH of the transposed graph: UP'(x) = {(y, w) : DOWN edge y -> x},
// DOWN'(y) = {(x, w) : UP edge x -> y}. Distances from t in it are the
// distances to t in the original (the reference's reverse PHAST runs its
// upward phase over DownReverseAdjFlat and pulls over UpAdjFlat,
// route/src/range/phast.rs:879-1001).
//
// Length weights (two-channel graphs) travel with their edges.
bf_status build_graph(const bf_cch_csr* csr, const bf_config* cfg, Graph* g,
                      const uint32_t* up_len, const uint32_t* down_len) {
  const bool two = up_len != nullptr;
  if (!(cfg && (cfg->flags & BF_FLAG_REVERSE)))
    return build_graph_impl(csr, cfg, g, two, up_len, down_len);
  const uint32_t n = csr->n_nodes;
  const uint64_t* uo = csr->up_offsets;
  const uint64_t* dno = csr->down_offsets;
  for (uint32_t u = 0; u < n; ++u)
    if (uo[u + 1] < uo[u] || dno[u + 1] < dno[u]) {
      set_error("CSR offsets must be non-decreasing");
      return BF_ERR_INVALID;
    }
  std::vector<uint64_t> ro(n + 1, 0), rdo(n + 1, 0);
  for (uint32_t y = 0; y < n; ++y)
    for (uint64_t k = dno[y]; k < dno[y + 1]; ++k) {
      const uint32_t x = csr->down_targets[k];
      if (x >= y) {
        set_error("DOWN edge does not go to a lower rank");
        return BF_ERR_INVALID;
      }
      ro[x + 1]++;
    }
  for (uint32_t x = 0; x < n; ++x)
    for (uint64_t k = uo[x]; k < uo[x + 1]; ++k) {
      const uint32_t y = csr->up_targets[k];
      if (y >= n || y <= x) {
        set_error("UP edge does not go to a higher rank");
        return BF_ERR_INVALID;
      }
      rdo[y + 1]++;
    }
  for (uint32_t v = 0; v < n; ++v) {
    ro[v + 1] += ro[v];
    rdo[v + 1] += rdo[v];
  }
  std::vector<uint32_t> rt(ro[n]), rw(ro[n]), rdt(rdo[n]), rdw(rdo[n]);
  std::vector<uint32_t> rl(two ? ro[n] : 0), rdl(two ? rdo[n] : 0);
  {
    std::vector<uint64_t> f(ro.begin(), ro.end() - 1), fd(rdo.begin(), rdo.end() - 1);
    for (uint32_t y = 0; y < n; ++y)
      for (uint64_t k = dno[y]; k < dno[y + 1]; ++k) {
        const uint32_t x = csr->down_targets[k];
        rt[f[x]] = y;
        if (two) rl[f[x]] = down_len[k];
        rw[f[x]++] = csr->down_weights[k];
      }
    for (uint32_t x = 0; x < n; ++x)
      for (uint64_t k = uo[x]; k < uo[x + 1]; ++k) {
        const uint32_t y = csr->up_targets[k];
        rdt[fd[y]] = x;
        if (two) rdl[fd[y]] = up_len[k];
        rdw[fd[y]++] = csr->up_weights[k];
      }
  }
  bf_cch_csr t = *csr;
  t.up_offsets = ro.data();
  t.up_targets = rt.data();
  t.up_weights = rw.data();
  t.down_offsets = rdo.data();
  t.down_targets = rdt.data();
  t.down_weights = rdw.data();
  return build_graph_impl(&t, cfg, g, two, rl.data(), rdl.data());
}

static bf_status build_graph_impl(const bf_cch_csr* csr, const bf_config* cfg, Graph* g,
                                  bool two, const uint32_t* up_len, const uint32_t* down_len) {
  const uint32_t n = csr->n_nodes;
  g->n = n;
  const uint64_t* uo = csr->up_offsets;
  const uint64_t* dno = csr->down_offsets;
  for (uint32_t u = 0; u < n; ++u)
    if (uo[u + 1] < uo[u] || dno[u + 1] < dno[u]) {
      set_error("CSR offsets must be non-decreasing");
      return BF_ERR_INVALID;
    }
  if (two) {
    // the reference indexes its length flats as aligned with the time flats,
    // which holds only when both drop the same INF edges
    for (uint64_t k = 0; k < uo[n]; ++k)
      if ((csr->up_weights[k] == INF) != (up_len[k] == INF)) {
        set_error("UP length weight " + std::to_string(k) +
                  " is INF where the time weight is not (or the reverse)");
        return BF_ERR_INVALID;
      }
    for (uint64_t k = 0; k < dno[n]; ++k)
      if ((csr->down_weights[k] == INF) != (down_len[k] == INF)) {
        set_error("DOWN length weight " + std::to_string(k) +
                  " is INF where the time weight is not (or the reverse)");
        return BF_ERR_INVALID;
      }
  }
  // finite UP / DOWN edges, validated; parallel UP edges (one target listed
  // twice) become one record with the smallest (time, length), which is what
  // relaxing each of them gives - and the upward kernel relies on one record
  // per (source, target)
  std::vector<uint64_t> up_off(n + 1, 0), dn_cnt(n + 1, 0);
  std::vector<uint32_t> last_src(n, NONE);
  for (uint32_t u = 0; u < n; ++u) {
    uint64_t c = 0;
    for (uint64_t k = uo[u]; k < uo[u + 1]; ++k) {
      uint32_t t = csr->up_targets[k];
      if (t >= n || t <= u) {
        set_error("UP edge " + std::to_string(u) + "->" + std::to_string(t) +
                  " does not go to a higher rank");
        return BF_ERR_INVALID;
      }
      if (csr->up_weights[k] != INF && last_src[t] != u) {
        last_src[t] = u;
        ++c;
      }
    }
    up_off[u + 1] = up_off[u] + c;
    for (uint64_t k = dno[u]; k < dno[u + 1]; ++k) {
      uint32_t t = csr->down_targets[k];
      if (t >= u) {
        set_error("DOWN edge " + std::to_string(u) + "->" + std::to_string(t) +
                  " does not go to a lower rank");
        return BF_ERR_INVALID;
      }
      if (csr->down_weights[k] != INF) dn_cnt[t + 1]++;
    }
  }
  g->n_up = up_off[n];
  // in-edges of DOWN (pull layout) by target rank
  std::vector<uint64_t> in_off_r(n + 1, 0);
  for (uint32_t v = 0; v < n; ++v) in_off_r[v + 1] = in_off_r[v] + dn_cnt[v + 1];
  g->n_down = in_off_r[n];
  std::vector<uint32_t> in_src_r(g->n_down), in_w_r(g->n_down), in_l_r(two ? g->n_down : 0);
  {
    std::vector<uint64_t> f(in_off_r.begin(), in_off_r.end() - 1);
    for (uint32_t u = 0; u < n; ++u)
      for (uint64_t k = dno[u]; k < dno[u + 1]; ++k) {
        uint32_t w = csr->down_weights[k];
        if (w == INF) continue;
        uint32_t t = csr->down_targets[k];
        in_src_r[f[t]] = u;
        if (two) in_l_r[f[t]] = down_len[k];
        in_w_r[f[t]++] = w;
      }
  }
  // lower neighbours in the undirected union (for the elimination tree)
  // finite up edges u->v contribute u as a lower neighbour of v; finite down
  // edges r->t contribute t as a lower neighbour of r
  std::vector<uint64_t> low_cnt(n + 1, 0);
  for (uint32_t u = 0; u < n; ++u) {
    for (uint64_t k = uo[u]; k < uo[u + 1]; ++k)
      if (csr->up_weights[k] != INF) low_cnt[csr->up_targets[k] + 1]++;
    for (uint64_t k = dno[u]; k < dno[u + 1]; ++k)
      if (csr->down_weights[k] != INF) low_cnt[u + 1]++;
  }
  for (uint32_t v = 0; v < n; ++v) low_cnt[v + 1] += low_cnt[v];
  std::vector<uint32_t> low(low_cnt[n]);
  {
    std::vector<uint64_t> f(low_cnt.begin(), low_cnt.end() - 1);
    for (uint32_t u = 0; u < n; ++u) {
      for (uint64_t k = uo[u]; k < uo[u + 1]; ++k)
        if (csr->up_weights[k] != INF) low[f[csr->up_targets[k]]++] = u;
      for (uint64_t k = dno[u]; k < dno[u + 1]; ++k)
        if (csr->down_weights[k] != INF) low[f[u]++] = csr->down_targets[k];
    }
  }
  std::vector<uint32_t> parent(n, NONE);
  {
    std::vector<uint32_t> anc(n, NONE);
    for (uint32_t i = 0; i < n; ++i)
      for (uint64_t k = low_cnt[i]; k < low_cnt[i + 1]; ++k) {
        uint32_t j = low[k];
        while (j != NONE && j < i) {
          uint32_t nx = anc[j];
          anc[j] = i;
          if (nx == NONE) parent[j] = i;
          j = nx;
        }
      }
  }
  low.clear();
  low.shrink_to_fit();
  std::vector<uint32_t> depth(n, 0), run_end(n, 0);
  uint32_t maxd = 0;
  for (uint32_t r = n; r-- > 0;) {
    depth[r] = parent[r] == NONE ? 0 : depth[parent[r]] + 1;
    maxd = std::max(maxd, depth[r]);
    run_end[r] = (parent[r] == r + 1) ? run_end[r + 1] : r;
  }
  g->max_depth = maxd;
  // runs of consecutive ranks on the longest (in runs) root path: r's path
  // continues r + 1's run, or starts a run below its parent's path
  {
    std::vector<uint32_t> runs(n, 0);
    uint32_t maxr = 0;
    for (uint32_t r = n; r-- > 0;) {
      if (parent[r] == NONE) runs[r] = 1;
      else if (parent[r] == r + 1) runs[r] = runs[r + 1];
      else runs[r] = runs[parent[r]] + 1;
      maxr = std::max(maxr, runs[r]);
    }
    g->max_runs = maxr;
  }
  // UP records, one per (source, target)
  std::vector<uint2> up_rec(g->n_up);
  std::vector<uint32_t> up_l(two ? g->n_up : 0);
  std::fill(last_src.begin(), last_src.end(), NONE);
  std::vector<uint64_t> rec_at(n, 0);
  for (uint32_t u = 0; u < n; ++u) {
    uint64_t p = up_off[u];
    for (uint64_t k = uo[u]; k < uo[u + 1]; ++k) {
      uint32_t w = csr->up_weights[k];
      if (w == INF) continue;
      uint32_t v = csr->up_targets[k];
      const uint32_t l = two ? up_len[k] : 0;
      if (last_src[v] == u) {  // a parallel edge: keep the smaller (time, length)
        const uint64_t q = rec_at[v];
        if (w < up_rec[q].y || (two && w == up_rec[q].y && l < up_l[q])) {
          up_rec[q].y = w;
          if (two) up_l[q] = l;
        }
        continue;
      }
      last_src[v] = u;
      rec_at[v] = p;
      if (two) up_l[p] = l;
      up_rec[p++] = make_uint2(depth[u] - depth[v], w);
    }
  }
  last_src.clear();
  last_src.shrink_to_fit();
  rec_at.clear();
  rec_at.shrink_to_fit();
  // levels of the pull DAG
  std::vector<uint32_t> level(n, 0);
  uint32_t maxl = 0;
  for (uint32_t v = n; v-- > 0;) {
    uint32_t l = 0;
    for (uint64_t k = in_off_r[v]; k < in_off_r[v + 1]; ++k) l = std::max(l, level[in_src_r[k]] + 1);
    level[v] = l;
    maxl = std::max(maxl, l);
  }
  g->n_levels = n ? maxl + 1 : 0;
  g->lvl_start.assign(g->n_levels + 1, 0);
  for (uint32_t v = 0; v < n; ++v) g->lvl_start[level[v] + 1]++;
  for (uint32_t l = 0; l < g->n_levels; ++l) g->lvl_start[l + 1] += g->lvl_start[l];
  g->pos_of.assign(n, 0);
  std::vector<uint32_t> rank_at(n);
  {
    std::vector<uint32_t> f(g->lvl_start.begin(), g->lvl_start.end() - 1);
    for (uint32_t v = 0; v < n; ++v) {
      uint32_t p = f[level[v]]++;
      g->pos_of[v] = p;
      rank_at[p] = v;
    }
  }
  // pull CSR by position, sources sorted by position
  std::vector<uint64_t> in_off(n + 1, 0);
  for (uint32_t p = 0; p < n; ++p) {
    uint32_t v = rank_at[p];
    in_off[p + 1] = in_off[p] + (in_off_r[v + 1] - in_off_r[v]);
  }
  std::vector<uint2> in_rec(g->n_down);
  std::vector<uint32_t> in_len(two ? g->n_down : 0);
  std::vector<uint64_t> ord;
  for (uint32_t p = 0; p < n; ++p) {
    uint32_t v = rank_at[p];
    const uint64_t k0 = in_off_r[v], k1 = in_off_r[v + 1];
    // sources in ascending position; the sort key carries the edge index so
    // the length weight follows its edge
    ord.clear();
    for (uint64_t k = k0; k < k1; ++k) ord.push_back(((uint64_t)g->pos_of[in_src_r[k]] << 32) | (k - k0));
    std::sort(ord.begin(), ord.end());
    uint64_t q = in_off[p];
    for (uint64_t o : ord) {
      const uint64_t k = k0 + (uint32_t)o;
      if (two) in_len[q] = in_l_r[k];
      in_rec[q++] = make_uint2((uint32_t)(o >> 32), in_w_r[k]);
    }
  }

  // device
  BF_CUDA(cudaSetDevice(g->device));
  BF_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  for (auto& e : g->ev) BF_CUDA(cudaEventCreate(&e));
  bf_status s;
  if ((s = init_ctx(g->ctx))) return s;
  if ((s = dev_upload(&g->d_parent, parent.data(), n, g))) return s;
  if ((s = dev_upload(&g->d_run_end, run_end.data(), n, g))) return s;
  if ((s = dev_upload(&g->d_depth, depth.data(), n, g))) return s;
  if ((s = dev_upload(&g->d_up_off, up_off.data(), n + 1, g))) return s;
  if ((s = dev_upload(&g->d_up_rec, up_rec.data(), up_rec.size(), g))) return s;
  if (two && (s = dev_upload(&g->d_up_len, up_l.data(), up_l.size(), g))) return s;
  if ((s = dev_upload(&g->d_pos_of, g->pos_of.data(), n, g))) return s;
  if ((s = dev_upload(&g->d_rank_at, rank_at.data(), n, g))) return s;
  if ((s = dev_upload(&g->d_in_off, in_off.data(), n + 1, g))) return s;
  if ((s = dev_upload(&g->d_in_rec, in_rec.data(), in_rec.size(), g))) return s;
  if (two && (s = dev_upload(&g->d_in_len, in_len.data(), in_len.size(), g))) return s;
  if ((s = dev_upload(&g->d_lvl_start, g->lvl_start.data(), g->lvl_start.size(), g))) return s;
  uint32_t zero = 0;
  if ((s = dev_upload(&g->d_err, &zero, 1, g))) return s;
  g->rank_at = std::move(rank_at);
  g->h_in_off = std::move(in_off);
  g->h_in_rec = std::move(in_rec);
  g->h_in_len = std::move(in_len);
  g->has_len = two;
  (void)cfg;
  return BF_OK;
}

void free_graph(Graph* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  void* ptrs[] = {g->d_parent, g->d_run_end, g->d_depth, g->d_up_off, g->d_up_rec, g->d_up_len,
                  g->d_pos_of,  g->d_rank_at, g->d_in_off, g->d_in_rec, g->d_in_len,
                  g->d_lvl_start, g->d_bar, g->d_plain_prog, g->d_dist,
                  g->d_seed,    g->d_flag,    g->d_err,    g->d_io,
                  g->d_iso,     g->d_set_pre, g->d_set_out, g->d_set_off};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (g->h_set_stage) cudaFreeHost(g->h_set_stage);
  free_ctx(g->ctx);
  for (auto& e : g->ev)
    if (e) cudaEventDestroy(e);
  if (g->stream) cudaStreamDestroy(g->stream);
}

}  // namespace bf
