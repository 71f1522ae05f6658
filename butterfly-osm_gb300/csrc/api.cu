// api.cu — extern "C" entry points of bf_phast.h.
//
// Every entry point validates its arguments on the host, takes the graph's
// mutex (a graph is shared by host threads the way the reference shares its
// &self engines across rayon workers, batched_phast.rs:45), runs on the
// graph's stream (or the caller's), checks the device error word and returns
// a status; nothing aborts.

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>

#include "engine.cuh"

namespace bf {

static thread_local std::string t_err;

void set_error(const std::string& msg) { t_err = msg; }

bf_status cuda_status(cudaError_t e, const char* what) {
  cudaGetLastError();
  t_err = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return BF_ERR_OOM;
  return BF_ERR_DEVICE;
}

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  bf_status alloc(size_t bytes) {
    if (cudaMalloc(&p, std::max<size_t>(bytes, 4)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      set_error("cudaMalloc of " + std::to_string(bytes) + " bytes failed");
      return BF_ERR_OOM;
    }
    return BF_OK;
  }
  template <class T>
  T* as() {
    return (T*)p;
  }
};

bf_status check_ids(const uint32_t* ids, uint64_t m, uint32_t n, const char* what) {
  for (uint64_t i = 0; i < m; ++i)
    if (ids[i] >= n) {
      set_error(std::string(what) + "[" + std::to_string(i) + "] = " + std::to_string(ids[i]) +
                " is not a node of the graph (n_nodes = " + std::to_string(n) + ")");
      return BF_ERR_INVALID;
    }
  return BF_OK;
}

// Run the selected engine on device buffers.
bf_status run_matrix(Graph* g, const uint32_t* d_src, uint64_t S, const uint32_t* d_tgt,
                     uint64_t T, uint32_t threshold, uint32_t* d_out, cudaStream_t st,
                     bf_stats* stats) {
  bf_status s;
  if (g->engine == BF_ENGINE_PLAIN) {
    DevBuf tpos;
    if ((s = tpos.alloc(T * 4))) return s;
    if ((s = to_positions(g, d_tgt, T, tpos.as<uint32_t>(), st))) return s;
    if ((s = plain_matrix(g, d_src, S, tpos.as<uint32_t>(), T, threshold, d_out, st, stats)))
      return s;
    if (stats) stats->kernel_launches += 1;
  } else {
    if ((s = batched_matrix(g, g->ctx, d_src, S, d_tgt, T, threshold, d_out, st, stats))) return s;
  }
  return check_device_error(g, st);
}

}  // namespace
}  // namespace bf

using namespace bf;

struct bf_graph {
  Graph g;
};

namespace bf {
Graph* graph_of(bf_graph* h) { return &h->g; }
}  // namespace bf

extern "C" {

static bf_status graph_create(const bf_cch_csr* csr, const uint32_t* up_len,
                              const uint32_t* down_len, const bf_config* cfg, bf_graph** out) {
  if (out) *out = nullptr;
  if (!csr || !out || !csr->up_offsets || !csr->down_offsets || csr->n_nodes == 0) {
    set_error("bf_graph_create: null argument or empty graph");
    return BF_ERR_INVALID;
  }
  if ((csr->up_offsets[csr->n_nodes] && (!csr->up_targets || !csr->up_weights)) ||
      (csr->down_offsets[csr->n_nodes] && (!csr->down_targets || !csr->down_weights))) {
    set_error("bf_graph_create: edge arrays missing");
    return BF_ERR_INVALID;
  }
  bf_config c{};
  if (cfg) c = *cfg;
  if (c.engine > BF_ENGINE_BATCHED || (c.flags & ~BF_FLAG_REVERSE) ||
      (c.k_lanes && c.k_lanes != 16 && c.k_lanes != 32 && c.k_lanes != 64 && c.k_lanes != 128)) {
    set_error("bf_graph_create: invalid engine, flags or k_lanes");
    return BF_ERR_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device");
    return BF_ERR_DEVICE;
  }
  if (c.device < 0 || c.device >= ndev) {
    set_error("bf_graph_create: device ordinal out of range");
    return BF_ERR_INVALID;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, c.device) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaGetDeviceProperties failed");
    return BF_ERR_DEVICE;
  }
  const uint64_t l2_bytes = (uint64_t)prop.l2CacheSize;
  if (prop.major != 10 || prop.minor != 3) {
    set_error(std::string("this library is built for sm_103 (GB300); device is ") + prop.name);
    return BF_ERR_DEVICE;
  }
  bf_graph* h = new (std::nothrow) bf_graph();
  if (!h) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  Graph* g = &h->g;
  g->device = c.device;
  g->l2_bytes = l2_bytes;
  g->sm_count = (uint32_t)prop.multiProcessorCount;
  g->engine = c.engine == BF_ENGINE_AUTO ? BF_ENGINE_BATCHED : c.engine;
  g->k_lanes = c.k_lanes;
  if (cudaSetDevice(c.device) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    set_error("cudaSetDevice failed");
    return BF_ERR_DEVICE;
  }
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  g->hbm_budget = c.hbm_budget_bytes ? c.hbm_budget_bytes : (uint64_t)(fr * 0.85);
  bf_status s;
  try {
    s = build_graph(csr, &c, g, up_len, down_len);
    if (s == BF_OK) s = batched_prepare(g, c.subtree_nodes);
    if (s == BF_OK) {
      // load the no-alloc entry point's module and static scratch now, while
      // the caller still expects allocations (a failure here is reported by
      // that entry point's own first call instead)
      uint32_t* na = nullptr;
      if (na_scratch(g->device, &na) != BF_OK) cudaGetLastError();
    }
  } catch (const std::bad_alloc&) {
    set_error("out of host memory");
    s = BF_ERR_OOM;
  }
  if (s != BF_OK) {
    free_graph(g);
    delete h;
    return s;
  }
  *out = h;
  return BF_OK;
}

bf_status bf_graph_create(const bf_cch_csr* csr, const bf_config* cfg, bf_graph** out) {
  return graph_create(csr, nullptr, nullptr, cfg, out);
}

bf_status bf_graph_create_2ch(const bf_cch_csr* csr, const uint32_t* up_len_weights,
                              const uint32_t* down_len_weights, const bf_config* cfg,
                              bf_graph** out) {
  if (out) *out = nullptr;
  if (csr && csr->up_offsets && csr->down_offsets && csr->n_nodes &&
      ((csr->up_offsets[csr->n_nodes] && !up_len_weights) ||
       (csr->down_offsets[csr->n_nodes] && !down_len_weights))) {
    set_error("bf_graph_create_2ch: length weights missing");
    return BF_ERR_INVALID;
  }
  // an edgeless direction still marks the graph as two-channel
  static const uint32_t none = 0;
  return graph_create(csr, up_len_weights ? up_len_weights : &none,
                      down_len_weights ? down_len_weights : &none, cfg, out);
}

void bf_graph_destroy(bf_graph* h) {
  if (!h) return;
  free_graph(&h->g);
  delete h;
}

bf_status bf_graph_info_get(const bf_graph* h, bf_graph_info* o) {
  if (!h || !o) {
    set_error("bf_graph_info_get: null argument");
    return BF_ERR_INVALID;
  }
  const Graph& g = h->g;
  std::memset(o, 0, sizeof(*o));
  o->n_nodes = g.n;
  o->n_levels = g.n_levels;
  o->n_up = g.n_up;
  o->n_down = g.n_down;
  o->max_depth = g.max_depth;
  o->k_lanes = g.k_lanes;
  o->device_bytes = g.device_bytes;
  return BF_OK;
}

bf_status bf_graph_set_engine(bf_graph* h, uint32_t engine, uint32_t k_lanes) {
  if (!h || engine > BF_ENGINE_BATCHED ||
      (k_lanes && k_lanes != 16 && k_lanes != 32 && k_lanes != 64 && k_lanes != 128)) {
    set_error("bf_graph_set_engine: invalid argument");
    return BF_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(h->g.mu);
  h->g.engine = engine == BF_ENGINE_AUTO ? BF_ENGINE_BATCHED : engine;
  if (k_lanes) h->g.k_lanes = k_lanes;
  return BF_OK;
}

bf_status bf_matrix_device(bf_graph* h, const uint32_t* d_src, uint64_t S, const uint32_t* d_tgt,
                           uint64_t T, uint32_t threshold, uint32_t* d_out, void* stream,
                           bf_stats* st) {
  if (!h || (S && !d_src) || (T && !d_tgt) || (S && T && !d_out)) {
    set_error("bf_matrix_device: null argument");
    return BF_ERR_INVALID;
  }
  double t0 = now_s();
  Graph* g = &h->g;
  std::lock_guard<std::mutex> lk(g->mu);
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
  if (st) std::memset(st, 0, sizeof(*st));
  bf_status rc = BF_OK;
  if (S && T) rc = run_matrix(g, d_src, S, d_tgt, T, threshold, d_out, s, st);
  if (rc == BF_OK && cudaStreamSynchronize(s) != cudaSuccess)
    rc = cuda_status(cudaGetLastError(), "cudaStreamSynchronize");
  if (st) {
    st->n_sources = S;
    st->n_targets = T;
    st->total_ms = (now_s() - t0) * 1e3;
  }
  return rc;
}

static bf_tune to_c(const Tune& t) {
  bf_tune o{};
  o.threads_per_block = t.tpb;
  o.edges_per_item = t.split;
  o.graph_capture = t.graphs;
  o.lanes_per_wave = t.max_lanes;
  o.isochrone_lanes = t.iso_lanes;
  o.small_level_rows = t.small_rows;
  o.small_level_edges = t.small_split;
  o.overlap_levels = t.pdl;
  o.isochrone_16bit = t.iso_half;
  o.overlap_upward = t.overlap_up;
  o.mapped_output = t.mapped_out;
  o.hub_l2_mb = t.hub_mb;
  o.device_schedule = t.dev_sched;
  o.persistent_sweep = t.persist;
  o.staged_levels = t.staged;
  return o;
}

bf_status bf_set_tune(bf_graph* h, const bf_tune* t) {
  if (!h || !t || (t->threads_per_block != 32 && t->threads_per_block != 64 &&
                   t->threads_per_block != 128 && t->threads_per_block != 256) ||
      t->edges_per_item == 0 || t->edges_per_item > 1024 ||
      (t->lanes_per_wave && t->lanes_per_wave % 32) ||
      (t->isochrone_lanes && t->isochrone_lanes % 32) ||
      (t->small_level_rows && (t->small_level_edges == 0 || t->small_level_edges > 1024))) {
    set_error("bf_set_tune: invalid tunables");
    return BF_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(h->g.mu);
  h->g.tune.tpb = t->threads_per_block;
  h->g.tune.split = t->edges_per_item;
  h->g.tune.graphs = t->graph_capture ? 1 : 0;
  h->g.tune.max_lanes = t->lanes_per_wave;
  h->g.tune.iso_lanes = t->isochrone_lanes;
  h->g.tune.small_rows = t->small_level_rows;
  h->g.tune.small_split = t->small_level_rows ? t->small_level_edges : 8;
  h->g.tune.pdl = t->overlap_levels ? 1 : 0;
  h->g.tune.iso_half = t->isochrone_16bit ? 1 : 0;
  h->g.tune.overlap_up = t->overlap_upward ? 1 : 0;
  h->g.tune.mapped_out = t->mapped_output ? 1 : 0;
  h->g.tune.hub_mb = std::min<uint32_t>(t->hub_l2_mb, 1024);
  h->g.tune.dev_sched = t->device_schedule ? 1 : 0;
  h->g.tune.persist = t->persistent_sweep & 3u;
  h->g.tune.staged = t->staged_levels ? 1 : 0;
  return BF_OK;
}

bf_status bf_get_tune(const bf_graph* h, bf_tune* t) {
  if (!h || !t) {
    set_error("bf_get_tune: null argument");
    return BF_ERR_INVALID;
  }
  *t = to_c(h->g.tune);
  return BF_OK;
}

bf_status bf_autotune(bf_graph* h, const uint32_t* d_src, uint64_t S, const uint32_t* d_tgt,
                      uint64_t T, uint32_t reps, bf_tune* best) {
  if (!h || !d_src || !d_tgt || !S || !T || !best) {
    set_error("bf_autotune: null argument or empty sample");
    return BF_ERR_INVALID;
  }
  Graph* g = &h->g;
  std::lock_guard<std::mutex> lk(g->mu);
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  if (reps == 0) reps = 2;
  cudaStream_t s = g->stream;
  DevBuf out;
  bf_status rc;
  if ((rc = out.alloc(S * T * 4))) return rc;
  const Tune saved = g->tune;
  std::vector<Tune> cands;
  std::vector<uint32_t> lane_opts = {0};
  if (S >= 256) lane_opts.push_back((uint32_t)(((S / 2) + 31) & ~31ull));
  for (uint32_t tpb : {64u, 128u, 256u})
    for (uint32_t split : {8u, 16u, 32u})
      for (uint32_t lanes : lane_opts) {
        Tune t;
        t.tpb = tpb;
        t.split = split;
        t.graphs = 1;
        t.max_lanes = lanes;
        t.iso_lanes = saved.iso_lanes;
        cands.push_back(t);
      }
  double best_ms = 1e300;
  Tune best_t = saved;
  for (const Tune& t : cands) {
    g->tune = t;
    double sum = 0;
    for (uint32_t r = 0; r <= reps; ++r) {
      bf_stats st{};
      rc = batched_matrix(g, g->ctx, d_src, S, d_tgt, T, BF_INF, out.as<uint32_t>(), s, &st);
      if (rc == BF_OK) rc = check_device_error(g, s);
      if (rc != BF_OK) {
        g->tune = saved;
        return rc;
      }
      if (r) sum += st.upward_ms + st.downward_ms + st.extract_ms;
    }
    const double ms = sum / reps;
    if (ms < best_ms) {
      best_ms = ms;
      best_t = t;
    }
  }
  // second stage: short work items on the small top levels, on the winner
  uint32_t tried = (uint32_t)cands.size();
  for (uint32_t rows : {0u, 1024u}) {
    Tune t = best_t;
    t.small_rows = rows;
    t.small_split = 8;
    g->tune = t;
    double sum = 0;
    for (uint32_t r = 0; r <= reps; ++r) {
      bf_stats st{};
      rc = batched_matrix(g, g->ctx, d_src, S, d_tgt, T, BF_INF, out.as<uint32_t>(), s, &st);
      if (rc == BF_OK) rc = check_device_error(g, s);
      if (rc != BF_OK) {
        g->tune = saved;
        return rc;
      }
      if (r) sum += st.upward_ms + st.downward_ms + st.extract_ms;
    }
    ++tried;
    if (sum / reps < best_ms) {
      best_ms = sum / reps;
      best_t = t;
    }
  }
  g->tune = best_t;
  *best = to_c(best_t);
  best->step_ms = best_ms;
  best->tried = tried;
  return BF_OK;
}

bf_status bf_schedule_levels(const bf_graph* h, uint32_t cap, uint64_t* items, uint64_t* edges,
                             uint64_t* rows, uint32_t* n_levels) {
  if (!h || !n_levels || (cap && (!items || !edges || !rows))) {
    set_error("bf_schedule_levels: null argument");
    return BF_ERR_INVALID;
  }
  const Sched& sc = h->g.ctx.sc;
  if (!sc.valid || sc.lvl_item.size() < 2 || sc.lvl_row.size() != sc.lvl_item.size() ||
      sc.lvl_edge.size() != sc.lvl_item.size()) {
    set_error("bf_schedule_levels: no target-restricted schedule built yet");
    return BF_ERR_INVALID;
  }
  const uint32_t L = (uint32_t)sc.lvl_item.size() - 1;
  *n_levels = L;
  for (uint32_t l = 0; l < std::min(cap, L); ++l) {
    items[l] = sc.lvl_item[l + 1] - sc.lvl_item[l];
    edges[l] = sc.lvl_edge[l + 1] - sc.lvl_edge[l];
    rows[l] = sc.lvl_row[l + 1] - sc.lvl_row[l];
  }
  return BF_OK;
}

bf_status bf_autotune_isochrones(bf_graph* h, const uint32_t* d_orig, const uint32_t* d_thr,
                                 uint64_t n, uint32_t reps, bf_tune* best) {
  if (!h || !d_orig || !d_thr || !n || !best) {
    set_error("bf_autotune_isochrones: null argument or empty sample");
    return BF_ERR_INVALID;
  }
  Graph* g = &h->g;
  std::lock_guard<std::mutex> lk(g->mu);
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  if (reps == 0) reps = 2;
  cudaStream_t s = g->stream;
  const uint64_t w64 = (g->n + 63) / 64;
  DevBuf bits, counts;
  bf_status rc;
  if ((rc = bits.alloc(n * w64 * 8)) || (rc = counts.alloc(n * 8))) return rc;
  const Tune saved = g->tune;
  // wave widths (origins per wave) and the persistent form of the waves
  std::vector<Tune> cands;
  for (uint32_t lanes : {256u, 512u, 1024u, 2048u})
    for (uint32_t pers : {0u, 2u}) {
      if (lanes > ((n + 31) & ~31ull) && lanes != 256u) continue;  // wider than the sample
      Tune t = saved;
      t.iso_lanes = lanes;
      t.persist = (saved.persist & 1u) | pers;
      cands.push_back(t);
    }
  double best_ms = 1e300;
  Tune best_t = saved;
  for (const Tune& t : cands) {
    g->tune = t;
    double sum = 0;
    for (uint32_t r = 0; r <= reps; ++r) {
      bf_stats st{};
      BF_CUDA(cudaEventRecord(g->ev[4], s));
      rc = isochrone_bitsets(g, g->ctx, d_orig, d_thr, n, bits.as<uint64_t>(),
                             counts.as<uint64_t>(), s, nullptr);
      if (rc == BF_OK) rc = check_device_error(g, s);
      if (rc != BF_OK) {
        g->tune = saved;
        return rc;
      }
      BF_CUDA(cudaEventRecord(g->ev[5], s));
      BF_CUDA(cudaEventSynchronize(g->ev[5]));
      float ms = 0;
      BF_CUDA(cudaEventElapsedTime(&ms, g->ev[4], g->ev[5]));
      if (r) sum += ms;
    }
    if (sum / reps < best_ms) {
      best_ms = sum / reps;
      best_t = t;
    }
  }
  g->tune = best_t;
  *best = to_c(best_t);
  best->step_ms = best_ms;
  best->tried = (uint32_t)cands.size();
  return BF_OK;
}

// A tune cache file: one JSON object with the graph's fingerprint and the
// tunables. The fingerprint is the graph's counts and an FNV-1a hash of its
// level sizes, so a cache is applied only to the graph it was measured on.
namespace {

uint64_t graph_fingerprint(const Graph* g) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](uint64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (v >> (8 * i)) & 0xFF;
      h *= 1099511628211ull;
    }
  };
  mix(g->n);
  mix(g->n_up);
  mix(g->n_down);
  mix(g->n_levels);
  mix(g->max_depth);
  for (uint32_t v : g->lvl_start) mix(v);
  return h;
}

const char* const TUNE_KEYS[] = {"threads_per_block", "edges_per_item", "graph_capture",
                                 "lanes_per_wave",    "isochrone_lanes", "small_level_rows",
                                 "small_level_edges", "overlap_levels",  "isochrone_16bit",
                                 "overlap_upward",    "mapped_output",   "hub_l2_mb",
                                 "device_schedule",   "persistent_sweep", "staged_levels"};

void tune_fields(bf_tune& t, uint32_t* f[15]) {
  uint32_t* p[15] = {&t.threads_per_block, &t.edges_per_item, &t.graph_capture,
                     &t.lanes_per_wave,    &t.isochrone_lanes, &t.small_level_rows,
                     &t.small_level_edges, &t.overlap_levels,  &t.isochrone_16bit,
                     &t.overlap_upward,    &t.mapped_output,   &t.hub_l2_mb,
                     &t.device_schedule,   &t.persistent_sweep, &t.staged_levels};
  for (int i = 0; i < 15; ++i) f[i] = p[i];
}

}  // namespace

bf_status bf_tune_save(const bf_graph* h, const char* path) {
  if (!h || !path) {
    set_error("bf_tune_save: null argument");
    return BF_ERR_INVALID;
  }
  bf_tune t = to_c(h->g.tune);
  uint32_t* f[15];
  tune_fields(t, f);
  std::string js = "{\"graph\": \"" + std::to_string(graph_fingerprint(&h->g)) + "\"";
  for (int i = 0; i < 15; ++i) js += ", \"" + std::string(TUNE_KEYS[i]) + "\": " + std::to_string(*f[i]);
  js += "}\n";
  FILE* fp = std::fopen(path, "w");
  if (!fp) {
    set_error(std::string("bf_tune_save: cannot write ") + path);
    return BF_ERR_INVALID;
  }
  const bool ok = std::fwrite(js.data(), 1, js.size(), fp) == js.size();
  if (std::fclose(fp) != 0 || !ok) {
    set_error(std::string("bf_tune_save: write to ") + path + " failed");
    return BF_ERR_INVALID;
  }
  return BF_OK;
}

bf_status bf_tune_load(bf_graph* h, const char* path) {
  if (!h || !path) {
    set_error("bf_tune_load: null argument");
    return BF_ERR_INVALID;
  }
  FILE* fp = std::fopen(path, "r");
  if (!fp) {
    set_error(std::string("bf_tune_load: cannot read ") + path);
    return BF_ERR_INVALID;
  }
  std::string js;
  char buf[512];
  for (size_t k; (k = std::fread(buf, 1, sizeof(buf), fp)) > 0;) js.append(buf, k);
  std::fclose(fp);
  auto value_of = [&js](const std::string& key, std::string* out) {
    const std::string pat = "\"" + key + "\":";
    const size_t at = js.find(pat);
    if (at == std::string::npos) return false;
    size_t i = at + pat.size();
    while (i < js.size() && (js[i] == ' ' || js[i] == '"')) ++i;
    size_t j = i;
    while (j < js.size() && js[j] >= '0' && js[j] <= '9') ++j;
    if (j == i) return false;
    *out = js.substr(i, j - i);
    return true;
  };
  std::string v;
  if (!value_of("graph", &v) || v != std::to_string(graph_fingerprint(&h->g))) {
    set_error(std::string("bf_tune_load: ") + path + " holds no tunables for this graph");
    return BF_ERR_INVALID;
  }
  bf_tune t{};
  {
    std::lock_guard<std::mutex> lk(h->g.mu);
    t = to_c(h->g.tune);
  }
  uint32_t* f[15];
  tune_fields(t, f);
  for (int i = 0; i < 15; ++i) {
    if (!value_of(TUNE_KEYS[i], &v) || v.size() > 10) {
      set_error(std::string("bf_tune_load: ") + path + " lacks " + TUNE_KEYS[i]);
      return BF_ERR_INVALID;
    }
    const unsigned long long x = std::stoull(v);
    if (x > 0xFFFFFFFFull) {
      set_error(std::string("bf_tune_load: ") + TUNE_KEYS[i] + " out of range");
      return BF_ERR_INVALID;
    }
    *f[i] = (uint32_t)x;
  }
  return bf_set_tune(h, &t);
}

bf_status bf_matrix(bf_graph* h, const uint32_t* src, uint64_t S, const uint32_t* tgt, uint64_t T,
                    uint32_t threshold, uint32_t* out, bf_stats* st) {
  if (!h || (S && !src) || (T && !tgt) || (S && T && !out)) {
    set_error("bf_matrix: null argument");
    return BF_ERR_INVALID;
  }
  double t0 = now_s();
  Graph* g = &h->g;
  bf_status rc;
  if ((rc = check_ids(src, S, g->n, "sources"))) return rc;
  if ((rc = check_ids(tgt, T, g->n, "targets"))) return rc;
  std::lock_guard<std::mutex> lk(g->mu);
  if (st) std::memset(st, 0, sizeof(*st));
  if (!S || !T) return BF_OK;
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = g->stream;
  // A page-locked output buffer is written by the extraction kernel directly
  // (over the CPU-GPU link), which saves the device copy and the separate
  // device-to-host transfer; any other buffer gets the copy.
  uint32_t* d_direct = nullptr;
  {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, out) == cudaSuccess) {
      if (pa.type == cudaMemoryTypeHost && pa.devicePointer && g->tune.mapped_out)
        d_direct = static_cast<uint32_t*>(pa.devicePointer);
    } else {
      cudaGetLastError();
    }
  }
  // graph-owned I/O buffer: [sources | targets | matrix], grown on demand
  const size_t need = (S + T + (d_direct ? 0 : S * T)) * 4;
  if (need > g->io_bytes) {
    if (g->d_io) {
      cudaFree(g->d_io);
      g->device_bytes -= g->io_bytes;
      g->d_io = nullptr;
      g->io_bytes = 0;
    }
    if (cudaMalloc(&g->d_io, need) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc of " + std::to_string(need) + " bytes for matrix I/O failed");
      return BF_ERR_OOM;
    }
    g->io_bytes = need;
    g->device_bytes += need;
  }
  uint32_t* d_src = g->d_io;
  uint32_t* d_tgt = d_src + S;
  uint32_t* d_out = d_direct ? d_direct : d_tgt + T;
  BF_CUDA(cudaMemcpyAsync(d_src, src, S * 4, cudaMemcpyHostToDevice, s));
  BF_CUDA(cudaMemcpyAsync(d_tgt, tgt, T * 4, cudaMemcpyHostToDevice, s));
  if ((rc = run_matrix(g, d_src, S, d_tgt, T, threshold, d_out, s, st))) return rc;
  if (!d_direct) BF_CUDA(cudaMemcpyAsync(out, d_out, S * T * 4, cudaMemcpyDeviceToHost, s));
  BF_CUDA(cudaStreamSynchronize(s));
  if (st) {
    st->n_sources = S;
    st->n_targets = T;
    st->h2d_bytes = (S + T) * 4;
    st->d2h_bytes = S * T * 4;
    st->total_ms = (now_s() - t0) * 1e3;
  }
  return BF_OK;
}

bf_status bf_query_batch(bf_graph* h, const uint32_t* src, uint32_t k, uint32_t threshold,
                         uint32_t* dist_out) {
  if (!h || (k && (!src || !dist_out)) || k > 128) {
    set_error("bf_query_batch: null argument or k > 128");
    return BF_ERR_INVALID;
  }
  Graph* g = &h->g;
  bf_status rc;
  if ((rc = check_ids(src, k, g->n, "sources"))) return rc;
  if (!k) return BF_OK;
  std::lock_guard<std::mutex> lk(g->mu);
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = g->stream;
  DevBuf ds, dout;
  if ((rc = ds.alloc(k * 4)) || (rc = dout.alloc((size_t)k * g->n * 4))) return rc;
  BF_CUDA(cudaMemcpyAsync(ds.p, src, k * 4, cudaMemcpyHostToDevice, s));
  // every rank is a target: positions are the rank -> position table itself
  if ((rc = plain_matrix(g, ds.as<uint32_t>(), k, g->d_pos_of, g->n, threshold,
                         dout.as<uint32_t>(), s, nullptr)))
    return rc;
  if ((rc = check_device_error(g, s))) return rc;
  BF_CUDA(cudaMemcpyAsync(dist_out, dout.p, (size_t)k * g->n * 4, cudaMemcpyDeviceToHost, s));
  BF_CUDA(cudaStreamSynchronize(s));
  return BF_OK;
}

bf_status bf_query_batch_noalloc(bf_graph* h, const uint32_t* d_src, uint32_t k,
                                 uint32_t threshold, uint32_t* d_out, void* stream) {
  if (!h || (k && (!d_src || !d_out))) {
    set_error("bf_query_batch_noalloc: null argument");
    return BF_ERR_INVALID;
  }
  Graph* g = &h->g;
  std::lock_guard<std::mutex> lk(g->mu);
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
  bf_status rc = query_batch_noalloc(g, d_src, k, threshold, d_out, s);
  if (rc != BF_OK) return rc;
  return check_device_error(g, s);
}

bf_status bf_phast_query(bf_graph* h, uint32_t origin, uint32_t* dist_out) {
  return bf_query_batch(h, &origin, 1, BF_INF, dist_out);
}

static bf_status check_seedsets(const bf_seed* seeds, const uint64_t* off, uint64_t m,
                                uint32_t n, const char* what) {
  if (!off || off[0] != 0) {
    set_error(std::string(what) + " offsets must start at 0");
    return BF_ERR_INVALID;
  }
  for (uint64_t i = 0; i < m; ++i)
    if (off[i + 1] < off[i]) {
      set_error(std::string(what) + " offsets must be non-decreasing");
      return BF_ERR_INVALID;
    }
  if (off[m] && !seeds) {
    set_error(std::string(what) + " seeds missing");
    return BF_ERR_INVALID;
  }
  for (uint64_t k = 0; k < off[m]; ++k)
    if (seeds[k].rank >= n) {
      set_error(std::string(what) + " seed rank " + std::to_string(seeds[k].rank) +
                " is not a node of the graph");
      return BF_ERR_INVALID;
    }
  return BF_OK;
}

bf_status bf_matrix_seeded(bf_graph* h, const bf_seed* src_seeds, const uint64_t* src_off,
                           uint64_t S, const bf_seed* tgt_seeds, const uint64_t* tgt_off,
                           uint64_t T, uint32_t threshold, uint32_t* out, uint64_t* conflicts,
                           uint64_t conflict_cap, uint64_t* n_conflicts, bf_stats* st) {
  if (!h || (S && T && !out) || (conflict_cap && !conflicts)) {
    set_error("bf_matrix_seeded: null argument");
    return BF_ERR_INVALID;
  }
  double t0 = now_s();
  Graph* g = &h->g;
  bf_status rc;
  if ((rc = check_seedsets(src_seeds, src_off, S, g->n, "source")) ||
      (rc = check_seedsets(tgt_seeds, tgt_off, T, g->n, "target")))
    return rc;
  std::lock_guard<std::mutex> lk(g->mu);
  if (st) std::memset(st, 0, sizeof(*st));
  if (n_conflicts) *n_conflicts = 0;
  if (!S || !T) return BF_OK;
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  rc = matrix_seeded(g, g->ctx, src_seeds, src_off, S, tgt_seeds, tgt_off, T, threshold, out, conflicts,
                     conflict_cap, n_conflicts, st);
  if (st) {
    st->n_sources = S;
    st->n_targets = T;
    st->total_ms = (now_s() - t0) * 1e3;
  }
  return rc;
}

bf_status bf_phast_bounded_seeded(bf_graph* h, const bf_seed* seeds, uint32_t n_seeds,
                                  uint32_t threshold, uint32_t* out_rank, uint32_t* out_dist,
                                  uint64_t cap, uint64_t* n_out) {
  if (!h || (n_seeds && !seeds) || (cap && (!out_rank || !out_dist))) {
    set_error("bf_phast_bounded_seeded: null argument");
    return BF_ERR_INVALID;
  }
  Graph* g = &h->g;
  for (uint32_t i = 0; i < n_seeds; ++i)
    if (seeds[i].rank >= g->n) {
      set_error("bf_phast_bounded_seeded: seed rank " + std::to_string(seeds[i].rank) +
                " is not a node of the graph");
      return BF_ERR_INVALID;
    }
  std::lock_guard<std::mutex> lk(g->mu);
  if (n_out) *n_out = 0;
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  return bounded_seeded(g, g->ctx, seeds, n_seeds, threshold, out_rank, out_dist, cap, n_out);
}

static bf_status check_seedsets2(const bf_seed2* seeds, const uint64_t* off, uint64_t m,
                                 uint32_t n, const char* what) {
  if (!off || off[0] != 0) {
    set_error(std::string(what) + " offsets must start at 0");
    return BF_ERR_INVALID;
  }
  for (uint64_t i = 0; i < m; ++i)
    if (off[i + 1] < off[i]) {
      set_error(std::string(what) + " offsets must be non-decreasing");
      return BF_ERR_INVALID;
    }
  if (off[m] && !seeds) {
    set_error(std::string(what) + " seeds missing");
    return BF_ERR_INVALID;
  }
  for (uint64_t k = 0; k < off[m]; ++k)
    if (seeds[k].rank >= n) {
      set_error(std::string(what) + " seed rank " + std::to_string(seeds[k].rank) +
                " is not a node of the graph");
      return BF_ERR_INVALID;
    }
  return BF_OK;
}

bf_status bf_matrix_seeded_2ch(bf_graph* h, const bf_seed2* src_seeds, const uint64_t* src_off,
                               uint64_t S, const bf_seed2* tgt_seeds, const uint64_t* tgt_off,
                               uint64_t T, uint32_t threshold, uint32_t* out_time,
                               uint32_t* out_len, uint64_t* conflicts, uint64_t conflict_cap,
                               uint64_t* n_conflicts, bf_stats* st) {
  if (!h || (S && T && (!out_time || !out_len)) || (conflict_cap && !conflicts)) {
    set_error("bf_matrix_seeded_2ch: null argument");
    return BF_ERR_INVALID;
  }
  double t0 = now_s();
  Graph* g = &h->g;
  if (!g->has_len) {
    set_error("bf_matrix_seeded_2ch: the graph has no length weights (use bf_graph_create_2ch)");
    return BF_ERR_UNSUPPORTED;
  }
  bf_status rc;
  if ((rc = check_seedsets2(src_seeds, src_off, S, g->n, "source")) ||
      (rc = check_seedsets2(tgt_seeds, tgt_off, T, g->n, "target")))
    return rc;
  std::lock_guard<std::mutex> lk(g->mu);
  if (st) std::memset(st, 0, sizeof(*st));
  if (n_conflicts) *n_conflicts = 0;
  if (!S || !T) return BF_OK;
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  try {
    rc = matrix_seeded_2ch(g, g->ctx, src_seeds, src_off, S, tgt_seeds, tgt_off, T, threshold,
                           out_time, out_len, conflicts, conflict_cap, n_conflicts, st);
  } catch (const std::bad_alloc&) {
    set_error("out of host memory");
    rc = BF_ERR_OOM;
  }
  if (st) {
    st->n_sources = S;
    st->n_targets = T;
    st->total_ms = (now_s() - t0) * 1e3;
  }
  return rc;
}

bf_status bf_phast_bounded_seeded_2ch(bf_graph* h, const bf_seed2* seeds, uint32_t n_seeds,
                                      uint32_t threshold, uint32_t* out_rank, uint32_t* out_time,
                                      uint32_t* out_len, uint64_t cap, uint64_t* n_out) {
  if (!h || (n_seeds && !seeds) || (cap && (!out_rank || !out_time || !out_len))) {
    set_error("bf_phast_bounded_seeded_2ch: null argument");
    return BF_ERR_INVALID;
  }
  Graph* g = &h->g;
  if (!g->has_len) {
    set_error("bf_phast_bounded_seeded_2ch: the graph has no length weights");
    return BF_ERR_UNSUPPORTED;
  }
  for (uint32_t i = 0; i < n_seeds; ++i)
    if (seeds[i].rank >= g->n) {
      set_error("bf_phast_bounded_seeded_2ch: seed rank " + std::to_string(seeds[i].rank) +
                " is not a node of the graph");
      return BF_ERR_INVALID;
    }
  std::lock_guard<std::mutex> lk(g->mu);
  if (n_out) *n_out = 0;
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  try {
    return bounded_seeded_2ch(g, g->ctx, seeds, n_seeds, threshold, out_rank, out_time, out_len,
                              cap, n_out);
  } catch (const std::bad_alloc&) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
}

// update_cost_ewma (bucket_ch.rs:6663-6671): the first sample is taken as is,
// later ones move the estimate by a quarter; never below 1.
void bf_router_observe(bf_router* r, uint32_t which, uint64_t sample_ns) {
  if (!r || which > BF_COST_SCAN) return;
  uint64_t* cell = which == BF_COST_SWEEP ? &r->sweep_ns : &r->scan_ns;
  uint64_t prev = __atomic_load_n(cell, __ATOMIC_RELAXED);
  for (;;) {
    uint64_t next = prev == 0 ? sample_ns : prev - prev / 4 + sample_ns / 4;
    if (next < 1) next = 1;
    if (__atomic_compare_exchange_n(cell, &prev, next, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
      return;
  }
}

// The GPU computes every source's field in one call: its per-source share of
// the call is the scan cost the router compares against bucket sweeps.
void bf_router_observe_stats(bf_router* r, const bf_stats* st) {
  if (!r || !st || st->n_sources == 0 || !(st->total_ms > 0)) return;
  const double ns = st->total_ms * 1e6 / (double)st->n_sources;
  bf_router_observe(r, BF_COST_SCAN, ns < 1.0 ? 1 : (uint64_t)ns);
}

// phast_wins (bucket_ch.rs:6677-6712).
int bf_router_phast_wins(const bf_router* r, uint64_t n_sources, uint64_t n_targets,
                         uint64_t n_nodes, uint32_t force) {
  if (force == BF_ROUTE_BUCKET) return 0;
  if (force == BF_ROUTE_PHAST) return n_sources <= n_targets;
  if (n_sources > n_targets) return 0;
  const uint64_t sweep = r ? __atomic_load_n(&r->sweep_ns, __ATOMIC_RELAXED) : 0;
  const uint64_t scan = r ? __atomic_load_n(&r->scan_ns, __ATOMIC_RELAXED) : 0;
  unsigned __int128 scan_cost, sweep_cost;
  if (sweep > 0 && scan > 0) {
    scan_cost = scan;
    sweep_cost = sweep;
  } else {
    scan_cost = n_nodes;
    sweep_cost = std::min<uint64_t>(std::max<uint64_t>(n_nodes / 400, 500), 20000);
  }
  const unsigned __int128 phast = (unsigned __int128)n_sources * scan_cost;
  const unsigned __int128 bucket = (unsigned __int128)(n_sources + n_targets) * sweep_cost;
  return phast < bucket ? 1 : 0;
}

bf_status bf_isochrone_bitsets_device(bf_graph* h, const uint32_t* d_orig, const uint32_t* d_thr,
                                      uint64_t n, uint64_t* d_bits, uint64_t* d_counts,
                                      void* stream, bf_stats* st) {
  if (!h || (n && (!d_orig || !d_thr || !d_bits || !d_counts))) {
    set_error("bf_isochrone_bitsets_device: null argument");
    return BF_ERR_INVALID;
  }
  double t0 = now_s();
  Graph* g = &h->g;
  std::lock_guard<std::mutex> lk(g->mu);
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
  if (st) std::memset(st, 0, sizeof(*st));
  bf_status rc = BF_OK;
  if (n) rc = isochrone_bitsets(g, g->ctx, d_orig, d_thr, n, d_bits, d_counts, s, st);
  if (rc == BF_OK) rc = check_device_error(g, s);
  if (st) {
    st->n_sources = n;
    st->n_targets = g->n;
    st->total_ms = (now_s() - t0) * 1e3;
  }
  return rc;
}

bf_status bf_isochrone_bitsets(bf_graph* h, const uint32_t* orig, const uint32_t* thr, uint64_t n,
                               uint64_t* bits, uint64_t* counts, bf_stats* st) {
  if (!h || (n && (!orig || !thr || !bits))) {
    set_error("bf_isochrone_bitsets: null argument");
    return BF_ERR_INVALID;
  }
  double t0 = now_s();
  Graph* g = &h->g;
  bf_status rc;
  if ((rc = check_ids(orig, n, g->n, "origins"))) return rc;
  if (st) std::memset(st, 0, sizeof(*st));
  if (!n) return BF_OK;
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = g->stream;
  const uint64_t w64 = (g->n + 63) / 64;
  // origins per chunk: bitset rows of at most ~8 GB on the device
  uint64_t chunk = std::max<uint64_t>(32, (8ull << 30) / (w64 * 8));
  chunk = std::min<uint64_t>(chunk, n);
  const size_t need = chunk * (4 + 4 + 8) + chunk * w64 * 8;
  if (need > g->iso_bytes) {
    if (g->d_iso) {
      cudaFree(g->d_iso);
      g->device_bytes -= g->iso_bytes;
      g->d_iso = nullptr;
      g->iso_bytes = 0;
    }
    if (cudaMalloc(&g->d_iso, need) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc of " + std::to_string(need) + " bytes for isochrone I/O failed");
      return BF_ERR_OOM;
    }
    g->iso_bytes = need;
    g->device_bytes += need;
  }
  uint64_t* d_bits = reinterpret_cast<uint64_t*>(g->d_iso);
  uint64_t* d_counts = d_bits + chunk * w64;
  uint32_t* d_orig = reinterpret_cast<uint32_t*>(d_counts + chunk);
  uint32_t* d_thr = d_orig + chunk;
  std::vector<uint64_t> tmp_counts;
  for (uint64_t c0 = 0; c0 < n; c0 += chunk) {
    const uint64_t m = std::min<uint64_t>(chunk, n - c0);
    BF_CUDA(cudaMemcpyAsync(d_orig, orig + c0, m * 4, cudaMemcpyHostToDevice, s));
    BF_CUDA(cudaMemcpyAsync(d_thr, thr + c0, m * 4, cudaMemcpyHostToDevice, s));
    if ((rc = isochrone_bitsets(g, g->ctx, d_orig, d_thr, m, d_bits, d_counts, s, st))) return rc;
    BF_CUDA(cudaMemcpyAsync(bits + c0 * w64, d_bits, m * w64 * 8, cudaMemcpyDeviceToHost, s));
    if (counts)
      BF_CUDA(cudaMemcpyAsync(counts + c0, d_counts, m * 8, cudaMemcpyDeviceToHost, s));
    BF_CUDA(cudaStreamSynchronize(s));
  }
  if ((rc = check_device_error(g, s))) return rc;
  if (st) {
    st->n_sources = n;
    st->n_targets = g->n;
    st->h2d_bytes = n * 8;
    st->d2h_bytes = n * w64 * 8 + (counts ? n * 8 : 0);
    st->total_ms = (now_s() - t0) * 1e3;
  }
  return BF_OK;
}

}  // extern "C"

namespace bf {

bf_status settled_waves(Graph* g, const uint32_t* orig, const uint32_t* thr, uint64_t n,
                        SettledSink& sink, bf_stats* st) {
  bf_status rc;
  if ((rc = check_ids(orig, n, g->n, "origins"))) return rc;
  if (st) std::memset(st, 0, sizeof(*st));
  if (cudaSetDevice(g->device) != cudaSuccess) return cuda_status(cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = g->stream;
  const uint64_t w64 = (g->n + 63) / 64;
  uint64_t chunk = std::max<uint64_t>(32, (8ull << 30) / (w64 * 8));
  chunk = std::min<uint64_t>(chunk, std::max<uint64_t>(n, 1));
  const size_t need = chunk * (4 + 4 + 8) + chunk * w64 * 8;
  if (need > g->iso_bytes) {
    if (g->d_iso) {
      cudaFree(g->d_iso);
      g->device_bytes -= g->iso_bytes;
      g->d_iso = nullptr;
      g->iso_bytes = 0;
    }
    if (cudaMalloc(&g->d_iso, need) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc of " + std::to_string(need) + " bytes for isochrone I/O failed");
      return BF_ERR_OOM;
    }
    g->iso_bytes = need;
    g->device_bytes += need;
  }
  uint64_t* d_bits = reinterpret_cast<uint64_t*>(g->d_iso);
  uint64_t* d_counts = d_bits + chunk * w64;
  uint32_t* d_orig = reinterpret_cast<uint32_t*>(d_counts + chunk);
  uint32_t* d_thr = d_orig + chunk;
  for (uint64_t c0 = 0; c0 < n; c0 += chunk) {
    const uint64_t m = std::min<uint64_t>(chunk, n - c0);
    sink.base = c0;
    BF_CUDA(cudaMemcpyAsync(d_orig, orig + c0, m * 4, cudaMemcpyHostToDevice, s));
    BF_CUDA(cudaMemcpyAsync(d_thr, thr + c0, m * 4, cudaMemcpyHostToDevice, s));
    try {
      if ((rc = isochrone_bitsets(g, g->ctx, d_orig, d_thr, m, d_bits, d_counts, s, st, &sink)))
        return rc;
    } catch (const std::bad_alloc&) {
      set_error("out of host memory");
      return BF_ERR_OOM;
    }
  }
  return check_device_error(g, s);
}

}  // namespace bf

extern "C" {

bf_status bf_isochrone_settled(bf_graph* h, const uint32_t* orig, const uint32_t* thr, uint64_t n,
                               uint64_t* offsets, uint32_t** ranks, uint32_t** dists,
                               bf_stats* st) {
  if (ranks) *ranks = nullptr;
  if (dists) *dists = nullptr;
  if (!h || !offsets || !ranks || !dists || (n && (!orig || !thr))) {
    set_error("bf_isochrone_settled: null argument");
    return BF_ERR_INVALID;
  }
  double t0 = now_s();
  Graph* g = &h->g;
  bf_status rc;
  std::lock_guard<std::mutex> lk(g->mu);  // the staging is the graph's until the copy ends
  SettledSink sink;
  try {
    sink.r_at.assign(n, 0);
    sink.d_at.assign(n, 0);
    sink.cnt.assign(n, 0);
  } catch (const std::bad_alloc&) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  if ((rc = settled_waves(g, orig, thr, n, sink, st))) return rc;
  offsets[0] = 0;
  for (uint64_t i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + sink.cnt[i];
  const uint64_t total = offsets[n];
  uint32_t* r = (uint32_t*)std::malloc(std::max<uint64_t>(total, 1) * 4);
  uint32_t* d = (uint32_t*)std::malloc(std::max<uint64_t>(total, 1) * 4);
  if (!r || !d) {
    std::free(r);
    std::free(d);
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  // staging (wave order) -> output (input order), in pieces of 256 Ki entries
  const uint64_t piece = 1ull << 18;
  const uint32_t* stage = g->h_set_stage;
  parallel_for((total + piece - 1) / piece, [&](uint64_t p) {
    uint64_t a = p * piece;
    const uint64_t e = std::min(total, a + piece);
    uint64_t i = (uint64_t)(std::upper_bound(offsets, offsets + n + 1, a) - offsets) - 1;
    for (; a < e; ++i) {
      const uint64_t b = std::min(e, offsets[i + 1]);
      const uint64_t k = a - offsets[i];
      std::memcpy(r + a, stage + sink.r_at[i] + k, (b - a) * 4);
      std::memcpy(d + a, stage + sink.d_at[i] + k, (b - a) * 4);
      a = b;
    }
  });
  *ranks = r;
  *dists = d;
  if (st) {
    st->n_sources = n;
    st->n_targets = g->n;
    st->h2d_bytes = n * 8;
    st->d2h_bytes = total * 8;
    st->total_ms = (now_s() - t0) * 1e3;
  }
  return BF_OK;
}

void bf_settled_free(uint32_t* p) { std::free(p); }

const char* bf_last_error(void) { return t_err.c_str(); }

}  // extern "C"
