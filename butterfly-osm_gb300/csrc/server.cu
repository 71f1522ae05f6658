// server.cu — device-resident serving loop with continuous batching.
//
// The reference serves matrices and isochrones from request handlers that
// run one engine call per request on a CPU pool (do_matrix with 1000-source
// tiles, route/src/server/flight.rs:589,957-1110; isochrone_bulk_handler,
// route/src/server/isochrone_handler.rs:1535-1750). Here requests are queued
// and two worker slots, each with its own stream, distance slab and
// schedule (a Ctx), form batches continuously: whenever a slot is free it
// takes the waiting requests of one kind (in arrival order, up to the slot's
// lane budget and max_inflight), so requests that arrive while the other slot
// computes are admitted as soon as that slot frees, and the two slots' work
// overlaps on the device.
//
//   matrix batch     the sources of all admitted requests are the lanes of
//                    one sweep restricted to the union of their targets; each
//                    request's rows and columns are then extracted into its
//                    own output with its own threshold (exact: the shared
//                    sweep is unbounded).
//   isochrone batch  the origins are the lanes of one gated full-graph sweep
//                    (bf_isochrone_bitsets semantics).
//
// Every device wait is bounded by timeout_ms (polling an event); a request
// whose wait runs out completes with BF_ERR_TIMEOUT.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>

#include "engine.cuh"

namespace bf {

namespace {

double wall_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct Job {
  uint64_t ticket = 0;
  bf_request r{};
  std::vector<uint32_t> src, tgt;  // copies of the request's ids
  double submit_s = 0, admit_s = 0;
  bool cancelled = false;
};

struct Slot {
  Ctx ctx;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  uint8_t* d_buf = nullptr;  // per-batch device I/O
  size_t buf_bytes = 0;
  std::thread th;
};

}  // namespace

struct Server {
  Graph* g = nullptr;
  bf_server_cfg cfg{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::unordered_map<uint64_t, Job*> inflight;
  std::vector<bf_completion> done;
  uint64_t next_ticket = 1;
  bool stop = false;
  Slot slot[2];
};

namespace {

bf_status grow(Graph* g, Slot& sl, size_t need) {
  if (need <= sl.buf_bytes) return BF_OK;
  if (sl.d_buf) {
    cudaFree(sl.d_buf);
    g->device_bytes -= sl.buf_bytes;
    sl.d_buf = nullptr;
    sl.buf_bytes = 0;
  }
  if (cudaMalloc(&sl.d_buf, need) != cudaSuccess) {
    cudaGetLastError();
    set_error("serving slot: cudaMalloc of " + std::to_string(need) + " bytes failed");
    return BF_ERR_OOM;
  }
  sl.buf_bytes = need;
  g->device_bytes += need;
  return BF_OK;
}

// Wait for the slot's stream with a deadline (no unbounded device wait).
bf_status wait_slot(Slot& sl, uint32_t timeout_ms) {
  BF_CUDA(cudaEventRecord(sl.done, sl.stream));
  const double deadline = wall_s() + timeout_ms * 1e-3;
  for (;;) {
    cudaError_t e = cudaEventQuery(sl.done);
    if (e == cudaSuccess) return BF_OK;
    if (e != cudaErrorNotReady) return cuda_status(e, "cudaEventQuery");
    if (wall_s() > deadline) {
      set_error("serving slot: device work exceeded timeout_ms");
      return BF_ERR_TIMEOUT;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

void complete(Server* sv, Job* j, int status) {
  bf_completion c{};
  c.user_tag = j->r.user_tag;
  c.ticket = j->ticket;
  c.status = j->cancelled ? BF_ERR_CANCELLED : status;
  c.submit_s = j->submit_s;
  c.admit_s = j->admit_s;
  c.done_s = wall_s();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->inflight.erase(j->ticket);
    sv->done.push_back(c);
  }
  sv->cv_done.notify_all();
  delete j;
}

__global__ void k_gather(const uint32_t* __restrict__ table, const uint32_t* __restrict__ idx,
                         uint64_t m, uint32_t* __restrict__ out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = table[idx[i]];
}

bf_status run_matrix_batch(Server* sv, Slot& sl, std::vector<Job*>& jobs) {
  Graph* g = sv->g;
  cudaStream_t st = sl.stream;
  Ctx& c = sl.ctx;
  bf_status s;
  uint64_t L = 0, TT = 0, OUT = 0;
  std::vector<uint64_t> lane_off, t_off, o_off;
  for (Job* j : jobs) {
    lane_off.push_back(L);
    t_off.push_back(TT);
    o_off.push_back(OUT);
    L += j->src.size();
    TT += j->tgt.size();
    OUT += j->src.size() * j->tgt.size();
  }
  std::vector<uint32_t> hs, ht;
  hs.reserve(L);
  ht.reserve(TT);
  for (Job* j : jobs) {
    hs.insert(hs.end(), j->src.begin(), j->src.end());
    ht.insert(ht.end(), j->tgt.begin(), j->tgt.end());
  }
  std::vector<uint32_t> uni(ht);
  std::sort(uni.begin(), uni.end());
  uni.erase(std::unique(uni.begin(), uni.end()), uni.end());
  if ((s = grow(g, sl, (L + 2 * TT + OUT) * 4 + 64))) return s;
  uint32_t* d_src = reinterpret_cast<uint32_t*>(sl.d_buf);
  uint32_t* d_tgt = d_src + L;
  uint32_t* d_trow = d_tgt + TT;
  uint32_t* d_out = d_trow + TT;
  BF_CUDA(cudaMemcpyAsync(d_src, hs.data(), L * 4, cudaMemcpyHostToDevice, st));
  BF_CUDA(cudaMemcpyAsync(d_tgt, ht.data(), TT * 4, cudaMemcpyHostToDevice, st));
  if ((s = build_schedule(g, c, c.sc, uni.data(), uni.size(), false, st))) return s;
  if (TT) k_gather<<<(unsigned)((TT + 255) / 256), 256, 0, st>>>(c.sc.d_cidx, d_tgt, TT, d_trow);
  BF_CUDA(cudaGetLastError());
  if (L == 0) return wait_slot(sl, sv->cfg.timeout_ms);
  const uint64_t rows = std::max<uint32_t>(c.sc.n_r, 1);
  uint64_t max_lanes = ctx_budget(g, c) / (rows * 4);
  max_lanes = max_lanes >= 32 ? max_lanes & ~31ull : 0;
  if (!max_lanes) {
    set_error("serving slot budget too small for one 32-lane wave");
    return BF_ERR_OOM;
  }
  const uint64_t wave = std::min<uint64_t>(max_lanes, (L + 3) & ~3ull);
  const uint32_t Kp = (uint32_t)((wave + 3) & ~3ull);
  if ((s = ensure_slab(g, c, (size_t)rows * Kp * 4))) return s;
  uint64_t launches = 0;
  for (uint64_t w0 = 0; w0 < L; w0 += wave) {
    const uint64_t kw = std::min<uint64_t>(wave, L - w0);
    if ((s = batched_wave(g, c, d_src + w0, kw, Kp, st, &launches, false))) return s;
    for (size_t i = 0; i < jobs.size(); ++i) {
      const uint64_t a = std::max(lane_off[i], w0);
      const uint64_t b = std::min(lane_off[i] + jobs[i]->src.size(), w0 + kw);
      if (a >= b || jobs[i]->tgt.empty()) continue;
      const uint64_t T = jobs[i]->tgt.size();
      launch_extract_lanes(c.d_slab + (a - w0), Kp, d_trow + t_off[i], T, (uint32_t)(b - a),
                           jobs[i]->r.threshold, d_out + o_off[i] + (a - lane_off[i]) * T, st);
    }
    BF_CUDA(cudaGetLastError());
  }
  for (size_t i = 0; i < jobs.size(); ++i) {
    const uint64_t cells = jobs[i]->src.size() * jobs[i]->tgt.size();
    if (cells)
      BF_CUDA(cudaMemcpyAsync(jobs[i]->r.out, d_out + o_off[i], cells * 4, cudaMemcpyDeviceToHost,
                              st));
  }
  return wait_slot(sl, sv->cfg.timeout_ms);
}

bf_status run_iso_batch(Server* sv, Slot& sl, std::vector<Job*>& jobs) {
  Graph* g = sv->g;
  cudaStream_t st = sl.stream;
  bf_status s;
  const uint64_t n = jobs.size(), w64 = (g->n + 63) / 64;
  if ((s = grow(g, sl, n * (8 + 8 + w64 * 8) + 64))) return s;
  uint64_t* d_bits = reinterpret_cast<uint64_t*>(sl.d_buf);
  uint64_t* d_counts = d_bits + n * w64;
  uint32_t* d_o = reinterpret_cast<uint32_t*>(d_counts + n);
  uint32_t* d_t = d_o + n;
  std::vector<uint32_t> ho(2 * n);
  for (uint64_t i = 0; i < n; ++i) {
    ho[i] = jobs[i]->src[0];
    ho[n + i] = jobs[i]->r.threshold;
  }
  BF_CUDA(cudaMemcpyAsync(d_o, ho.data(), 2 * n * 4, cudaMemcpyHostToDevice, st));
  if ((s = isochrone_bitsets(g, sl.ctx, d_o, d_t, n, d_bits, d_counts, st, nullptr))) return s;
  for (uint64_t i = 0; i < n; ++i)
    BF_CUDA(cudaMemcpyAsync(jobs[i]->r.out, d_bits + i * w64, w64 * 8, cudaMemcpyDeviceToHost,
                            st));
  return wait_slot(sl, sv->cfg.timeout_ms);
}

void worker(Server* sv, int si) {
  Slot& sl = sv->slot[si];
  cudaSetDevice(sv->g->device);
  const uint64_t lane_cap[3] = {0, 16384, 4096};
  for (;;) {
    std::vector<Job*> batch;
    uint32_t kind = 0;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] { return sv->stop || !sv->queue.empty(); });
      if (sv->stop) return;
      kind = sv->queue.front()->r.kind;
      uint64_t lanes = 0;
      const double now = wall_s();
      for (auto it = sv->queue.begin(); it != sv->queue.end() && batch.size() < sv->cfg.max_inflight;) {
        Job* j = *it;
        if (j->r.kind != kind) {
          ++it;
          continue;
        }
        const uint64_t add = kind == BF_REQ_MATRIX ? j->src.size() : 1;
        if (!batch.empty() && lanes + add > lane_cap[kind]) break;
        batch.push_back(j);
        lanes += add;
        it = sv->queue.erase(it);
        j->admit_s = now;
        sv->inflight[j->ticket] = j;
      }
    }
    bf_status rc = kind == BF_REQ_MATRIX ? run_matrix_batch(sv, sl, batch)
                                         : run_iso_batch(sv, sl, batch);
    // a device-side error of the batch (a grid barrier that ran out, an
    // inconsistent id) fails its requests
    if (rc == BF_OK) rc = check_device_error(sv->g, sl.stream);
    if (rc != BF_OK && rc != BF_ERR_TIMEOUT) cudaStreamSynchronize(sl.stream);
    if (rc == BF_ERR_TIMEOUT) {
      // the jobs complete with TIMEOUT now; the slot is reused only after its
      // stream drained (the kernels themselves always terminate)
      for (Job* j : batch) complete(sv, j, rc);
      cudaStreamSynchronize(sl.stream);
      continue;
    }
    for (Job* j : batch) complete(sv, j, rc);
  }
}

}  // namespace

}  // namespace bf

using namespace bf;

struct bf_server {
  Server s;
};

extern "C" {

bf_status bf_server_create(bf_graph* gh, const bf_server_cfg* cfg, bf_server** out) {
  if (out) *out = nullptr;
  if (!gh || !out) {
    set_error("bf_server_create: null argument");
    return BF_ERR_INVALID;
  }
  Graph* g = graph_of(gh);
  bf_server* h = new (std::nothrow) bf_server();
  if (!h) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  Server* sv = &h->s;
  sv->g = g;
  if (cfg) sv->cfg = *cfg;
  if (!sv->cfg.max_inflight) sv->cfg.max_inflight = 64;
  if (!sv->cfg.max_queue) sv->cfg.max_queue = 4096;
  if (!sv->cfg.timeout_ms) sv->cfg.timeout_ms = 10000;
  if (cudaSetDevice(g->device) != cudaSuccess) {
    delete h;
    return cuda_status(cudaGetLastError(), "cudaSetDevice");
  }
  uint64_t budget = sv->cfg.hbm_budget_bytes;
  if (!budget) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    budget = (uint64_t)(fr * 0.8);
  }
  for (Slot& sl : sv->slot) {
    sl.ctx.budget = budget / 2;
    bf_status rc = init_ctx(sl.ctx);
    if (rc == BF_OK && (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
                        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess))
      rc = cuda_status(cudaGetLastError(), "stream/event create");
    // the full-graph schedule isochrone batches sweep is built here, once per
    // slot, so that no request waits for it
    if (rc == BF_OK) {
      try {
        rc = build_schedule(g, sl.ctx, sl.ctx.full, nullptr, 0, true, sl.stream);
      } catch (const std::bad_alloc&) {
        set_error("out of host memory");
        rc = BF_ERR_OOM;
      }
    }
    if (rc != BF_OK) {
      bf_server_destroy(h);
      return rc;
    }
  }
  for (int i = 0; i < 2; ++i) sv->slot[i].th = std::thread(worker, sv, i);
  *out = h;
  return BF_OK;
}

bf_status bf_server_submit(bf_server* h, const bf_request* req, uint64_t* ticket) {
  if (!h || !req || !ticket) {
    set_error("bf_server_submit: null argument");
    return BF_ERR_INVALID;
  }
  Server* sv = &h->s;
  const uint32_t n = sv->g->n;
  if (req->kind != BF_REQ_MATRIX && req->kind != BF_REQ_ISOCHRONE) {
    set_error("bf_server_submit: unknown request kind");
    return BF_ERR_INVALID;
  }
  const bool iso = req->kind == BF_REQ_ISOCHRONE;
  if ((iso && req->n_sources != 1) || (req->n_sources && !req->sources) ||
      (!iso && req->n_targets && !req->targets) ||
      (!req->out && (iso || req->n_sources * req->n_targets))) {
    set_error("bf_server_submit: malformed request");
    return BF_ERR_INVALID;
  }
  Job* j = new (std::nothrow) Job();
  if (!j) {
    set_error("out of host memory");
    return BF_ERR_OOM;
  }
  j->r = *req;
  j->src.assign(req->sources, req->sources + req->n_sources);
  if (!iso) j->tgt.assign(req->targets, req->targets + req->n_targets);
  for (uint32_t x : j->src)
    if (x >= n) {
      delete j;
      set_error("bf_server_submit: source id out of range");
      return BF_ERR_INVALID;
    }
  for (uint32_t x : j->tgt)
    if (x >= n) {
      delete j;
      set_error("bf_server_submit: target id out of range");
      return BF_ERR_INVALID;
    }
  j->submit_s = wall_s();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->queue.size() >= sv->cfg.max_queue) {
      delete j;
      set_error("bf_server_submit: queue full");
      return BF_ERR_BUSY;
    }
    j->ticket = sv->next_ticket++;
    *ticket = j->ticket;
    sv->queue.push_back(j);
  }
  sv->cv_work.notify_one();
  return BF_OK;
}

bf_status bf_server_poll(bf_server* h, bf_completion* out, uint32_t cap, uint32_t wait_ms,
                         uint32_t* n_out) {
  if (!h || !n_out || (cap && !out)) {
    set_error("bf_server_poll: null argument");
    return BF_ERR_INVALID;
  }
  Server* sv = &h->s;
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !sv->done.empty(); });
  const uint32_t m = (uint32_t)std::min<size_t>(cap, sv->done.size());
  for (uint32_t i = 0; i < m; ++i) out[i] = sv->done[i];
  sv->done.erase(sv->done.begin(), sv->done.begin() + m);
  *n_out = m;
  return BF_OK;
}

bf_status bf_server_cancel(bf_server* h, uint64_t ticket) {
  if (!h) {
    set_error("bf_server_cancel: null argument");
    return BF_ERR_INVALID;
  }
  Server* sv = &h->s;
  Job* queued = nullptr;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it)
      if ((*it)->ticket == ticket) {
        queued = *it;
        sv->queue.erase(it);
        break;
      }
    if (!queued) {
      auto f = sv->inflight.find(ticket);
      if (f == sv->inflight.end()) {
        set_error("bf_server_cancel: unknown or completed ticket");
        return BF_ERR_INVALID;
      }
      f->second->cancelled = true;  // its result is discarded on completion
      return BF_OK;
    }
    sv->inflight[ticket] = queued;
  }
  queued->cancelled = true;
  complete(sv, queued, BF_ERR_CANCELLED);
  return BF_OK;
}

void bf_server_destroy(bf_server* h) {
  if (!h) return;
  Server* sv = &h->s;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (Slot& sl : sv->slot)
    if (sl.th.joinable()) sl.th.join();
  cudaSetDevice(sv->g->device);
  for (Job* j : sv->queue) delete j;
  for (Slot& sl : sv->slot) {
    free_ctx(sl.ctx);
    if (sl.d_buf) {
      cudaFree(sl.d_buf);
      sv->g->device_bytes -= sl.buf_bytes;
    }
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  delete h;
}

}  // extern "C"
