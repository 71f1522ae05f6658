// server.cu — device-resident serving loop with continuous batching.
//
// The reference serves matrices and isochrones from request handlers that
// run one engine call per request on a CPU pool (do_matrix with 1000-source
// tiles, route/src/server/flight.rs:589,957-1110; isochrone_bulk_handler,
// route/src/server/isochrone_handler.rs:1535-1750). Here requests are queued
// and worker slots (four by default), each with its own stream, distance
// slab and schedule (a Ctx), form batches continuously: whenever a slot is
// free it takes the waiting requests of one kind (in arrival order, up to the
// slot's lane cap and max_inflight, and while their device I/O fits the
// budget and the device's free memory), so requests that arrive while other
// slots compute are admitted as soon as a slot frees, and the slots' work
// overlaps on the device: a sweep is a chain of ~1100 dependent levels, most
// of them far too small to fill the GPU, so concurrent sweeps share it.
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
  uint64_t io_bytes = 0;           // device I/O of the request in a batch
};

constexpr int MAX_SLOTS = 8;
// free device memory a batch leaves untouched (other users of the device,
// schedule growth, the slab's own reallocation)
constexpr uint64_t FREE_MARGIN = 1ull << 30;

struct Slot {
  Ctx ctx;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  uint8_t* d_buf = nullptr;  // per-batch device I/O
  size_t buf_bytes = 0;
  double batch_start_s = 0;  // host clock when the current batch began
  void* h_stage = nullptr;   // page-locked staging of results bound for pageable buffers
  size_t stage_bytes = 0;
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
  int n_slots = 4;
  Ctx shared;                   // holds the full-graph schedule every slot sweeps
  uint64_t budget = 0;          // device bytes for request I/O and slabs
  uint64_t io_budget = 0;       // the part of it request I/O may take
  uint64_t admitted_io = 0;     // I/O bytes of the batches in flight
  Slot slot[MAX_SLOTS];
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

// Wait for the slot's stream with a deadline: the batch's device work may
// take timeout_ms from the batch's start (no unbounded device wait).
bf_status wait_slot(Slot& sl, uint32_t timeout_ms) {
  BF_CUDA(cudaEventRecord(sl.done, sl.stream));
  const double deadline = sl.batch_start_s + timeout_ms * 1e-3;
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
  // Results go straight into page-locked caller buffers; pageable ones are
  // staged in the slot's page-locked buffer and copied on the host after the
  // bounded wait (a copy into pageable memory would block this thread until
  // the device finished, defeating the bound, and nothing may write a
  // caller's buffer after its request completed with BF_ERR_TIMEOUT).
  std::vector<std::pair<size_t, uint64_t>> staged;  // (job, offset in the staging buffer)
  uint64_t stage_need = 0;
  for (size_t i = 0; i < jobs.size(); ++i) {
    const uint64_t cells = jobs[i]->src.size() * jobs[i]->tgt.size();
    if (!cells) continue;
    cudaPointerAttributes pa{};
    const bool pinned = cudaPointerGetAttributes(&pa, jobs[i]->r.out) == cudaSuccess &&
                        pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    if (pinned) {
      BF_CUDA(cudaMemcpyAsync(jobs[i]->r.out, d_out + o_off[i], cells * 4, cudaMemcpyDeviceToHost,
                              st));
    } else {
      staged.emplace_back(i, stage_need);
      stage_need += cells * 4;
    }
  }
  if (stage_need > sl.stage_bytes) {
    if (sl.h_stage) cudaFreeHost(sl.h_stage);
    sl.h_stage = nullptr;
    sl.stage_bytes = 0;
    BF_CUDA(cudaHostAlloc(&sl.h_stage, stage_need, cudaHostAllocDefault));
    sl.stage_bytes = stage_need;
  }
  for (auto& [i, off] : staged)
    BF_CUDA(cudaMemcpyAsync(static_cast<uint8_t*>(sl.h_stage) + off, d_out + o_off[i],
                            jobs[i]->src.size() * jobs[i]->tgt.size() * 4, cudaMemcpyDeviceToHost,
                            st));
  if ((s = wait_slot(sl, sv->cfg.timeout_ms))) return s;
  for (auto& [i, off] : staged)
    std::memcpy(jobs[i]->r.out, static_cast<uint8_t*>(sl.h_stage) + off,
                jobs[i]->src.size() * jobs[i]->tgt.size() * 4);
  return BF_OK;
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

// Device bytes a slot's batch of these requests needs for its I/O buffers
// (the d_buf layout of run_matrix_batch / run_iso_batch).
uint64_t io_bytes_of(const Job* j, uint64_t n) {
  if (j->r.kind == BF_REQ_ISOCHRONE) return 16 + 8 + ((n + 63) / 64) * 8;
  return (j->src.size() + 2 * j->tgt.size() + j->src.size() * j->tgt.size()) * 4;
}

void worker(Server* sv, int si) {
  Slot& sl = sv->slot[si];
  cudaSetDevice(sv->g->device);
  // lanes per batch: a matrix batch sweeps the union of its requests'
  // targets for all their sources, so its work grows with (sources) x (rows
  // reaching the union); the cap keeps batching from outgrowing what it saves
  // (one sweep's fixed cost of ~1100 dependent levels per batch)
  const uint64_t lane_cap[3] = {0, 4096, 4096};
  for (;;) {
    std::vector<Job*> batch;
    uint32_t kind = 0;
    uint64_t io = 0;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] { return sv->stop || !sv->queue.empty(); });
      if (sv->stop) return;
      kind = sv->queue.front()->r.kind;
      uint64_t lanes = 0;
      // admission: the batch's I/O must fit what the budget leaves beside the
      // batches in flight and, with a margin, the device's free memory now
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        fr = 0;
      }
      const uint64_t room_budget =
          sv->io_budget > sv->admitted_io ? sv->io_budget - sv->admitted_io : 0;
      const uint64_t room_free = fr > FREE_MARGIN ? fr - FREE_MARGIN : 0;
      const uint64_t room = std::min(room_budget, room_free + sl.buf_bytes);
      const double now = wall_s();
      for (auto it = sv->queue.begin(); it != sv->queue.end() && batch.size() < sv->cfg.max_inflight;) {
        Job* j = *it;
        if (j->r.kind != kind) {
          ++it;
          continue;
        }
        const uint64_t add = kind == BF_REQ_MATRIX ? j->src.size() : 1;
        if (!batch.empty() && lanes + add > lane_cap[kind]) break;
        if (io + j->io_bytes > room) break;  // waits for memory (arrival order kept)
        batch.push_back(j);
        lanes += add;
        io += j->io_bytes;
        it = sv->queue.erase(it);
        j->admit_s = now;
        sv->inflight[j->ticket] = j;
      }
      if (batch.empty()) {
        // nothing fits now: wait for a batch in flight to complete and free
        // memory (or, if none is in flight, for the device's memory to free)
        sv->cv_work.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
      sv->admitted_io += io;
    }
    sl.batch_start_s = wall_s();
    bf_status rc = kind == BF_REQ_MATRIX ? run_matrix_batch(sv, sl, batch)
                                         : run_iso_batch(sv, sl, batch);
    // a device-side error of the batch (a grid barrier that ran out, an
    // inconsistent id) fails its requests
    if (rc == BF_OK) rc = check_device_error(sv->g, sl.stream);
    if (rc != BF_OK && rc != BF_ERR_TIMEOUT) cudaStreamSynchronize(sl.stream);
    if (rc == BF_ERR_TIMEOUT) {
      // the jobs complete with TIMEOUT once the slot's stream has drained
      // (the kernels always terminate): no copy may still be writing into a
      // caller's buffer after its completion is reported
      cudaStreamSynchronize(sl.stream);
      for (Job* j : batch) complete(sv, j, rc);
    } else {
      for (Job* j : batch) complete(sv, j, rc);
    }
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->admitted_io -= io;
    }
    sv->cv_work.notify_all();  // memory freed: waiting slots may admit now
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
  sv->n_slots = sv->cfg.slots ? (int)std::min<uint32_t>(sv->cfg.slots, MAX_SLOTS) : 4;
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
  // half of the budget for request I/O, half for the slots' distance slabs
  sv->budget = budget;
  sv->io_budget = budget / 2;
  // the full-graph schedule that isochrone batches sweep is built here, once
  // for all slots (it is read-only while sweeping), so no request waits for it
  bf_status rc0 = init_ctx(sv->shared);
  if (rc0 == BF_OK) {
    try {
      rc0 = build_schedule(g, sv->shared, sv->shared.full, nullptr, 0, true, g->stream);
    } catch (const std::bad_alloc&) {
      set_error("out of host memory");
      rc0 = BF_ERR_OOM;
    }
  }
  if (rc0 != BF_OK) {
    bf_server_destroy(h);
    return rc0;
  }
  for (int i = 0; i < sv->n_slots; ++i) {
    Slot& sl = sv->slot[i];
    sl.ctx.budget = budget / 2 / sv->n_slots;
    sl.ctx.shared_full = &sv->shared.full;
    bf_status rc = init_ctx(sl.ctx);
    if (rc == BF_OK && (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
                        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess))
      rc = cuda_status(cudaGetLastError(), "stream/event create");
    if (rc != BF_OK) {
      bf_server_destroy(h);
      return rc;
    }
  }
  for (int i = 0; i < sv->n_slots; ++i) sv->slot[i].th = std::thread(worker, sv, i);
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
  j->io_bytes = io_bytes_of(j, n);
  if (j->io_bytes > sv->io_budget) {
    const uint64_t need = j->io_bytes;
    delete j;
    set_error("bf_server_submit: the request's " + std::to_string(need) +
              " bytes of device I/O exceed the server's budget for request I/O (" +
              std::to_string(sv->io_budget) + " bytes)");
    return BF_ERR_BUSY;
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
  free_ctx(sv->shared);
  for (Slot& sl : sv->slot) {
    free_ctx(sl.ctx);
    if (sl.d_buf) {
      cudaFree(sl.d_buf);
      sv->g->device_bytes -= sl.buf_bytes;
    }
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.h_stage) cudaFreeHost(sl.h_stage);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  delete h;
}

}  // extern "C"
