/*
 * bf_phast.h — C ABI of the GB300 K-lane PHAST engine.
 *
 * Drop-in device layer for butterfly-route's batched PHAST path: many-to-many
 * duration matrices and bulk isochrones over a rank-aligned CCH. The entry
 * points mirror the Rust call surface they replace (paths relative to the
 * butterfly-osm repository):
 *
 *   bf_graph_create        BatchedPhastEngine::new / PhastEngine::new
 *                          route/src/matrix/batched_phast.rs:89, route/src/range/phast.rs:86
 *                          (+ the INF-filtering flats UpAdjFlat::build_with, DownAdjFlat::build,
 *                           DownReverseAdjFlat::build_with, route/src/matrix/bucket_ch.rs:191,282,355)
 *   bf_graph_info          BatchedPhastEngine::n_nodes  batched_phast.rs:115
 *   bf_query_batch         BatchedPhastEngine::query_batch          batched_phast.rs:131
 *                          BatchedPhastEngine::query_batch_bounded  batched_phast.rs:271
 *   bf_phast_query         PhastEngine::query                        phast.rs:155
 *   bf_matrix              BatchedPhastEngine::compute_matrix_flat   batched_phast.rs:667
 *                          (and compute_matrix_flat_soa :756, compute_matrix_block_gated :1223)
 *   bf_matrix_seeded       table_phast_lopsided                      route/src/matrix/bucket_ch.rs:6717
 *   bf_phast_bounded_seeded run_phast_bounded_fast_seeded            route/src/server/isochrone_handler.rs:338
 *   bf_graph_create_2ch    the optional len-along-time flats         route/src/server/state.rs:2962
 *   bf_router_*            phast_wins / update_cost_ewma             bucket_ch.rs:6655-6712
 *   bf_matrix_seeded_2ch   table_phast_lopsided_2ch                  bucket_ch.rs:6381-6521
 *   bf_phast_bounded_seeded_2ch run_phast_bounded_fast_seeded_2ch    isochrone_handler.rs:500-625
 *   bf_isochrone_bitsets   the PHAST part of isochrone_bulk_handler  isochrone_handler.rs:1668-1709
 *   bf_isochrone_settled   run_phast_bounded_fast_seeded for many origins  isochrone_handler.rs:338
 *                          and BatchedIsochroneEngine::query_many    route/src/range/batched_isochrone.rs:216
 *   bf_server_*            the tiling / admission loop of do_matrix  route/src/server/flight.rs:589,957-1110
 *   bf_cch_customize       customize_cch_time_in_memory (weights)    route/src/customization.rs:571
 *   bf_cch_relax[_lex]     triangle_relax_parallel / _lex_parallel   customization.rs:1083, :1253
 *   bf_cch_bottom_up       bottom_up_customize / _with_external_middles  customization.rs:1005, :953
 *   bf_contour_rasters     generate_sparse_contour_anchored, steps 1-3  route/src/range/sparse_contour.rs:650
 *   bf_contour_polygons    generate_sparse_contour_anchored, steps 4-5  sparse_contour.rs:770
 *   bf_isochrone_polygons  build_isochrone_geometry for many origins  route/src/server/geometry.rs:239
 *   bf_tile_emit[_device]  build_matrix_batch / build_matrix_tile_batch  route/src/server/flight.rs:432,509
 *
 * Conventions (as in the reference):
 *   - node ids are CCH ranks (rank-aligned CCH, node_id == rank);
 *   - distances are u32 deciseconds (any unit works: arithmetic is exact
 *     saturating u32 min-plus); 0xFFFFFFFF means unreachable;
 *   - a weight of 0xFFFFFFFF in the input CSR is an INF edge and is dropped,
 *     exactly like the reference flats;
 *   - bounded results are exact for values <= threshold; the engine reports
 *     every cell / node above the threshold as 0xFFFFFFFF (the server-side
 *     post-filter of the reference, bucket_ch.rs:6800-6803).
 *
 * Ownership: the library owns graph and server handles; callers own every
 * input and output buffer. A graph is immutable after creation; calls on one
 * graph from several host threads are serialised internally.
 *
 * Errors: every entry point returns a bf_status and never aborts. The
 * message of the last failure on the calling thread is bf_last_error().
 * The status style follows dl/include/butterfly.h:66-72 of the reference.
 */
#ifndef BF_PHAST_H
#define BF_PHAST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bf_status {
  BF_OK = 0,
  BF_ERR_INVALID = 1,     /* bad argument (null pointer, id out of range, ...)   */
  BF_ERR_OOM = 2,         /* device or pinned-host allocation failed             */
  BF_ERR_DEVICE = 3,      /* CUDA error or no usable sm_103 device               */
  BF_ERR_TIMEOUT = 4,     /* a bounded device wait ran out                       */
  BF_ERR_CANCELLED = 5,   /* request cancelled                                   */
  BF_ERR_BUSY = 6,        /* admission refused: HBM budget or queue full         */
  BF_ERR_UNSUPPORTED = 7  /* option not supported on this graph / build          */
} bf_status;

#define BF_INF 0xFFFFFFFFu

/* Rank-aligned CCH adjacency: CchTopo + CchWeights of the reference
 * (route/src/formats/cch_topo.rs:250-284, cch_weights.rs:359). UP edges go
 * from a node to higher ranks, DOWN edges to lower ranks, both indexed by
 * source rank. Weights of 0xFFFFFFFF are INF and dropped. */
typedef struct bf_cch_csr {
  uint32_t n_nodes;
  uint32_t reserved;
  const uint64_t* up_offsets;   /* [n_nodes + 1] */
  const uint32_t* up_targets;   /* [up_offsets[n_nodes]] */
  const uint32_t* up_weights;   /* [up_offsets[n_nodes]] */
  const uint64_t* down_offsets; /* [n_nodes + 1] */
  const uint32_t* down_targets; /* [down_offsets[n_nodes]] */
  const uint32_t* down_weights; /* [down_offsets[n_nodes]] */
} bf_cch_csr;

/* Engines behind bf_matrix / bf_matrix_device. */
typedef enum bf_engine {
  BF_ENGINE_AUTO = 0,     /* batched engine (the default)                        */
  BF_ENGINE_PLAIN = 1,    /* one K=32 batch at a time: upward launch, one sweep
                             launch per level, one extraction launch             */
  BF_ENGINE_BATCHED = 2   /* persistent multi-batch kernels, shared-memory
                             subtrees, CUDA-graph level schedule, autotuned K    */
} bf_engine;

typedef struct bf_config {
  int32_t device;             /* CUDA device ordinal                               */
  uint32_t engine;            /* bf_engine                                         */
  uint32_t k_lanes;           /* lanes per batch for the batched engine (0 = autotune;
                                 16, 32, 64 or 128)                                */
  uint32_t flags;             /* BF_FLAG_* bits                                    */
  uint64_t hbm_budget_bytes;  /* cap on device memory for distance slabs and
                                 scratch (0 = 85% of free memory at creation)      */
  uint32_t subtree_nodes;     /* max nodes of a shared-memory subtree (0 = auto)   */
  uint32_t reserved2;
} bf_config;

/* bf_config.flags: build the CCH of the transposed graph. Every entry point
 * then answers the all-to-one (arrive-by) question: bf_phast_query(g, t) is
 * PhastEngine::query_block_gated_reverse (route/src/range/phast.rs:879), the
 * isochrones are the reverse isochrones of run_phast_bounded_fast_reverse_seeded
 * (route/src/server/isochrone_handler.rs:657-780), and bf_matrix(g, T, S)
 * is the transpose of the forward S x T matrix. */
#define BF_FLAG_REVERSE 1u

typedef struct bf_graph bf_graph;

typedef struct bf_graph_info {
  uint32_t n_nodes;
  uint32_t n_levels;          /* levels of the downward pull DAG                   */
  uint64_t n_up;              /* finite UP edges                                   */
  uint64_t n_down;            /* finite DOWN edges                                 */
  uint32_t max_depth;         /* elimination-tree depth (upward path length - 1)   */
  uint32_t n_top_nodes;       /* nodes above the shared-memory subtrees            */
  uint32_t n_subtrees;        /* shared-memory subtrees                            */
  uint32_t k_lanes;           /* lanes per batch chosen for the batched engine     */
  uint64_t device_bytes;      /* device memory held by the graph                   */
} bf_graph_info;

/* Per-call statistics (BatchedPhastStats, batched_phast.rs:67-80). Times are
 * device times from CUDA events, in milliseconds. */
typedef struct bf_stats {
  uint64_t n_sources;
  uint64_t n_targets;
  uint64_t n_batches;
  uint64_t kernel_launches;   /* kernels launched by the call                      */
  double upward_ms;
  double downward_ms;
  double extract_ms;
  double total_ms;            /* whole call, host clock                            */
  uint64_t h2d_bytes;
  uint64_t d2h_bytes;
  uint64_t swept_nodes;       /* rows processed by the downward sweep (per wave)  */
  uint64_t swept_edges;       /* DOWN edges relaxed per lane (per wave)           */
  uint64_t lanes;             /* lanes (sources) per wave, padded to 4            */
  uint64_t waves;             /* sweeps run                                       */
  double schedule_ms;         /* host time building sweep schedules (0 on reuse)  */
  uint64_t sweep_bytes;       /* isochrone calls: algorithmic bytes of the gated
                                 sweeps (schedule records scanned, active source
                                 rows gathered, rows written), summed over waves */
  uint64_t active_rows;       /* isochrone calls: rows written by the sweeps      */
} bf_stats;

bf_status bf_graph_create(const bf_cch_csr* csr, const bf_config* cfg, bf_graph** out);
void bf_graph_destroy(bf_graph* g);
bf_status bf_graph_info_get(const bf_graph* g, bf_graph_info* out);
/* Select the engine used by bf_matrix / bf_matrix_device on this graph. */
bf_status bf_graph_set_engine(bf_graph* g, uint32_t engine, uint32_t k_lanes);

/* Tunables of the batched engine's sweep. */
typedef struct bf_tune {
  uint32_t threads_per_block;  /* sweep block size (each thread owns 4 lanes)    */
  uint32_t edges_per_item;     /* max in-edges per work item (larger in-degrees
                                  are split into slices combined by atomicMin)   */
  uint32_t graph_capture;      /* replay the level schedule from a CUDA graph   */
  uint32_t lanes_per_wave;     /* 0 = as many lanes as the HBM budget allows     */
  double step_ms;              /* device time of the sample under this choice    */
  uint32_t tried;              /* candidates timed by bf_autotune               */
  uint32_t isochrone_lanes;    /* origins per isochrone wave (0 = budget-limited;
                                  small waves keep the gated active set compact) */
  uint32_t small_level_rows;   /* levels with fewer rows than this use ...        */
  uint32_t small_level_edges;  /* ... at most this many in-edges per work item:
                                  short dependent load chains where a level is
                                  too small to hide latency (0 = off)           */
  uint32_t overlap_levels;     /* 1: launch each level as a programmatic
                                  dependent of the previous one, so its blocks
                                  are scheduled while that level drains        */
  uint32_t isochrone_16bit;    /* 1: isochrone calls whose thresholds are all
                                  below 0xFFFF keep 16-bit lanes clamped at the
                                  threshold (exact, half the bytes)             */
  uint32_t overlap_upward;     /* 1: matrix waves run the upward pass on a side
                                  stream while the slab is reset               */
  uint32_t mapped_output;      /* 1: bf_matrix into page-locked host memory is
                                  written by the extraction kernel directly     */
  uint32_t hub_l2_mb;          /* L2 megabytes kept for the most-gathered rows
                                  (evict-last cache hints; 0 = no hints)         */
  uint32_t device_schedule;    /* 1: target-restricted schedules are built on
                                  the device; 0: by host threads (same rows)    */
  uint32_t persistent_sweep;   /* bit 0 (default): the plain engine's sweep of a
                                  K = 32 batch, bit 1: each 16-bit isochrone
                                  wave's sweep, runs as one cooperative launch
                                  walking all levels (grid barriers with a
                                  deadline: BF_ERR_TIMEOUT if one runs out);
                                  clear: one launch per level                    */
  uint32_t staged_levels;      /* 1: runs of small levels of 16-bit isochrone
                                  waves bulk-copy each level's work items and
                                  edge records into shared memory (cp.async.bulk
                                  with an mbarrier) while the previous level is
                                  swept; 0: the records are read from global
                                  memory (same results)                          */
} bf_tune;

/* Time candidate tunables on a sample matrix (device buffers: d_sources,
 * d_targets) and keep the fastest for this graph; *best receives it. reps
 * timed repetitions per candidate (after one warm-up). */
bf_status bf_autotune(bf_graph* g, const uint32_t* d_sources, uint64_t n_sources,
                      const uint32_t* d_targets, uint64_t n_targets, uint32_t reps,
                      bf_tune* best);
/* Set (e.g. from a cached autotune result) or read back the tunables. */
bf_status bf_set_tune(bf_graph* g, const bf_tune* t);
bf_status bf_get_tune(const bf_graph* g, bf_tune* t);

/* Time bulk-isochrone candidates on a device-resident sample of n origins
 * and thresholds (isochrone_lanes in {256, 512, 1024, 2048} up to the sample
 * size, with and without persistent waves, bit 1 of persistent_sweep) and
 * keep the fastest for this graph; the other tunables are left as they are.
 * No reference counterpart: the reference's isochrone batch width is the
 * fixed K_LANES (route/src/range/batched_isochrone.rs). */
bf_status bf_autotune_isochrones(bf_graph* g, const uint32_t* d_origins,
                                 const uint32_t* d_thresholds, uint64_t n, uint32_t reps,
                                 bf_tune* best);

/* Per level of the last target-restricted schedule of the graph's C-ABI
 * matrix calls: work items, edge records and rows (first min(cap, levels)
 * entries; *n_levels = levels). For profiling: the k-th launch of a sweep
 * processes the k-th level with items. No reference counterpart. */
bf_status bf_schedule_levels(const bf_graph* g, uint32_t cap, uint64_t* items, uint64_t* edges,
                             uint64_t* rows, uint32_t* n_levels);

/* Tune cache: write the graph's current tunables to a JSON file keyed by a
 * fingerprint of the graph (node and edge counts, levels, depth and the
 * level sizes), and apply such a file to a graph; a file written for
 * another graph, or incomplete, is refused with BF_ERR_INVALID. No
 * reference counterpart. */
bf_status bf_tune_save(const bf_graph* g, const char* path);
bf_status bf_tune_load(bf_graph* g, const char* path);

/* Distances from k sources to every node: dist_out[lane * n_nodes + node]
 * (the AoS Vec<Vec<u32>> of query_batch). threshold == BF_INF is unbounded;
 * otherwise entries above the threshold are BF_INF. k is at most 128. */
bf_status bf_query_batch(bf_graph* g, const uint32_t* sources, uint32_t k, uint32_t threshold,
                         uint32_t* dist_out);

/* Fixed size of the device scratch array behind bf_query_batch_noalloc. */
#define BF_NOALLOC_SCRATCH_BYTES (4u << 20)

/* bf_query_batch for callers that cannot allocate memory. It has no
 * counterpart in the reference. Callers whose device memory is all reserved
 * up front by their own pool allocator, or who cannot afford cudaMalloc's
 * implicit device synchronisation on their hot path, pass device buffers:
 * d_sources (k ranks) and d_dist_out (k * n_nodes u32, laid out as
 * bf_query_batch's dist_out). The call allocates nothing: its only scratch
 * (the upward pass's ancestor paths, 8 * (max_depth + 1) bytes per source) is
 * a static device array of BF_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library holds until exit. Limits: k <= 32 and k * 8 * (max_depth + 1) <=
 * BF_NOALLOC_SCRATCH_BYTES, else BF_ERR_INVALID. CUDA loads the array (and
 * the code that uses it) lazily; bf_graph_create loads it on the graph's
 * device, and a call with k = 0 loads it and resolves its address without
 * doing any work: make such a call before reserving the rest of the device
 * memory for another allocator and before any stream capture. All calls
 * share the array: calls whose work overlaps on the GPU race and must be
 * serialised by the caller. stream is a cudaStream_t or NULL for the graph's
 * stream; the call returns after the work completed. */
bf_status bf_query_batch_noalloc(bf_graph* g, const uint32_t* d_sources, uint32_t k,
                                 uint32_t threshold, uint32_t* d_dist_out, void* stream);

/* Single-source unbounded PHAST (PhastEngine::query). */
bf_status bf_phast_query(bf_graph* g, uint32_t origin, uint32_t* dist_out);

/* S x T duration matrix, row-major out[s * T + t], host buffers. threshold
 * == BF_INF is unbounded; otherwise cells above it are BF_INF. st may be
 * NULL. */
bf_status bf_matrix(bf_graph* g, const uint32_t* sources, uint64_t n_sources,
                    const uint32_t* targets, uint64_t n_targets, uint32_t threshold,
                    uint32_t* out, bf_stats* st);

/* Same as bf_matrix with device pointers (sources, targets and out in device
 * memory of the graph's device). stream is a cudaStream_t or NULL for the
 * library's own stream; the call returns after the work completed. */
bf_status bf_matrix_device(bf_graph* g, const uint32_t* d_sources, uint64_t n_sources,
                           const uint32_t* d_targets, uint64_t n_targets, uint32_t threshold,
                           uint32_t* d_out, void* stream, bf_stats* st);

/* Phantom-seeded matrix (table_phast_lopsided, bucket_ch.rs:6717-6852).
 * Source s has seeds src_seeds[src_off[s] .. src_off[s+1]), each a (rank,
 * cost) pair entered into its field F_s with that cost (a super-source);
 * target t's value is min over its seeds (rank, part) of F_s[rank] - part
 * (saturating, unreachable seeds skipped). Cells above the threshold are
 * BF_INF. A pair whose source and target share a seed rank (a same-edge
 * move, which the reference recomputes with its bucket engine,
 * bucket_ch.rs:6786-6845) is a conflict: its cell is left BF_INF and its
 * index s * n_targets + t is reported in conflict_cells (ascending, at most
 * conflict_cap written; *n_conflicts receives the total) for the caller's
 * bucket path. conflict_cells may be NULL when conflict_cap is 0. */
typedef struct bf_seed {
  uint32_t rank;
  uint32_t cost;
} bf_seed;
bf_status bf_matrix_seeded(bf_graph* g, const bf_seed* src_seeds, const uint64_t* src_off,
                           uint64_t n_sources, const bf_seed* tgt_seeds, const uint64_t* tgt_off,
                           uint64_t n_targets, uint32_t threshold, uint32_t* out,
                           uint64_t* conflict_cells, uint64_t conflict_cap,
                           uint64_t* n_conflicts, bf_stats* st);

/* run_phast_bounded_fast_seeded: settled (rank, dist <= threshold) pairs in
 * ascending rank order. Writes at most cap pairs; *n_out receives the full
 * count. */
bf_status bf_phast_bounded_seeded(bf_graph* g, const bf_seed* seeds, uint32_t n_seeds,
                                  uint32_t threshold, uint32_t* out_rank, uint32_t* out_dist,
                                  uint64_t cap, uint64_t* n_out);

/* ---- two channels: time and length along the time-optimal path ----------
 * A graph created with bf_graph_create_2ch also carries a length weight per
 * CCH edge (the reference's cch_weights_len_along_time, same indexing as the
 * time weights). Both channels follow the same path: labels are compared by
 * time, ties by length (the reference's lexicographic tie-break,
 * isochrone_handler.rs:543-571, :599-611). The length weights must be
 * 0xFFFFFFFF exactly where the time weights are (the reference's length flats
 * drop INF edges independently and index them as aligned with the time
 * flats); otherwise BF_ERR_INVALID. The 2ch calls return BF_ERR_UNSUPPORTED
 * on a graph created without lengths. */
bf_status bf_graph_create_2ch(const bf_cch_csr* csr, const uint32_t* up_len_weights,
                              const uint32_t* down_len_weights, const bf_config* cfg,
                              bf_graph** out);

/* A two-channel seed: (rank, time cost, length cost), the reference's
 * EngineSeed (rank, part_time, part_len) (bucket_ch.rs:6039). */
typedef struct bf_seed2 {
  uint32_t rank;
  uint32_t cost;
  uint32_t len;
} bf_seed2;

/* table_phast_lopsided_2ch: out_time as bf_matrix_seeded; out_len[s*T + t] is
 * F_len[rank] - part_len of the first target seed (in the given order) that
 * attains the cell's time, BF_INF where the time cell is BF_INF. Several
 * seeds of one source on the same rank keep the first with the smallest
 * cost (isochrone_handler.rs:527-531). Conflicts as in bf_matrix_seeded; both
 * cells stay BF_INF there. */
bf_status bf_matrix_seeded_2ch(bf_graph* g, const bf_seed2* src_seeds, const uint64_t* src_off,
                               uint64_t n_sources, const bf_seed2* tgt_seeds,
                               const uint64_t* tgt_off, uint64_t n_targets, uint32_t threshold,
                               uint32_t* out_time, uint32_t* out_len, uint64_t* conflict_cells,
                               uint64_t conflict_cap, uint64_t* n_conflicts, bf_stats* st);

/* run_phast_bounded_fast_seeded_2ch: settled (rank, time <= threshold, len)
 * triples in ascending rank order; at most cap written, *n_out = total. */
bf_status bf_phast_bounded_seeded_2ch(bf_graph* g, const bf_seed2* seeds, uint32_t n_seeds,
                                      uint32_t threshold, uint32_t* out_rank, uint32_t* out_time,
                                      uint32_t* out_len, uint64_t cap, uint64_t* n_out);

/* ---- router cost model (phast_wins, bucket_ch.rs:6655-6712) ---------------
 * Chooses between the seeded PHAST matrix and the caller's bucket engine:
 * PHAST iff n_sources <= n_targets and n_sources * scan < (n_sources +
 * n_targets) * sweep, with scan / sweep the EWMA (alpha 1/4) of measured
 * per-field and per-sweep nanoseconds, or before both are measured the
 * structural bound scan = n_nodes, sweep = clamp(n_nodes / 400, 500, 20000).
 * One bf_router per process replaces the reference's two static atomics;
 * updates and reads are atomic. Feed the GPU's cost with
 * bf_router_observe_stats (the per-source share of a bf_matrix_seeded call)
 * and the bucket engine's with BF_COST_SWEEP samples. `force` carries the
 * caller's BUTTERFLY_MATRIX_ALGO override. Returns 1 for PHAST, 0 for bucket. */
typedef struct bf_router {
  uint64_t sweep_ns;  /* 0 = not measured yet */
  uint64_t scan_ns;
} bf_router;
enum { BF_COST_SWEEP = 0, BF_COST_SCAN = 1 };
enum { BF_ROUTE_AUTO = 0, BF_ROUTE_BUCKET = 1, BF_ROUTE_PHAST = 2 };
void bf_router_observe(bf_router* r, uint32_t which, uint64_t sample_ns);
void bf_router_observe_stats(bf_router* r, const bf_stats* st);
int bf_router_phast_wins(const bf_router* r, uint64_t n_sources, uint64_t n_targets,
                         uint64_t n_nodes, uint32_t force);

/* Bulk isochrones: origin i with threshold thresholds[i]; bit r of row i
 * (rows of ceil(n_nodes / 64) u64 words) is set iff dist(origin_i, r) <=
 * thresholds[i]; counts_out[i] is the row's popcount. counts_out may be
 * NULL. */
bf_status bf_isochrone_bitsets(bf_graph* g, const uint32_t* origins, const uint32_t* thresholds,
                               uint64_t n_origins, uint64_t* bits_out, uint64_t* counts_out,
                               bf_stats* st);

/* bf_isochrone_bitsets with device buffers (d_origins, d_thresholds: n
 * entries; d_bits: n rows of ceil(n_nodes / 64) u64; d_counts: n u64) on the
 * given stream (NULL = the graph's stream); returns after completion. */
bf_status bf_isochrone_bitsets_device(bf_graph* g, const uint32_t* d_origins,
                                      const uint32_t* d_thresholds, uint64_t n_origins,
                                      uint64_t* d_bits, uint64_t* d_counts, void* stream,
                                      bf_stats* st);

/* Settled sets of bulk isochrones: for origin i, the ranks r with
 * dist(origin_i, r) <= thresholds[i], ascending, and their distances — the
 * run_phast_bounded_fast_seeded output (isochrone_handler.rs:338-491) of
 * every origin, computed with the same waves as bf_isochrone_bitsets.
 * Origin i owns entries [offsets[i], offsets[i + 1]) (n + 1 offsets) of
 * *ranks and *dists, buffers released with bf_settled_free. */
bf_status bf_isochrone_settled(bf_graph* g, const uint32_t* origins, const uint32_t* thresholds,
                               uint64_t n_origins, uint64_t* offsets, uint32_t** ranks,
                               uint32_t** dists, bf_stats* st);
void bf_settled_free(uint32_t* p);

/* ---- serving loop (continuous batching of matrix and isochrone requests) ---- */

typedef struct bf_server bf_server;

typedef struct bf_server_cfg {
  uint64_t hbm_budget_bytes;  /* device memory for in-flight requests: their I/O
                                 buffers and the slots' distance slabs (0 = 80%
                                 of free memory at creation)                     */
  uint32_t max_inflight;      /* requests admitted into one batch (0 = 64)        */
  uint32_t max_queue;         /* queued requests before BF_ERR_BUSY (0 = 4096)    */
  uint32_t timeout_ms;        /* bound on a matrix batch's device work from its
                                 start; past it the batch's requests complete
                                 with BF_ERR_TIMEOUT (outputs undefined) once its
                                 stream drained (0 = 10000)                       */
  uint32_t slots;             /* worker slots computing batches concurrently, each
                                 with its own stream (0 = 4, at most 8)          */
} bf_server_cfg;

typedef enum bf_request_kind { BF_REQ_MATRIX = 1, BF_REQ_ISOCHRONE = 2 } bf_request_kind;

/* A request. For BF_REQ_MATRIX: sources/targets (n_sources x n_targets) and
 * out (n_sources * n_targets u32). For BF_REQ_ISOCHRONE: one origin in
 * sources[0], threshold, and out = bitset words (ceil(n_nodes/64) u64 as u32
 * pairs, little-endian). Buffers are owned by the caller and must stay valid
 * until the request completes. */
typedef struct bf_request {
  uint32_t kind;
  uint32_t threshold;
  const uint32_t* sources;
  uint64_t n_sources;
  const uint32_t* targets;
  uint64_t n_targets;
  void* out;
  uint64_t user_tag;
} bf_request;

typedef struct bf_completion {
  uint64_t user_tag;
  uint64_t ticket;
  int32_t status;            /* bf_status of the request                        */
  uint32_t reserved;
  double submit_s;           /* host clock, seconds                             */
  double admit_s;
  double done_s;
} bf_completion;

bf_status bf_server_create(bf_graph* g, const bf_server_cfg* cfg, bf_server** out);
/* Queue a request; *ticket identifies it. Returns BF_ERR_BUSY when the queue
 * is full or the request's device I/O alone exceeds the HBM budget.
 * Admission: a free slot forms a batch from the waiting requests of one kind
 * while their device I/O fits both what the budget leaves beside the batches
 * in flight and the device's free memory (cudaMemGetInfo, less a margin); a
 * request that does not fit waits until a batch completes. */
bf_status bf_server_submit(bf_server* s, const bf_request* req, uint64_t* ticket);
/* Collect up to cap completions; waits up to wait_ms for the first one. */
bf_status bf_server_poll(bf_server* s, bf_completion* out, uint32_t cap, uint32_t wait_ms,
                         uint32_t* n_out);
bf_status bf_server_cancel(bf_server* s, uint64_t ticket);
void bf_server_destroy(bf_server* s);

/* ---- CCH customization (route/src/customization.rs:953-1436) ---------------
 * A bf_cch holds one rank-space CCH topology on the device (the reference's
 * CchTopo, formats/cch_topo.rs:250-290): UP edges u -> v (v > u) and DOWN
 * edges u -> v (v < u) as two CSRs, targets strictly ascending per node,
 * optional per-edge shortcut flags and contraction middles (u32::MAX on an
 * original arc). Every call keeps the reference's array layout: one u32 per
 * UP edge and one per DOWN edge, u32::MAX = no edge / unreachable.
 *
 * The relaxation's result is, for every edge, the smaller of its seed and
 * the minimum over its lower triangles x -> m -> y of
 * (w(x -> m) + w(m -> y), m), packed weight-major with the apex as
 * tie-break, sums saturating, legs of weight u32::MAX skipped. That value is
 * unique, so one pass in elimination-tree order returns bit for bit what the
 * reference's passes-until-stable return, middles included. */
typedef struct bf_cch bf_cch;

/* bf_cch_topo.flags: search each triangle's target edge in every call
 * instead of precomputing it (4 bytes per triangle, taken when that fits a
 * quarter of the free device memory). */
#define BF_CCH_SEARCH_TARGETS 1u

typedef struct bf_cch_topo {
  uint32_t n_nodes;
  uint32_t flags;                   /* BF_CCH_* */
  const uint64_t* up_offsets;       /* [n_nodes + 1]                                */
  const uint32_t* up_targets;
  const uint8_t* up_is_shortcut;    /* 0/1 per UP edge; NULL = no shortcuts        */
  const uint32_t* up_middle;        /* per UP edge; NULL = all u32::MAX            */
  const uint64_t* down_offsets;     /* [n_nodes + 1]                                */
  const uint32_t* down_targets;
  const uint8_t* down_is_shortcut;
  const uint32_t* down_middle;
} bf_cch_topo;

typedef struct bf_cch_stats {
  uint32_t n_nodes;
  uint32_t levels;                /* elimination-tree levels                        */
  uint64_t up_edges;
  uint64_t down_edges;
  uint64_t triangles;             /* x -> m -> y with x != y over the pair rows      */
  uint64_t bottom_up_shortcuts;
  uint32_t apexes;                /* nodes with at least one triangle               */
  uint32_t etree_levels;          /* 1: heights of the elimination tree, 0: longest path */
  uint32_t target_index;          /* 1: target slots precomputed per pair candidate  */
  uint32_t pairs;                 /* unordered node pairs (one 16-byte slot each)     */
  double plan_ms;                 /* bf_cch_create                                  */
  double last_device_ms;          /* last call: device time without host copies     */
  double last_total_ms;           /* last call: wall time with host copies          */
} bf_cch_stats;

/* Uploads the topology and builds the level plan (reverse DOWN adjacency,
 * elimination-tree levels, triangle prefix). Replaces
 * build_reverse_down_adj_for_relax (customization.rs:832-875) and the
 * topology load before customize_cch / customize_cch_time_in_memory. */
bf_status bf_cch_create(const bf_cch_topo* topo, int device, bf_cch** out);
void bf_cch_destroy(bf_cch* c);
bf_status bf_cch_info(const bf_cch* c, bf_cch_stats* out);

/* triangle_relax_parallel (customization.rs:1083-1200): seeds in, converged
 * weights and middles out, in place. */
bf_status bf_cch_relax(bf_cch* c, uint32_t* up_w, uint32_t* down_w, uint32_t* up_mid,
                       uint32_t* down_mid);

/* bottom_up_customize + triangle_relax_parallel (customization.rs:571-650,
 * customize_cch_time_in_memory): original arc weights in (entries of
 * shortcut edges ignored), customized weights and middles out. A shortcut's
 * bottom-up seed is dominated by the triangle through its own contraction
 * middle, so the relaxation is seeded with u32::MAX there: same result. */
bf_status bf_cch_customize(bf_cch* c, const uint32_t* orig_up, const uint32_t* orig_down,
                           uint32_t* up_w, uint32_t* down_w, uint32_t* up_mid,
                           uint32_t* down_mid);

/* triangle_relax_lex_parallel (customization.rs:1253-1436): (time, length)
 * seeds, compared time first; times and middles updated in place. Each
 * shortcut elects the smallest apex whose (time, length) sum equals its
 * converged pair; original edges and shortcuts without such an apex keep the
 * given middle. Needs the topology's shortcut flags. */
bf_status bf_cch_relax_lex(bf_cch* c, uint32_t* up_t, uint32_t* down_t, const uint32_t* up_len,
                           const uint32_t* down_len, uint32_t* up_mid, uint32_t* down_mid);

/* bottom_up_with_external_middles / bottom_up_customize
 * (customization.rs:953-1052): an original edge takes its original weight,
 * a shortcut u -> v with middle m takes w(u -> m) + w(m -> v) (saturating; a
 * missing leg, or a middle not below both endpoints, reads u32::MAX). Middles
 * NULL = the topology's. BF_ERR_INVALID when a shortcut's middle is not a
 * rank (the reference indexes out of bounds there). */
bf_status bf_cch_bottom_up(bf_cch* c, const uint32_t* orig_up, const uint32_t* orig_down,
                           const uint32_t* up_mid, const uint32_t* down_mid, uint32_t* up_w,
                           uint32_t* down_w);

/* ---- isochrone contour rasters (range/sparse_contour.rs:650-770) ----------
 * Steps 1-3 of the reference's contour pipeline for a batch of isochrones:
 * stamp each isochrone's reachable segments (Bresenham between the cells of
 * consecutive points, then every point, stamp_line :112-144), the anchor's
 * 3x3 disk, then `dilation` 3x3 dilations and `erosion` 3x3 erosions.
 * Points are Web-Mercator (x, y) metres as the reference's to_mercator gives
 * them (:441-445; project once per static polyline vertex, with the libm the
 * rest of the caller uses). Isochrone k owns segments [iso_seg[k],
 * iso_seg[k + 1]), segment s owns points [seg_pt[s], seg_pt[s + 1]) of xy
 * (x, y pairs); its grid origin is (min x - 3 cells, min y - 3 cells) over
 * its points, cell size cell_m[k]; has_anchor / anchor_xy (x, y per
 * isochrone) may be NULL. Cell (c, r) is set in isochrone k's raster iff
 * the reference's closed tile map holds it: bit (c - col0) % 64 of word
 * word_offset + (r - row0) * width_words + (c - col0) / 64.
 * Rasters are described in `rasters` (n_iso entries); *words receives a
 * buffer of *n_words words that the caller releases with bf_contour_free.
 * With words == NULL only the layout is computed, on the host. */
typedef struct bf_raster {
  int32_t col0, row0;       /* grid cell of bit 0 of the raster's first word   */
  uint32_t width_words;     /* 64-cell words per row                            */
  uint32_t height;          /* rows                                              */
  uint64_t word_offset;     /* first word of this raster in `words`              */
  double origin_x, origin_y; /* grid origin in Mercator metres                   */
} bf_raster;

bf_status bf_contour_rasters(const double* xy, const uint64_t* seg_pt, const uint64_t* iso_seg,
                             uint32_t n_iso, const double* cell_m, const uint8_t* has_anchor,
                             const double* anchor_xy, uint32_t dilation, uint32_t erosion,
                             int device, bf_raster* rasters, uint64_t** words, uint64_t* n_words);
void bf_contour_free(uint64_t* words);
/* bf_contour_rasters keeps its device buffers and stream per device between
 * calls (they only grow); this releases them. */
void bf_contour_release(int device);

/* Steps 4-5 of generate_sparse_contour_anchored (sparse_contour.rs:770-830,
 * 831-1183) on the rasters of bf_contour_rasters (host arrays, in any order),
 * on the current CUDA device: boundary tracing with cell-centre vertices,
 * the ring containing the anchor (Mercator x, y; else the ring with the
 * most vertices, the last of equal length), back-projection to (lon, lat)
 * and Douglas-Peucker with tolerance simplify_m[k] / 111000 degrees. Ring k
 * is points [ring_off[k], ring_off[k + 1]) of *lonlat (n_iso + 1 offsets),
 * a buffer released with bf_contour_free_polygons. */
bf_status bf_contour_polygons(const bf_raster* rasters, const uint64_t* words, uint32_t n_iso,
                              const double* cell_m, const double* simplify_m,
                              const uint8_t* has_anchor, const double* anchor_xy,
                              uint64_t* ring_off, double** lonlat);
void bf_contour_free_polygons(double* lonlat);

/* ---- isochrone polygons end to end (server/geometry.rs:239-368) -----------
 * Travel modes of SparseContourConfig (sparse_contour.rs:476-546). */
enum { BF_MODE_CAR = 0, BF_MODE_BIKE = 1, BF_MODE_FOOT = 2 };

/* SparseContourConfig::for_mode_name_with_threshold: cell size, closing
 * rounds and simplification tolerance for a travel mode and threshold. */
bf_status bf_contour_config(uint32_t mode, uint32_t threshold_s, double* cell_m,
                            uint32_t* dilation, uint32_t* erosion, double* simplify_m);

/* to_mercator (sparse_contour.rs:441-445) of n (lat_e7, lon_e7) points into
 * (x, y) metres, on host threads with the host libm. */
bf_status bf_mercator(uint64_t n, const int32_t* lat_lon_e7, double* xy);

/* Road geometry per graph rank: rank r's polyline is points
 * [poly_off[r], poly_off[r + 1]) of poly_e7 ((lat_e7, lon_e7) pairs), its
 * traversal weight node_w[r] (the reference's node_weights: 0 or u32::MAX =
 * not stamped). Vertices are projected once here. */
typedef struct bf_geometry bf_geometry;
bf_status bf_geometry_create(uint32_t n_nodes, const uint64_t* poly_off, const int32_t* poly_e7,
                             const uint32_t* node_w, bf_geometry** out);
void bf_geometry_destroy(bf_geometry* geo);

/* build_isochrone_geometry for n origins: settled sets (bf_isochrone_settled),
 * each settled road stamped whole or cut at the threshold with the
 * reference's f32 fraction, the minimum-distance road's first vertex as the
 * anchor, contour rasters (bf_contour_rasters) and polygons
 * (bf_contour_polygons) with the configuration of `mode` at
 * tier_thresholds[i] (NULL = thresholds, when both are in seconds). Ring i
 * is points [ring_off[i], ring_off[i + 1]) of *lonlat, released with
 * bf_contour_free_polygons. phase_ms (4 entries, may be NULL): settled sets,
 * segments, rasters, polygons. */
bf_status bf_isochrone_polygons(bf_graph* g, const bf_geometry* geo, const uint32_t* origins,
                                const uint32_t* thresholds, const uint32_t* tier_thresholds,
                                uint64_t n, uint32_t mode, uint64_t* ring_off, double** lonlat,
                                double* phase_ms);

/* ---- matrix tile emission: the RecordBatch columns of a matrix block ----
 *
 * build_matrix_batch / build_matrix_tile_batch (route/src/server/flight.rs:
 * 432-500, 509-589) on the GPU. The n_src x n_dst row-major durations
 * `matrix` (and the optional length-along-time `lat`, same shape) become the
 * columns source_idx, target_idx, duration_ms, distance_m in row-major cell
 * order: source_idx / target_idx are the original indices src_orig[si] /
 * dst_orig[di]; a cell is pruned (u32::MAX) when the radius mask is given
 * (mask_off != NULL: source o's sorted list of original destination indices
 * is mask[mask_off[o] .. mask_off[o + 1]), o < n_mask_src) and lacks the
 * destination; a cell above `threshold` reads u32::MAX (0xFFFFFFFF = no
 * bound, as build_matrix_batch); with `sparse` cells whose duration is
 * u32::MAX are dropped; duration_ms = min(d * 1000, u32::MAX), distance_m =
 * lat's cell or u32::MAX, both u32::MAX on a dropped-duration cell. Each
 * column must hold n_src * n_dst values; *n_rows gets the rows written (0
 * for an all-sentinel sparse block: the reference's None). The columns are
 * Arrow UInt32 arrays without nulls, ready to wrap.
 */
typedef struct bf_tile_columns {
  uint32_t* source_idx;
  uint32_t* target_idx;
  uint32_t* duration_ms;
  uint32_t* distance_m;
} bf_tile_columns;

/* Host arrays in and out (page-locked host memory copies fastest). */
bf_status bf_tile_emit(const uint32_t* matrix, const uint32_t* lat, uint32_t n_src,
                       uint32_t n_dst, const uint32_t* src_orig, const uint32_t* dst_orig,
                       uint32_t threshold, const uint64_t* mask_off, const uint32_t* mask,
                       uint32_t n_mask_src, uint32_t sparse, int device,
                       const bf_tile_columns* out, uint64_t* n_rows);

/* Device arrays of `device` in and out (for example the output of
 * bf_matrix_device), on `stream` (NULL: the library's own); n_mask is the
 * length of d_mask. Returns after the work completed. */
bf_status bf_tile_emit_device(const uint32_t* d_matrix, const uint32_t* d_lat, uint32_t n_src,
                              uint32_t n_dst, const uint32_t* d_src_orig,
                              const uint32_t* d_dst_orig, uint32_t threshold,
                              const uint64_t* d_mask_off, const uint32_t* d_mask,
                              uint32_t n_mask_src, uint64_t n_mask, uint32_t sparse, int device,
                              void* stream, const bf_tile_columns* d_out, uint64_t* n_rows);

/* Frees the tile emission's device buffers and stream on `device`. */
void bf_tile_release(int device);

const char* bf_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* BF_PHAST_H */
