/*
 * bf_cch.h — host-side CCH build pipeline for synthetic road graphs.
 *
 * This library produces the rank-aligned, INF-filtered CCH adjacency that the
 * K-lane PHAST engine (include/bf_phast.h) and the CPU oracle consume. It
 * restates the reference's offline build steps in C++:
 *
 *   step 5  node weights + turn penalties   route/src/weights.rs:289-420
 *   step 4  edge-based graph, U-turn rule   route/src/ebg/mod.rs:370-421
 *   step 6  nested-dissection order         route/src/ordering.rs:203 (own partitioner, see below)
 *   step 7  CCH contraction                 route/src/contraction.rs:235-420
 *   step 8  basic customization             route/src/customization.rs:1005-1200, 1443-1520
 *   flats   INF-filtered CSR                route/src/matrix/bucket_ch.rs:191-418
 *
 * The contraction is computed as the chordal completion of the undirected
 * edge-based graph (symbolic elimination along the elimination tree).  After
 * customization an edge u->w of that completion is finite exactly when a
 * directed path u->..->w through lower-ranked nodes exists, which is the edge
 * set the reference's directed in_higher x out_higher contraction produces
 * (contraction.rs:235-330); the INF filter of the flats removes the rest, so
 * the flats are the same either way.
 *
 * The ordering is this library's own nested dissection (balanced minimum
 * edge-cut sweep along the longer coordinate axis, greedy vertex cover of the
 * cut, bit-mask minimum degree on leaves of <= 64 nodes).  It is a fixture
 * generator: any valid order gives a correct CCH, and the oracle and the GPU
 * engine always run on the same order.
 *
 * All arithmetic is integer (coordinates in centimetres, integer square root),
 * so the same seed gives the same graph on x86-64 and aarch64.
 */
#ifndef BF_CCH_H
#define BF_CCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Synthetic graph families. */
enum {
  BFC_KIND_GRID = 0,      /* jittered 4-neighbour grid, 5% removed, 10% one-way      */
  BFC_KIND_COUNTRY = 1    /* jittered lattice with motorway/arterial lines and
                             local-street cells (road hierarchy)                    */
};

typedef struct bfc_synth_params {
  uint32_t kind;          /* BFC_KIND_*                                             */
  uint32_t rows;          /* lattice rows                                           */
  uint32_t cols;          /* lattice columns                                        */
  uint32_t spacing_cm;    /* lattice spacing in centimetres (0 -> 10000 = 100 m)    */
  uint32_t jitter_cm;     /* max |jitter| per coordinate (0 -> spacing / 4)         */
  uint32_t reserved;
  uint64_t seed;          /* RNG seed (default 42 in callers)                       */
} bfc_synth_params;

typedef struct bfc_graph bfc_graph;

/* Edge-based graph (the filtered EBG of the reference). States are directed
 * road segments; arcs are permitted turns. arc weight = node_weight[dst] +
 * turn penalty (customization.rs:1443-1462). */
typedef struct bfc_ebg_view {
  uint32_t n_intersections;
  uint32_t n_states;
  uint64_t n_roads;
  uint64_t n_arcs;
  const uint64_t* arc_off;      /* [n_states + 1]                                    */
  const uint32_t* arc_dst;      /* [n_arcs]                                          */
  const uint32_t* arc_w;        /* [n_arcs] deciseconds                              */
  const uint32_t* node_weight;  /* [n_states] deciseconds, >= 1                      */
  const uint32_t* state_tail;   /* [n_states] intersection id                        */
  const uint32_t* state_head;   /* [n_states] intersection id                        */
  const uint8_t* state_class;   /* [n_states] 0 local, 1 arterial, 2 motorway        */
  const int64_t* ix;            /* [n_intersections] x in cm                         */
  const int64_t* iy;            /* [n_intersections] y in cm                         */
} bfc_ebg_view;

/* Rank-aligned CCH flats (INF edges already removed). */
typedef struct bfc_cch_view {
  uint32_t n_nodes;
  uint32_t reserved;
  uint64_t n_up;                /* finite UP edges   (u -> v, rank v > rank u)        */
  uint64_t n_down;              /* finite DOWN edges (u -> v, rank v < rank u)        */
  uint64_t n_chordal;           /* undirected edges of the chordal completion         */
  const uint64_t* up_off;       /* [n_nodes + 1]                                     */
  const uint32_t* up_tgt;       /* [n_up]                                            */
  const uint32_t* up_w;         /* [n_up]                                            */
  const uint64_t* down_off;     /* [n_nodes + 1]                                     */
  const uint32_t* down_tgt;     /* [n_down]                                          */
  const uint32_t* down_w;       /* [n_down]                                          */
  const uint32_t* rank_to_state;/* [n_nodes]                                         */
  const uint32_t* state_to_rank;/* [n_nodes]                                         */
  double t_generate_s;
  double t_order_s;
  double t_contract_s;
  double t_customize_s;
} bfc_cch_view;

/* The chordal completion behind the flats, in upper-neighbour form: edge e of
 * rank j joins j and tgt[e] (> j); orig_up[e] / orig_down[e] are the original
 * arc weights of j -> tgt[e] / tgt[e] -> j (INF: no arc), cust_* the weights
 * after this library's customization (INF edges are the ones the flats drop). */
typedef struct bfc_topo_view {
  uint32_t n_nodes;
  uint32_t reserved;
  uint64_t n_edges;
  const uint64_t* off;          /* [n_nodes + 1]                                     */
  const uint32_t* tgt;          /* [n_edges]                                         */
  const uint32_t* orig_up;      /* [n_edges]                                         */
  const uint32_t* orig_down;    /* [n_edges]                                         */
  const uint32_t* cust_up;      /* [n_edges]                                         */
  const uint32_t* cust_down;    /* [n_edges]                                         */
} bfc_topo_view;

/* Build a synthetic road graph, its EBG and its CCH. n_threads <= 0 uses all
 * hardware threads. Returns 0 on success; on failure *out is NULL and
 * bfc_last_error() describes the problem. */
int bfc_build_synthetic(const bfc_synth_params* p, int n_threads, bfc_graph** out);

/* Build the CCH of a caller-supplied edge-based graph (arcs with weights and
 * one coordinate pair per state). Used by tests on hand-built graphs. */
int bfc_build_from_arcs(uint32_t n_states, uint64_t n_arcs, const uint32_t* arc_src,
                        const uint32_t* arc_dst, const uint32_t* arc_w, const int64_t* sx,
                        const int64_t* sy, int n_threads, bfc_graph** out);

void bfc_free(bfc_graph* g);
void bfc_ebg(const bfc_graph* g, bfc_ebg_view* out);
void bfc_cch(const bfc_graph* g, bfc_cch_view* out);
void bfc_topo(const bfc_graph* g, bfc_topo_view* out);
const char* bfc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* BF_CCH_H */
