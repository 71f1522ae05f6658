"""Python host binding of the C ABI in include/bf_phast.h (ctypes).

This mirrors the reference engine's call surface for tests and benchmarks:

  Graph(csr)                 BatchedPhastEngine::new      route/src/matrix/batched_phast.rs:89
  Graph.query_batch(src, T)  query_batch / query_batch_bounded  batched_phast.rs:131, :271
  Graph.phast_query(o)       PhastEngine::query           route/src/range/phast.rs:155
  Graph.matrix(src, tgt, T)  compute_matrix_flat          batched_phast.rs:667
  Cch(topo).customize(...)   customize_cch_time_in_memory route/src/customization.rs:571
  Cch.relax / relax_lex      triangle_relax[_lex]_parallel customization.rs:1083, :1253
  Cch.bottom_up(...)         bottom_up_with_external_middles customization.rs:953

The native library is mandatory: importing this module raises if
lib/libbf_phast.so is missing. There is no CPU fallback.
"""
import ctypes
import pathlib

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libbf_phast.so"
INF = 0xFFFFFFFF

BF_OK, BF_ERR_INVALID, BF_ERR_OOM, BF_ERR_DEVICE, BF_ERR_TIMEOUT, BF_ERR_CANCELLED, BF_ERR_BUSY, \
    BF_ERR_UNSUPPORTED = range(8)
ENGINE_AUTO, ENGINE_PLAIN, ENGINE_BATCHED = 0, 1, 2
FLAG_REVERSE = 1
CCH_SEARCH_TARGETS = 1
MODE_CAR, MODE_BIKE, MODE_FOOT = 0, 1, 2
REQ_MATRIX, REQ_ISOCHRONE = 1, 2

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class CchCsr(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("up_offsets", _u64p), ("up_targets", _u32p), ("up_weights", _u32p),
                ("down_offsets", _u64p), ("down_targets", _u32p), ("down_weights", _u32p)]


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("engine", ctypes.c_uint32),
                ("k_lanes", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("hbm_budget_bytes", ctypes.c_uint64), ("subtree_nodes", ctypes.c_uint32),
                ("reserved2", ctypes.c_uint32)]


class GraphInfo(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint32), ("n_levels", ctypes.c_uint32),
                ("n_up", ctypes.c_uint64), ("n_down", ctypes.c_uint64),
                ("max_depth", ctypes.c_uint32), ("n_top_nodes", ctypes.c_uint32),
                ("n_subtrees", ctypes.c_uint32), ("k_lanes", ctypes.c_uint32),
                ("device_bytes", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("n_sources", ctypes.c_uint64), ("n_targets", ctypes.c_uint64),
                ("n_batches", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("upward_ms", ctypes.c_double), ("downward_ms", ctypes.c_double),
                ("extract_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("swept_nodes", ctypes.c_uint64), ("swept_edges", ctypes.c_uint64),
                ("lanes", ctypes.c_uint64), ("waves", ctypes.c_uint64),
                ("schedule_ms", ctypes.c_double), ("sweep_bytes", ctypes.c_uint64),
                ("active_rows", ctypes.c_uint64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Tune(ctypes.Structure):
    _fields_ = [("threads_per_block", ctypes.c_uint32), ("edges_per_item", ctypes.c_uint32),
                ("graph_capture", ctypes.c_uint32), ("lanes_per_wave", ctypes.c_uint32),
                ("step_ms", ctypes.c_double), ("tried", ctypes.c_uint32),
                ("isochrone_lanes", ctypes.c_uint32), ("small_level_rows", ctypes.c_uint32),
                ("small_level_edges", ctypes.c_uint32), ("overlap_levels", ctypes.c_uint32),
                ("isochrone_16bit", ctypes.c_uint32), ("overlap_upward", ctypes.c_uint32),
                ("mapped_output", ctypes.c_uint32), ("hub_l2_mb", ctypes.c_uint32),
                ("device_schedule", ctypes.c_uint32), ("persistent_sweep", ctypes.c_uint32),
                ("staged_levels", ctypes.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Seed(ctypes.Structure):
    _fields_ = [("rank", ctypes.c_uint32), ("cost", ctypes.c_uint32)]


class Seed2(ctypes.Structure):
    _fields_ = [("rank", ctypes.c_uint32), ("cost", ctypes.c_uint32), ("len", ctypes.c_uint32)]


class Router(ctypes.Structure):
    _fields_ = [("sweep_ns", ctypes.c_uint64), ("scan_ns", ctypes.c_uint64)]


COST_SWEEP, COST_SCAN = 0, 1
ROUTE_AUTO, ROUTE_BUCKET, ROUTE_PHAST = 0, 1, 2


class ServerCfg(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("max_queue", ctypes.c_uint32), ("timeout_ms", ctypes.c_uint32),
                ("slots", ctypes.c_uint32)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("threshold", ctypes.c_uint32),
                ("sources", _u32p), ("n_sources", ctypes.c_uint64),
                ("targets", _u32p), ("n_targets", ctypes.c_uint64),
                ("out", ctypes.c_void_p), ("user_tag", ctypes.c_uint64)]


class Completion(ctypes.Structure):
    _fields_ = [("user_tag", ctypes.c_uint64), ("ticket", ctypes.c_uint64),
                ("status", ctypes.c_int32), ("reserved", ctypes.c_uint32),
                ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("done_s", ctypes.c_double)]


class CchTopo(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("up_offsets", _u64p), ("up_targets", _u32p),
                ("up_is_shortcut", ctypes.c_void_p), ("up_middle", _u32p),
                ("down_offsets", _u64p), ("down_targets", _u32p),
                ("down_is_shortcut", ctypes.c_void_p), ("down_middle", _u32p)]


class CchStats(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint32), ("levels", ctypes.c_uint32),
                ("up_edges", ctypes.c_uint64), ("down_edges", ctypes.c_uint64),
                ("triangles", ctypes.c_uint64), ("bottom_up_shortcuts", ctypes.c_uint64),
                ("apexes", ctypes.c_uint32), ("etree_levels", ctypes.c_uint32),
                ("target_index", ctypes.c_uint32), ("pairs", ctypes.c_uint32),
                ("plan_ms", ctypes.c_double), ("last_device_ms", ctypes.c_double),
                ("last_total_ms", ctypes.c_double)]


class Raster(ctypes.Structure):
    _fields_ = [("col0", ctypes.c_int32), ("row0", ctypes.c_int32),
                ("width_words", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("word_offset", ctypes.c_uint64), ("origin_x", ctypes.c_double),
                ("origin_y", ctypes.c_double)]


class TileColumns(ctypes.Structure):
    _fields_ = [("source_idx", ctypes.c_void_p), ("target_idx", ctypes.c_void_p),
                ("duration_ms", ctypes.c_void_p), ("distance_m", ctypes.c_void_p)]


# Every symbol include/bf_phast.h declares, with its ctypes signature.
_SIGNATURES = {
    "bf_graph_create": (ctypes.c_int, [ctypes.POINTER(CchCsr), ctypes.POINTER(Config),
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "bf_graph_create_2ch": (ctypes.c_int, [ctypes.POINTER(CchCsr), _u32p, _u32p,
                                           ctypes.POINTER(Config),
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "bf_graph_destroy": (None, [ctypes.c_void_p]),
    "bf_graph_info_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(GraphInfo)]),
    "bf_graph_set_engine": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]),
    "bf_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                   ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                   ctypes.POINTER(Tune)]),
    "bf_set_tune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tune)]),
    "bf_get_tune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tune)]),
    "bf_autotune_isochrones": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_uint64, ctypes.c_uint32,
                                              ctypes.POINTER(Tune)]),
    "bf_schedule_levels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _u64p, _u64p, _u64p,
                                          ctypes.POINTER(ctypes.c_uint32)]),
    "bf_tune_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "bf_tune_load": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "bf_query_batch": (ctypes.c_int, [ctypes.c_void_p, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                                      _u32p]),
    "bf_phast_query": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _u32p]),
    "bf_query_batch_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                              ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]),
    "bf_matrix": (ctypes.c_int, [ctypes.c_void_p, _u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64,
                                 ctypes.c_uint32, _u32p, ctypes.POINTER(Stats)]),
    "bf_matrix_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                        ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "bf_matrix_seeded": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Seed), _u64p,
                                        ctypes.c_uint64, ctypes.POINTER(Seed), _u64p,
                                        ctypes.c_uint64, ctypes.c_uint32, _u32p, _u64p,
                                        ctypes.c_uint64, _u64p, ctypes.POINTER(Stats)]),
    "bf_phast_bounded_seeded": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Seed),
                                               ctypes.c_uint32, ctypes.c_uint32, _u32p, _u32p,
                                               ctypes.c_uint64, _u64p]),
    "bf_matrix_seeded_2ch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Seed2), _u64p,
                                            ctypes.c_uint64, ctypes.POINTER(Seed2), _u64p,
                                            ctypes.c_uint64, ctypes.c_uint32, _u32p, _u32p, _u64p,
                                            ctypes.c_uint64, _u64p, ctypes.POINTER(Stats)]),
    "bf_phast_bounded_seeded_2ch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Seed2),
                                                   ctypes.c_uint32, ctypes.c_uint32, _u32p,
                                                   _u32p, _u32p, ctypes.c_uint64, _u64p]),
    "bf_router_observe": (None, [ctypes.POINTER(Router), ctypes.c_uint32, ctypes.c_uint64]),
    "bf_router_observe_stats": (None, [ctypes.POINTER(Router), ctypes.POINTER(Stats)]),
    "bf_router_phast_wins": (ctypes.c_int, [ctypes.POINTER(Router), ctypes.c_uint64,
                                            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32]),
    "bf_isochrone_bitsets": (ctypes.c_int, [ctypes.c_void_p, _u32p, _u32p, ctypes.c_uint64,
                                            _u64p, _u64p, ctypes.POINTER(Stats)]),
    "bf_isochrone_bitsets_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.c_uint64,
                                                   ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "bf_isochrone_settled": (ctypes.c_int, [ctypes.c_void_p, _u32p, _u32p, ctypes.c_uint64, _u64p,
                                            ctypes.POINTER(_u32p), ctypes.POINTER(_u32p),
                                            ctypes.POINTER(Stats)]),
    "bf_settled_free": (None, [_u32p]),
    "bf_server_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerCfg),
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "bf_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Request), _u64p]),
    "bf_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Completion),
                                      ctypes.c_uint32, ctypes.c_uint32, _u32p]),
    "bf_server_cancel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "bf_server_destroy": (None, [ctypes.c_void_p]),
    "bf_cch_create": (ctypes.c_int, [ctypes.POINTER(CchTopo), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_void_p)]),
    "bf_cch_destroy": (None, [ctypes.c_void_p]),
    "bf_cch_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CchStats)]),
    "bf_cch_relax": (ctypes.c_int, [ctypes.c_void_p, _u32p, _u32p, _u32p, _u32p]),
    "bf_cch_customize": (ctypes.c_int, [ctypes.c_void_p, _u32p, _u32p, _u32p, _u32p, _u32p,
                                        _u32p]),
    "bf_cch_relax_lex": (ctypes.c_int, [ctypes.c_void_p, _u32p, _u32p, _u32p, _u32p, _u32p,
                                        _u32p]),
    "bf_cch_bottom_up": (ctypes.c_int, [ctypes.c_void_p, _u32p, _u32p, _u32p, _u32p, _u32p,
                                        _u32p]),
    "bf_contour_rasters": (ctypes.c_int, [ctypes.c_void_p, _u64p, _u64p, ctypes.c_uint32,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                          ctypes.POINTER(Raster), ctypes.POINTER(_u64p), _u64p]),
    "bf_contour_free": (None, [_u64p]),
    "bf_contour_release": (None, [ctypes.c_int]),
    "bf_contour_polygons": (ctypes.c_int, [ctypes.POINTER(Raster), _u64p, ctypes.c_uint32,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, _u64p,
                                           ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]),
    "bf_contour_free_polygons": (None, [ctypes.POINTER(ctypes.c_double)]),
    "bf_contour_config": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.POINTER(ctypes.c_double), _u32p, _u32p,
                                         ctypes.POINTER(ctypes.c_double)]),
    "bf_mercator": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]),
    "bf_geometry_create": (ctypes.c_int, [ctypes.c_uint32, _u64p, ctypes.c_void_p, _u32p,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "bf_geometry_destroy": (None, [ctypes.c_void_p]),
    "bf_isochrone_polygons": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, _u32p, _u32p,
                                             ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                             _u64p, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                             ctypes.c_void_p]),
    "bf_tile_emit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                    ctypes.POINTER(TileColumns), _u64p]),
    "bf_tile_emit_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                           ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                           ctypes.c_int, ctypes.c_void_p,
                                           ctypes.POINTER(TileColumns), _u64p]),
    "bf_tile_release": (None, [ctypes.c_int]),
    "bf_last_error": (ctypes.c_char_p, []),
}

_lib = None


def load(path=LIB_PATH):
    """Load the native library (raises OSError if it is missing)."""
    global _lib
    if _lib is None:
        if not pathlib.Path(path).exists():
            raise OSError("native engine %s is missing: run __graft_entry__.build()" % path)
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class BfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("bf status %d: %s" % (status, msg))
        self.status = status


def _check(rc):
    if rc != BF_OK:
        raise BfError(rc, load().bf_last_error().decode(errors="replace"))


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _ptr(a, t=_u32p):
    return a.ctypes.data_as(t)


class Graph:
    """A CCH resident on the GPU (owns a bf_graph handle)."""

    def __init__(self, n_nodes, up_off, up_tgt, up_w, down_off, down_tgt, down_w, device=0,
                 engine=ENGINE_AUTO, k_lanes=0, subtree_nodes=0, hbm_budget=0, reverse=False,
                 up_len=None, down_len=None):
        """up_len / down_len (optional): length-along-time weight per CCH edge,
        INF exactly where the time weight is; they make a two-channel graph."""
        lib = load()
        self._keep = [np.ascontiguousarray(up_off, dtype=np.uint64), _u32(up_tgt), _u32(up_w),
                      np.ascontiguousarray(down_off, dtype=np.uint64), _u32(down_tgt),
                      _u32(down_w)]
        uo, ut, uw, do, dt, dw = self._keep
        csr = CchCsr(n_nodes, 0, _ptr(uo, _u64p), _ptr(ut), _ptr(uw), _ptr(do, _u64p), _ptr(dt),
                     _ptr(dw))
        cfg = Config(device, engine, k_lanes, FLAG_REVERSE if reverse else 0, hbm_budget,
                     subtree_nodes, 0)
        h = ctypes.c_void_p()
        if up_len is not None or down_len is not None:
            ul, dl = _u32(up_len if up_len is not None else []), _u32(
                down_len if down_len is not None else [])
            _check(lib.bf_graph_create_2ch(ctypes.byref(csr), _ptr(ul), _ptr(dl),
                                           ctypes.byref(cfg), ctypes.byref(h)))
        else:
            _check(lib.bf_graph_create(ctypes.byref(csr), ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = None  # the library copied what it needs
        self.n = n_nodes

    @classmethod
    def from_cch(cls, cch, **kw):
        return cls(cch["n"], cch["up_off"], cch["up_tgt"], cch["up_w"], cch["down_off"],
                   cch["down_tgt"], cch["down_w"], **kw)

    def close(self):
        if getattr(self, "_h", None):
            load().bf_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def info(self):
        i = GraphInfo()
        _check(load().bf_graph_info_get(self._h, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in i._fields_}

    def set_engine(self, engine, k_lanes=0):
        _check(load().bf_graph_set_engine(self._h, engine, k_lanes))

    def autotune(self, d_src, S, d_tgt, T, reps=2):
        """Time candidate tunables on a device-resident sample; keeps the best."""
        t = Tune()
        _check(load().bf_autotune(self._h, ctypes.c_void_p(d_src), S, ctypes.c_void_p(d_tgt), T,
                                  reps, ctypes.byref(t)))
        return t.as_dict()

    def set_tune(self, threads_per_block=128, edges_per_item=16, graph_capture=1,
                 lanes_per_wave=0, isochrone_lanes=1024, small_level_rows=64,
                 small_level_edges=8, overlap_levels=1, isochrone_16bit=1, overlap_upward=1,
                 mapped_output=1, hub_l2_mb=48, device_schedule=1, persistent_sweep=1,
                 staged_levels=0):
        t = Tune(threads_per_block, edges_per_item, graph_capture, lanes_per_wave, 0.0, 0,
                 isochrone_lanes, small_level_rows, small_level_edges, overlap_levels,
                 isochrone_16bit, overlap_upward, mapped_output, hub_l2_mb, device_schedule,
                 persistent_sweep, staged_levels)
        _check(load().bf_set_tune(self._h, ctypes.byref(t)))

    def get_tune(self):
        t = Tune()
        _check(load().bf_get_tune(self._h, ctypes.byref(t)))
        return t.as_dict()

    def autotune_isochrones(self, d_orig, d_thr, n, reps=2):
        """Time bulk-isochrone candidates on a device-resident sample; keeps the best."""
        t = Tune()
        _check(load().bf_autotune_isochrones(self._h, ctypes.c_void_p(d_orig),
                                             ctypes.c_void_p(d_thr), n, reps, ctypes.byref(t)))
        return t.as_dict()

    def schedule_levels(self):
        """(items, edges, rows) per level of the last restricted matrix schedule."""
        cap = self.info()["n_levels"]
        a = [np.zeros(cap, np.uint64) for _ in range(3)]
        L = ctypes.c_uint32()
        _check(load().bf_schedule_levels(self._h, cap, _ptr(a[0], _u64p), _ptr(a[1], _u64p),
                                         _ptr(a[2], _u64p), ctypes.byref(L)))
        return [x[:L.value] for x in a]

    def tune_save(self, path):
        _check(load().bf_tune_save(self._h, str(path).encode()))

    def tune_load(self, path):
        _check(load().bf_tune_load(self._h, str(path).encode()))

    def query_batch(self, sources, threshold=INF):
        s = _u32(sources)
        out = np.empty((len(s), self.n), dtype=np.uint32)
        _check(load().bf_query_batch(self._h, _ptr(s), len(s), threshold, _ptr(out)))
        return out

    def phast_query(self, origin):
        out = np.empty(self.n, dtype=np.uint32)
        _check(load().bf_phast_query(self._h, int(origin), _ptr(out)))
        return out

    def matrix(self, sources, targets, threshold=INF, out=None, stats=False):
        s, t = _u32(sources), _u32(targets)
        if out is None:
            out = np.empty((len(s), len(t)), dtype=np.uint32)
        st = Stats()
        _check(load().bf_matrix(self._h, _ptr(s), len(s), _ptr(t), len(t), threshold, _ptr(out),
                                ctypes.byref(st)))
        return (out, st.as_dict()) if stats else out

    def matrix_device(self, d_src, S, d_tgt, T, d_out, threshold=INF, stream=None):
        """Device-pointer variant: d_* are integer device addresses."""
        st = Stats()
        _check(load().bf_matrix_device(self._h, ctypes.c_void_p(d_src), S, ctypes.c_void_p(d_tgt),
                                       T, threshold, ctypes.c_void_p(d_out),
                                       ctypes.c_void_p(stream or 0), ctypes.byref(st)))
        return st.as_dict()

    def matrix_seeded(self, src_seeds, tgt_seeds, threshold=INF, with_conflicts=False):
        """src_seeds / tgt_seeds: lists of lists of (rank, cost). Returns the
        matrix (conflict cells INF) and, if asked, the conflict cell indices."""
        def pack(sets):
            off = np.zeros(len(sets) + 1, dtype=np.uint64)
            flat = []
            for i, ss in enumerate(sets):
                flat.extend(ss)
                off[i + 1] = len(flat)
            arr = (Seed * max(1, len(flat)))(*[Seed(int(r), int(c)) for r, c in flat])
            return arr, off
        sa, so = pack(src_seeds)
        ta, to = pack(tgt_seeds)
        out = np.empty((len(src_seeds), len(tgt_seeds)), dtype=np.uint32)
        st = Stats()
        cap = len(src_seeds) * len(tgt_seeds)
        conf = np.empty(max(1, cap), dtype=np.uint64)
        nconf = ctypes.c_uint64()
        _check(load().bf_matrix_seeded(self._h, sa, _ptr(so, _u64p), len(src_seeds), ta,
                                       _ptr(to, _u64p), len(tgt_seeds), threshold, _ptr(out),
                                       _ptr(conf, _u64p), cap, ctypes.byref(nconf),
                                       ctypes.byref(st)))
        if with_conflicts:
            return out, conf[:min(cap, nconf.value)].copy()
        return out

    def phast_bounded_seeded(self, seeds, threshold):
        arr = (Seed * max(1, len(seeds)))(*[Seed(int(r), int(c)) for r, c in seeds])
        cap = self.n
        rk = np.empty(cap, dtype=np.uint32)
        ds = np.empty(cap, dtype=np.uint32)
        cnt = ctypes.c_uint64()
        _check(load().bf_phast_bounded_seeded(self._h, arr, len(seeds), threshold, _ptr(rk),
                                              _ptr(ds), cap, ctypes.byref(cnt)))
        c = cnt.value
        return rk[:c].copy(), ds[:c].copy()

    @staticmethod
    def _pack2(sets):
        off = np.zeros(len(sets) + 1, dtype=np.uint64)
        flat = []
        for i, ss in enumerate(sets):
            flat.extend(ss)
            off[i + 1] = len(flat)
        arr = (Seed2 * max(1, len(flat)))(*[Seed2(int(r), int(c), int(ln)) for r, c, ln in flat])
        return arr, off

    def matrix_seeded_2ch(self, src_seeds, tgt_seeds, threshold=INF, with_conflicts=False):
        """Seed sets of (rank, cost, len). Returns (time, length) matrices
        (conflict cells INF) and, if asked, the conflict cell indices."""
        sa, so = self._pack2(src_seeds)
        ta, to = self._pack2(tgt_seeds)
        S, T = len(src_seeds), len(tgt_seeds)
        ot = np.empty((S, T), dtype=np.uint32)
        ol = np.empty((S, T), dtype=np.uint32)
        st = Stats()
        cap = S * T
        conf = np.empty(max(1, cap), dtype=np.uint64)
        nconf = ctypes.c_uint64()
        _check(load().bf_matrix_seeded_2ch(self._h, sa, _ptr(so, _u64p), S, ta, _ptr(to, _u64p),
                                           T, threshold, _ptr(ot), _ptr(ol), _ptr(conf, _u64p),
                                           cap, ctypes.byref(nconf), ctypes.byref(st)))
        if with_conflicts:
            return ot, ol, conf[:min(cap, nconf.value)].copy()
        return ot, ol

    def phast_bounded_seeded_2ch(self, seeds, threshold):
        """Settled (ranks, times, lengths) with time <= threshold, ascending rank."""
        arr, _ = self._pack2([seeds])
        cap = self.n
        rk = np.empty(cap, dtype=np.uint32)
        tm = np.empty(cap, dtype=np.uint32)
        ln = np.empty(cap, dtype=np.uint32)
        cnt = ctypes.c_uint64()
        _check(load().bf_phast_bounded_seeded_2ch(self._h, arr, len(seeds), threshold, _ptr(rk),
                                                  _ptr(tm), _ptr(ln), cap, ctypes.byref(cnt)))
        c = cnt.value
        return rk[:c].copy(), tm[:c].copy(), ln[:c].copy()

    def isochrone_settled(self, origins, thresholds, stats=False):
        """bf_isochrone_settled: per origin (ranks, dists) within its
        threshold, ranks ascending (the bounded single query's output)."""
        o, t = _u32(origins), _u32(thresholds)
        off = np.zeros(len(o) + 1, np.uint64)
        r, d = _u32p(), _u32p()
        st = Stats()
        _check(load().bf_isochrone_settled(self._h, _ptr(o), _ptr(t), len(o), _ptr(off, _u64p),
                                           ctypes.byref(r), ctypes.byref(d), ctypes.byref(st)))
        try:
            total = int(off[-1])
            ranks = np.ctypeslib.as_array(r, shape=(max(total, 1),))[:total].copy()
            dists = np.ctypeslib.as_array(d, shape=(max(total, 1),))[:total].copy()
        finally:
            load().bf_settled_free(r)
            load().bf_settled_free(d)
        out = [(ranks[off[i]:off[i + 1]], dists[off[i]:off[i + 1]]) for i in range(len(o))]
        return (out, st.as_dict()) if stats else out

    def isochrone_bitsets(self, origins, thresholds, stats=False, out=None):
        """out: optional (bits, counts) arrays to fill (e.g. page-locked)."""
        o, t = _u32(origins), _u32(thresholds)
        words = (self.n + 63) // 64
        if out is None:
            bits = np.empty((len(o), words), dtype=np.uint64)
            counts = np.empty(len(o), dtype=np.uint64)
        else:
            bits, counts = out
            assert bits.shape == (len(o), words) and bits.dtype == np.uint64
            assert counts.shape == (len(o),) and counts.dtype == np.uint64
        st = Stats()
        _check(load().bf_isochrone_bitsets(self._h, _ptr(o), _ptr(t), len(o), _ptr(bits, _u64p),
                                           _ptr(counts, _u64p), ctypes.byref(st)))
        return (bits, counts, st.as_dict()) if stats else (bits, counts)

    def isochrone_bitsets_device(self, d_orig, d_thr, n, d_bits, d_counts, stream=None):
        """Device-pointer variant: d_* are integer device addresses."""
        st = Stats()
        _check(load().bf_isochrone_bitsets_device(
            self._h, ctypes.c_void_p(d_orig), ctypes.c_void_p(d_thr), n, ctypes.c_void_p(d_bits),
            ctypes.c_void_p(d_counts), ctypes.c_void_p(stream or 0), ctypes.byref(st)))
        return st.as_dict()


class Server:
    """Continuous-batching serving loop (bf_server_*). Output buffers of
    submitted requests are kept alive here until their completion is polled."""

    def __init__(self, graph, hbm_budget=0, max_inflight=0, max_queue=0, timeout_ms=0, slots=0):
        self.graph = graph
        cfg = ServerCfg(hbm_budget, max_inflight, max_queue, timeout_ms, slots)
        h = ctypes.c_void_p()
        _check(load().bf_server_create(graph.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._live = {}

    def _submit(self, kind, src, tgt, threshold, out, tag):
        req = Request(kind, threshold, _ptr(src), len(src),
                      _ptr(tgt) if tgt is not None else None,
                      len(tgt) if tgt is not None else 0, out.ctypes.data, tag)
        t = ctypes.c_uint64()
        _check(load().bf_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        self._live[t.value] = (src, tgt, out)
        return t.value

    def submit_matrix(self, sources, targets, threshold=INF, tag=0):
        s, t = _u32(sources), _u32(targets)
        out = np.empty((len(s), len(t)), dtype=np.uint32)
        return self._submit(REQ_MATRIX, s, t, threshold, out, tag), out

    def submit_isochrone(self, origin, threshold, tag=0):
        s = _u32([origin])
        out = np.empty((self.graph.n + 63) // 64, dtype=np.uint64)
        return self._submit(REQ_ISOCHRONE, s, None, threshold, out, tag), out

    def poll(self, wait_ms=100, cap=256):
        buf = (Completion * cap)()
        n = ctypes.c_uint32()
        _check(load().bf_server_poll(self._h, buf, cap, wait_ms, ctypes.byref(n)))
        res = []
        for i in range(n.value):
            c = buf[i]
            self._live.pop(c.ticket, None)
            res.append({f: getattr(c, f) for f, _ in c._fields_})
        return res

    def cancel(self, ticket):
        return load().bf_server_cancel(self._h, ticket)

    def close(self):
        if getattr(self, "_h", None):
            load().bf_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Cch:
    """A rank-space CCH topology on the GPU for customization (owns a bf_cch).

    Mirrors the reference's CchTopo (formats/cch_topo.rs:250-290): UP edges
    u -> v (v > u) and DOWN edges u -> v (v < u) as two CSRs with targets
    ascending per node, optional shortcut flags and contraction middles."""

    def __init__(self, n_nodes, up_off, up_tgt, down_off, down_tgt, up_short=None,
                 down_short=None, up_mid=None, down_mid=None, device=0, search_targets=False):
        lib = load()
        self._keep = [np.ascontiguousarray(up_off, dtype=np.uint64), _u32(up_tgt),
                      np.ascontiguousarray(down_off, dtype=np.uint64), _u32(down_tgt)]
        self.nu, self.nd = len(self._keep[1]), len(self._keep[3])
        t = CchTopo(n_nodes=int(n_nodes), flags=CCH_SEARCH_TARGETS if search_targets else 0)
        t.up_offsets, t.up_targets = _ptr(self._keep[0], _u64p), _ptr(self._keep[1])
        t.down_offsets, t.down_targets = _ptr(self._keep[2], _u64p), _ptr(self._keep[3])
        for name, arr, dt in (("up_is_shortcut", up_short, np.uint8),
                              ("down_is_shortcut", down_short, np.uint8),
                              ("up_middle", up_mid, np.uint32),
                              ("down_middle", down_mid, np.uint32)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dtype=dt)
                self._keep.append(a)
                setattr(t, name, a.ctypes.data if dt == np.uint8 else _ptr(a))
        h = ctypes.c_void_p()
        _check(lib.bf_cch_create(ctypes.byref(t), int(device), ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_oracle_topo(cls, t, with_short=True, device=0, search_targets=False):
        """From an oracle.CchTopo (same field meaning)."""
        return cls(t.n, t.up_off, t.up_tgt, t.down_off, t.down_tgt,
                   t.up_short if with_short else None, t.down_short if with_short else None,
                   t.up_mid, t.down_mid, device=device, search_targets=search_targets)

    def close(self):
        if getattr(self, "_h", None):
            load().bf_cch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        st = CchStats()
        _check(load().bf_cch_info(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in CchStats._fields_}

    def relax(self, up_w, down_w, up_mid, down_mid):
        """triangle_relax_parallel: returns (up_w, down_w, up_mid, down_mid)."""
        uw, dw, um, dm = (_u32(x).copy() for x in (up_w, down_w, up_mid, down_mid))
        _check(load().bf_cch_relax(self._h, _ptr(uw), _ptr(dw), _ptr(um), _ptr(dm)))
        return uw, dw, um, dm

    def customize(self, orig_up, orig_down, out=None):
        """bottom_up_customize + triangle_relax_parallel: returns
        (up_w, down_w, up_mid, down_mid), written into `out` (four u32 arrays
        of the UP, DOWN, UP, DOWN edge counts) when given."""
        ou, od = _u32(orig_up), _u32(orig_down)
        if out is None:
            uw, dw = np.empty(self.nu, np.uint32), np.empty(self.nd, np.uint32)
            um, dm = np.empty(self.nu, np.uint32), np.empty(self.nd, np.uint32)
        else:
            uw, dw, um, dm = out
            for a, k in zip(out, (self.nu, self.nd, self.nu, self.nd)):
                if a.dtype != np.uint32 or len(a) != k or not a.flags.c_contiguous:
                    raise ValueError("out: four contiguous u32 arrays of the edge counts")
        _check(load().bf_cch_customize(self._h, _ptr(ou), _ptr(od), _ptr(uw), _ptr(dw), _ptr(um),
                                       _ptr(dm)))
        return uw, dw, um, dm

    def relax_lex(self, up_t, down_t, up_len, down_len, up_mid, down_mid):
        """triangle_relax_lex_parallel: returns (up_t, down_t, up_mid, down_mid)."""
        ut, dt, um, dm = (_u32(x).copy() for x in (up_t, down_t, up_mid, down_mid))
        ul, dl = _u32(up_len), _u32(down_len)
        _check(load().bf_cch_relax_lex(self._h, _ptr(ut), _ptr(dt), _ptr(ul), _ptr(dl), _ptr(um),
                                       _ptr(dm)))
        return ut, dt, um, dm

    def bottom_up(self, orig_up, orig_down, up_mid=None, down_mid=None):
        """bottom_up_with_external_middles (the topology's middles when None):
        returns (up_w, down_w)."""
        ou, od = _u32(orig_up), _u32(orig_down)
        um = None if up_mid is None else _u32(up_mid)
        dm = None if down_mid is None else _u32(down_mid)
        uw, dw = np.empty(self.nu, np.uint32), np.empty(self.nd, np.uint32)
        _check(load().bf_cch_bottom_up(self._h, _ptr(ou), _ptr(od),
                                       None if um is None else _ptr(um),
                                       None if dm is None else _ptr(dm), _ptr(uw), _ptr(dw)))
        return uw, dw


def contour_rasters_flat(xy, seg_pt, iso_seg, cell_m, dilation, erosion, has_anchor=None,
                         anchor_xy=None, device=0):
    """bf_contour_rasters on flat arrays: xy (n, 2) Mercator points, seg_pt
    (segments + 1) and iso_seg (isochrones + 1) offsets, cell_m per isochrone,
    optional has_anchor (u8) and anchor_xy (isochrones, 2). Returns
    (rasters, words)."""
    lib = load()
    xy = np.ascontiguousarray(xy, np.float64)
    seg_pt = np.ascontiguousarray(seg_pt, np.uint64)
    iso_seg = np.ascontiguousarray(iso_seg, np.uint64)
    n = len(iso_seg) - 1
    cell = np.ascontiguousarray(cell_m, np.float64)
    has = None if has_anchor is None else np.ascontiguousarray(has_anchor, np.uint8)
    anc = None if anchor_xy is None else np.ascontiguousarray(anchor_xy, np.float64)
    ras = (Raster * max(n, 1))()
    nw = ctypes.c_uint64(0)
    out = _u64p()
    _check(lib.bf_contour_rasters(xy.ctypes.data, _ptr(seg_pt, _u64p), _ptr(iso_seg, _u64p), n,
                                  cell.ctypes.data, None if has is None else has.ctypes.data,
                                  None if anc is None else anc.ctypes.data, int(dilation),
                                  int(erosion), int(device), ras, ctypes.byref(out),
                                  ctypes.byref(nw)))
    try:
        words = np.ctypeslib.as_array(out, shape=(max(int(nw.value), 1),)).copy() if nw.value \
            else np.zeros(1, np.uint64)
    finally:
        lib.bf_contour_free(out)
    return [ras[k] for k in range(n)], words


def raster_cells(r, words):
    """The set cells of one raster as (col, row) rows ascending by row, col."""
    if r.height == 0:
        return np.zeros((0, 2), np.int32)
    w = words[r.word_offset:r.word_offset + r.height * r.width_words].reshape(r.height,
                                                                               r.width_words)
    bits = np.unpackbits(w.view(np.uint8).reshape(r.height, -1), axis=1, bitorder="little")
    rr, cc = np.nonzero(bits)
    return np.stack([cc + r.col0, rr + r.row0], axis=1).astype(np.int32)


def contour_rasters(isochrones, dilation, erosion, device=0):
    """bf_contour_rasters for a list of isochrones, each a dict with
    "segments" (list of (n, 2) float64 arrays of Mercator x, y), "cell_m" and
    optionally "anchor" (x, y). Returns per isochrone (cells, origin): the
    closed cells as (col, row) rows ascending by row then column, and the
    grid origin (x, y)."""
    pts, seg_pt, iso_seg = [], [0], [0]
    for iso in isochrones:
        for seg in iso["segments"]:
            a = np.asarray(seg, np.float64).reshape(-1, 2)
            pts.append(a)
            seg_pt.append(seg_pt[-1] + len(a))
        iso_seg.append(len(seg_pt) - 1)
    xy = np.concatenate(pts) if pts else np.zeros((0, 2))
    has = np.asarray([i.get("anchor") is not None for i in isochrones], np.uint8)
    anc = np.asarray([i.get("anchor") or (0.0, 0.0) for i in isochrones], np.float64).reshape(-1, 2)
    ras, words = contour_rasters_flat(xy, seg_pt, iso_seg, [i["cell_m"] for i in isochrones],
                                      dilation, erosion, has, anc, device)
    return [(raster_cells(r, words), (r.origin_x, r.origin_y)) for r in ras]


def contour_polygons(rasters, words, cell_m, simplify_m, has_anchor=None, anchor_xy=None):
    """bf_contour_polygons on the output of contour_rasters_flat: one
    (lon, lat) ring per isochrone."""
    lib = load()
    n = len(rasters)
    ras = (Raster * max(n, 1))(*rasters)
    words = np.ascontiguousarray(words, np.uint64)
    cell = np.ascontiguousarray(cell_m, np.float64)
    simp = np.ascontiguousarray(simplify_m, np.float64)
    has = None if has_anchor is None else np.ascontiguousarray(has_anchor, np.uint8)
    anc = None if anchor_xy is None else np.ascontiguousarray(anchor_xy, np.float64)
    off = np.zeros(n + 1, np.uint64)
    out = ctypes.POINTER(ctypes.c_double)()
    _check(lib.bf_contour_polygons(ras, _ptr(words, _u64p), n, cell.ctypes.data, simp.ctypes.data,
                                   None if has is None else has.ctypes.data,
                                   None if anc is None else anc.ctypes.data, _ptr(off, _u64p),
                                   ctypes.byref(out)))
    try:
        total = int(off[-1])
        flat = np.ctypeslib.as_array(out, shape=(max(2 * total, 1),))[:2 * total].copy()
    finally:
        lib.bf_contour_free_polygons(out)
    return [flat[2 * int(off[k]):2 * int(off[k + 1])].reshape(-1, 2) for k in range(n)]


def contour_config(mode, threshold_s):
    """bf_contour_config: (cell_m, dilation, erosion, simplify_m)."""
    c, s = ctypes.c_double(), ctypes.c_double()
    d, e = ctypes.c_uint32(), ctypes.c_uint32()
    _check(load().bf_contour_config(int(mode), int(threshold_s), ctypes.byref(c), ctypes.byref(d),
                                    ctypes.byref(e), ctypes.byref(s)))
    return c.value, d.value, e.value, s.value


def mercator(lat_lon_e7):
    """bf_mercator: (n, 2) (lat_e7, lon_e7) -> (n, 2) (x, y) metres."""
    p = np.ascontiguousarray(lat_lon_e7, np.int32).reshape(-1, 2)
    out = np.empty((len(p), 2), np.float64)
    _check(load().bf_mercator(len(p), p.ctypes.data, out.ctypes.data))
    return out


class Geometry:
    """Road polylines per rank for bf_isochrone_polygons (owns a bf_geometry)."""

    def __init__(self, poly_off, poly_e7, node_w):
        off = np.ascontiguousarray(poly_off, np.uint64)
        pts = np.ascontiguousarray(poly_e7, np.int32).reshape(-1, 2)
        w = _u32(node_w)
        h = ctypes.c_void_p()
        _check(load().bf_geometry_create(len(off) - 1, _ptr(off, _u64p), pts.ctypes.data, _ptr(w),
                                         ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().bf_geometry_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def isochrone_polygons(graph, geometry, origins, thresholds, tier_thresholds=None, mode=MODE_CAR):
    """bf_isochrone_polygons: one (lon, lat) ring per origin and the phase
    times (settled, segments, rasters, polygons) in ms."""
    lib = load()
    o, t = _u32(origins), _u32(thresholds)
    tt = None if tier_thresholds is None else _u32(tier_thresholds)
    off = np.zeros(len(o) + 1, np.uint64)
    out = ctypes.POINTER(ctypes.c_double)()
    ph = np.zeros(4)
    _check(lib.bf_isochrone_polygons(graph._h, geometry._h, _ptr(o), _ptr(t),
                                     None if tt is None else tt.ctypes.data, len(o), int(mode),
                                     _ptr(off, _u64p), ctypes.byref(out), ph.ctypes.data))
    try:
        total = int(off[-1])
        flat = np.ctypeslib.as_array(out, shape=(max(2 * total, 1),))[:2 * total].copy()
    finally:
        lib.bf_contour_free_polygons(out)
    return [flat[2 * int(off[k]):2 * int(off[k + 1])].reshape(-1, 2) for k in range(len(o))], ph


def _mask_csr(mask):
    if mask is None:
        return None, None, 0
    if isinstance(mask, tuple):
        off, flat = np.ascontiguousarray(mask[0], np.uint64), np.ascontiguousarray(mask[1], np.uint32)
    else:
        off = np.zeros(len(mask) + 1, np.uint64)
        off[1:] = np.cumsum([len(m) for m in mask]) if len(mask) else []
        flat = np.asarray([v for m in mask for v in m], np.uint32)
    return off, (flat if len(flat) else np.zeros(1, np.uint32)), len(off) - 1


def tile_emit(matrix, n_src, n_dst, src_orig, dst_orig, threshold=INF, mask=None, lat=None,
              sparse=False, device=0, out=None):
    """bf_tile_emit on host arrays: (source_idx, target_idx, duration_ms,
    distance_m) of a row-major n_src x n_dst block. `mask`: list (by original
    source index) of sorted original destination indices, or (offsets, flat).
    `out`: optional four u32 arrays of n_src * n_dst values to write into."""
    lib = load()
    m = np.ascontiguousarray(np.asarray(matrix).reshape(-1), np.uint32)
    so, do = _u32(src_orig), _u32(dst_orig)
    la = None if lat is None else np.ascontiguousarray(np.asarray(lat).reshape(-1), np.uint32)
    moff, mflat, n_mask = _mask_csr(mask)
    cap = max(1, n_src * n_dst)
    cols = out if out is not None else [np.empty(cap, np.uint32) for _ in range(4)]
    tc = TileColumns(*[c.ctypes.data for c in cols])
    rows = ctypes.c_uint64(0)
    _check(lib.bf_tile_emit(m.ctypes.data, None if la is None else la.ctypes.data, n_src, n_dst,
                            so.ctypes.data, do.ctypes.data, threshold,
                            None if moff is None else moff.ctypes.data,
                            None if mflat is None else mflat.ctypes.data, n_mask, int(sparse),
                            device, ctypes.byref(tc), ctypes.byref(rows)))
    k = rows.value
    return tuple(c[:k] for c in cols)


def tile_emit_device(d_matrix, n_src, n_dst, d_src_orig, d_dst_orig, d_cols, threshold=INF,
                     d_mask_off=None, d_mask=None, n_mask_src=0, n_mask=0, d_lat=None,
                     sparse=False, device=0, stream=None):
    """bf_tile_emit_device on device addresses (integers); d_cols: four device
    addresses of n_src * n_dst u32 each. Returns the rows written."""
    tc = TileColumns(*d_cols)
    rows = ctypes.c_uint64(0)
    _check(load().bf_tile_emit_device(d_matrix, d_lat, n_src, n_dst, d_src_orig, d_dst_orig,
                                      threshold, d_mask_off, d_mask, n_mask_src, n_mask,
                                      int(sparse), device, stream, ctypes.byref(tc),
                                      ctypes.byref(rows)))
    return rows.value
