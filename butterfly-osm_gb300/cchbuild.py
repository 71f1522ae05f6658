"""Python binding of the host CCH build pipeline (cch/bf_cch.h).

build_synthetic(kind, rows, cols, seed) returns the edge-based graph and the
rank-aligned INF-filtered CCH flats as numpy arrays. The two synthetic
families restate the workloads the engine is measured on:

  KIND_GRID     100 x 100 jittered 4-neighbour grid, 5% roads removed, 10%
                one-way, speed classes 30/50/90 km/h at 80/15/5%, turn
                penalties uniform 0-50 ds, 2% forbidden turns.
  KIND_COUNTRY  2000 x 2500 jittered lattice with a 3-level road hierarchy:
                motorway lines every 80 (120 km/h), arterial lines every 10
                (70 km/h), 9 x 9 local-street cells (random spanning tree +
                loops, 30-50 km/h) joined to the arterials on two sides.
"""
import ctypes
import pathlib

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libbf_cch.so"
KIND_GRID, KIND_COUNTRY = 0, 1


class _Params(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("rows", ctypes.c_uint32), ("cols", ctypes.c_uint32),
                ("spacing_cm", ctypes.c_uint32), ("jitter_cm", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("seed", ctypes.c_uint64)]


class _Ebg(ctypes.Structure):
    _fields_ = [("n_intersections", ctypes.c_uint32), ("n_states", ctypes.c_uint32),
                ("n_roads", ctypes.c_uint64), ("n_arcs", ctypes.c_uint64),
                ("arc_off", ctypes.c_void_p), ("arc_dst", ctypes.c_void_p),
                ("arc_w", ctypes.c_void_p), ("node_weight", ctypes.c_void_p),
                ("state_tail", ctypes.c_void_p), ("state_head", ctypes.c_void_p),
                ("state_class", ctypes.c_void_p), ("ix", ctypes.c_void_p),
                ("iy", ctypes.c_void_p)]


class _Cch(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("n_up", ctypes.c_uint64), ("n_down", ctypes.c_uint64),
                ("n_chordal", ctypes.c_uint64),
                ("up_off", ctypes.c_void_p), ("up_tgt", ctypes.c_void_p),
                ("up_w", ctypes.c_void_p), ("down_off", ctypes.c_void_p),
                ("down_tgt", ctypes.c_void_p), ("down_w", ctypes.c_void_p),
                ("rank_to_state", ctypes.c_void_p), ("state_to_rank", ctypes.c_void_p),
                ("t_generate_s", ctypes.c_double), ("t_order_s", ctypes.c_double),
                ("t_contract_s", ctypes.c_double), ("t_customize_s", ctypes.c_double)]


class _Topo(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("n_edges", ctypes.c_uint64), ("off", ctypes.c_void_p), ("tgt", ctypes.c_void_p),
                ("orig_up", ctypes.c_void_p), ("orig_down", ctypes.c_void_p),
                ("cust_up", ctypes.c_void_p), ("cust_down", ctypes.c_void_p)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise OSError("%s is missing: run __graft_entry__.build()" % LIB_PATH)
        lib = ctypes.CDLL(str(LIB_PATH))
        lib.bfc_build_synthetic.argtypes = [ctypes.POINTER(_Params), ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_void_p)]
        lib.bfc_build_from_arcs.argtypes = [ctypes.c_uint32, ctypes.c_uint64] + \
            [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        lib.bfc_free.argtypes = [ctypes.c_void_p]
        lib.bfc_ebg.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Ebg)]
        lib.bfc_cch.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Cch)]
        lib.bfc_topo.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Topo)]
        lib.bfc_last_error.restype = ctypes.c_char_p
        _lib = lib
    return _lib


def _copy(ptr, count, dtype):
    if count == 0:
        return np.zeros(0, dtype=dtype)
    ct = np.ctypeslib.as_ctypes_type(np.dtype(dtype))
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), shape=(count,)).copy()


def _extract(lib, h, with_topo=False):
    e, c = _Ebg(), _Cch()
    lib.bfc_ebg(h, ctypes.byref(e))
    lib.bfc_cch(h, ctypes.byref(c))
    n = c.n_nodes
    ebg = dict(n=e.n_states, n_intersections=e.n_intersections, n_roads=e.n_roads,
               n_arcs=e.n_arcs,
               arc_off=_copy(e.arc_off, e.n_states + 1, np.uint64),
               arc_dst=_copy(e.arc_dst, e.n_arcs, np.uint32),
               arc_w=_copy(e.arc_w, e.n_arcs, np.uint32))
    if e.n_intersections:
        ebg.update(node_weight=_copy(e.node_weight, e.n_states, np.uint32),
                   state_tail=_copy(e.state_tail, e.n_states, np.uint32),
                   state_head=_copy(e.state_head, e.n_states, np.uint32),
                   state_class=_copy(e.state_class, e.n_states, np.uint8))
    cch = dict(n=n, n_chordal=c.n_chordal,
               up_off=_copy(c.up_off, n + 1, np.uint64),
               up_tgt=_copy(c.up_tgt, c.n_up, np.uint32),
               up_w=_copy(c.up_w, c.n_up, np.uint32),
               down_off=_copy(c.down_off, n + 1, np.uint64),
               down_tgt=_copy(c.down_tgt, c.n_down, np.uint32),
               down_w=_copy(c.down_w, c.n_down, np.uint32),
               rank_to_state=_copy(c.rank_to_state, n, np.uint32),
               state_to_rank=_copy(c.state_to_rank, n, np.uint32),
               times=dict(generate_s=c.t_generate_s, order_s=c.t_order_s,
                          contract_s=c.t_contract_s, customize_s=c.t_customize_s))
    if with_topo:
        t = _Topo()
        lib.bfc_topo(h, ctypes.byref(t))
        m = t.n_edges
        cch["topo"] = dict(off=_copy(t.off, n + 1, np.uint64), tgt=_copy(t.tgt, m, np.uint32),
                           orig_up=_copy(t.orig_up, m, np.uint32),
                           orig_down=_copy(t.orig_down, m, np.uint32),
                           cust_up=_copy(t.cust_up, m, np.uint32),
                           cust_down=_copy(t.cust_down, m, np.uint32))
    return ebg, cch


def build_synthetic(kind, rows, cols, seed=42, threads=0, with_topo=False):
    """Build a synthetic road graph and its CCH; returns (ebg, cch) dicts.
    with_topo adds cch["topo"]: the chordal completion in upper-neighbour form
    with original and customized weights (for customization tests)."""
    lib = load()
    p = _Params(kind, rows, cols, 0, 0, 0, seed)
    h = ctypes.c_void_p()
    if lib.bfc_build_synthetic(ctypes.byref(p), threads, ctypes.byref(h)) != 0:
        raise RuntimeError("bfc_build_synthetic: " + lib.bfc_last_error().decode())
    try:
        return _extract(lib, h, with_topo)
    finally:
        lib.bfc_free(h)


def build_from_arcs(n_states, arc_src, arc_dst, arc_w, sx, sy, threads=0):
    """CCH of a caller-supplied edge-based graph; returns (ebg, cch)."""
    lib = load()
    s = np.ascontiguousarray(arc_src, dtype=np.uint32)
    d = np.ascontiguousarray(arc_dst, dtype=np.uint32)
    w = np.ascontiguousarray(arc_w, dtype=np.uint32)
    x = np.ascontiguousarray(sx, dtype=np.int64)
    y = np.ascontiguousarray(sy, dtype=np.int64)
    h = ctypes.c_void_p()
    if lib.bfc_build_from_arcs(n_states, len(s), s.ctypes.data, d.ctypes.data, w.ctypes.data,
                               x.ctypes.data, y.ctypes.data, threads, ctypes.byref(h)) != 0:
        raise RuntimeError("bfc_build_from_arcs: " + lib.bfc_last_error().decode())
    try:
        return _extract(lib, h)
    finally:
        lib.bfc_free(h)
