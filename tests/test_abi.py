"""The C-ABI library loads and exports every symbol include/*.h declares.

No compute call is made here (these run without a GPU)."""
import ctypes
import pathlib
import re
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(bf_[a-z_0-9]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = _declared()
    for want in ("bf_graph_create", "bf_matrix", "bf_matrix_device", "bf_query_batch",
                 "bf_isochrone_bitsets", "bf_server_create", "bf_last_error"):
        assert want in names


def test_library_exports_every_declared_symbol(built):
    import bfphast
    lib = bfphast.load()
    for name in _declared():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(bfphast.LIB_PATH)],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (bf_[a-z_0-9]+)", out))
    assert _declared() <= exported


def test_python_binding_covers_header(built):
    import bfphast
    assert _declared() == set(bfphast._SIGNATURES)


def test_graph_create_rejects_bad_input_without_gpu(built):
    import bfphast
    lib = bfphast.load()
    h = ctypes.c_void_p()
    rc = lib.bf_graph_create(None, None, ctypes.byref(h))
    assert rc == bfphast.BF_ERR_INVALID
    assert b"null" in lib.bf_last_error()


def test_missing_library_fails_loudly(tmp_path):
    import bfphast
    with pytest.raises(OSError):
        bfphast._lib = None
        try:
            bfphast.load(tmp_path / "nope.so")
        finally:
            bfphast._lib = None


def test_cch_create_rejects_bad_topology(built):
    # host-side validation runs before any device call: targets must ascend
    # strictly, UP targets above their node and DOWN targets below it
    import ctypes
    import numpy as np
    import bfphast
    lib = bfphast.load()
    for up_tgt, down_tgt in (([2, 1], [0]), ([1, 1], [0]), ([0, 2], [0]), ([1, 2], [2])):
        keep = [np.array([0, 2, 2, 2], np.uint64), np.array(up_tgt, np.uint32),
                np.array([0, 0, 1, 1], np.uint64), np.array(down_tgt, np.uint32)]
        t = bfphast.CchTopo(n_nodes=3)
        t.up_offsets = keep[0].ctypes.data_as(bfphast._u64p)
        t.up_targets = keep[1].ctypes.data_as(bfphast._u32p)
        t.down_offsets = keep[2].ctypes.data_as(bfphast._u64p)
        t.down_targets = keep[3].ctypes.data_as(bfphast._u32p)
        h = ctypes.c_void_p()
        assert lib.bf_cch_create(ctypes.byref(t), 0, ctypes.byref(h)) == bfphast.BF_ERR_INVALID
        assert not h.value


def test_contour_layout_without_device(built):
    # the layout pass of bf_contour_rasters runs on the host: grid origins
    # are the oracle's (minimum corner less three cells) with no device call
    import ctypes
    import sys
    import numpy as np
    import bfphast
    sys.path.insert(0, str(__import__("pathlib").Path(__file__).parent))
    import contourgen
    from oracle import oracle as orc
    rng = np.random.default_rng(2)
    segs, _ = contourgen.isochrone(rng, 50)
    m = contourgen.mercator_segments(segs)
    xy = np.ascontiguousarray(np.concatenate(m))
    seg_pt = np.asarray([0] + list(np.cumsum([len(a) for a in m])), np.uint64)
    iso_seg = np.asarray([0, len(m)], np.uint64)
    cell = np.asarray([30.0])
    ras = (bfphast.Raster * 1)()
    nw = ctypes.c_uint64(0)
    rc = bfphast.load().bf_contour_rasters(xy.ctypes.data, seg_pt.ctypes.data_as(bfphast._u64p),
                                           iso_seg.ctypes.data_as(bfphast._u64p), 1,
                                           cell.ctypes.data, None, None, 2, 2, 0, ras, None,
                                           ctypes.byref(nw))
    assert rc == bfphast.BF_OK and nw.value > 0
    _, grid = orc.sparse_closed(segs, 30.0, 2, 2)
    assert (ras[0].origin_x, ras[0].origin_y) == tuple(grid)
    assert ras[0].width_words * ras[0].height == nw.value


def test_contour_and_customization_input_errors(built):
    # host-side validation: bad offsets, non-positive cell sizes, unknown
    # topology flags are BF_ERR_INVALID without touching a device
    import ctypes
    import numpy as np
    import bfphast
    lib = bfphast.load()
    xy = np.zeros((4, 2))
    ras = (bfphast.Raster * 2)()
    nw = ctypes.c_uint64(0)
    for seg_pt, iso_seg, cell in (([0, 2, 1, 4], [0, 3], [30.0]),   # decreasing seg_pt
                                  ([0, 2, 4], [0, 2, 1], [30.0, 30.0]),  # decreasing iso_seg
                                  ([0, 2, 4], [0, 2], [0.0])):       # cell size 0
        sp = np.asarray(seg_pt, np.uint64)
        isg = np.asarray(iso_seg, np.uint64)
        c = np.asarray(cell)
        rc = lib.bf_contour_rasters(xy.ctypes.data, sp.ctypes.data_as(bfphast._u64p),
                                    isg.ctypes.data_as(bfphast._u64p), len(isg) - 1,
                                    c.ctypes.data, None, None, 2, 2, 0, ras, None,
                                    ctypes.byref(nw))
        assert rc == bfphast.BF_ERR_INVALID
    keep = [np.array([0, 1, 1], np.uint64), np.array([1], np.uint32),
            np.array([0, 0, 1], np.uint64), np.array([0], np.uint32)]
    t = bfphast.CchTopo(n_nodes=2, flags=8)
    t.up_offsets = keep[0].ctypes.data_as(bfphast._u64p)
    t.up_targets = keep[1].ctypes.data_as(bfphast._u32p)
    t.down_offsets = keep[2].ctypes.data_as(bfphast._u64p)
    t.down_targets = keep[3].ctypes.data_as(bfphast._u32p)
    h = ctypes.c_void_p()
    assert lib.bf_cch_create(ctypes.byref(t), 0, ctypes.byref(h)) == bfphast.BF_ERR_INVALID


def test_tile_polygon_and_geometry_input_errors(built):
    # null arguments and malformed offsets are BF_ERR_INVALID before any
    # device is touched (tile emission, geometry, polygons, settled sets)
    import ctypes
    import numpy as np
    import bfphast
    lib = bfphast.load()
    m = np.zeros(4, np.uint32)
    ids = np.arange(2, dtype=np.uint32)
    cols = [np.zeros(4, np.uint32) for _ in range(4)]
    tc = bfphast.TileColumns(*[c.ctypes.data for c in cols])
    rows = ctypes.c_uint64(0)
    # no output struct / no row count / no matrix for a non-empty block
    assert lib.bf_tile_emit(m.ctypes.data, None, 2, 2, ids.ctypes.data, ids.ctypes.data,
                            bfphast.INF, None, None, 0, 0, 0, None,
                            ctypes.byref(rows)) == bfphast.BF_ERR_INVALID
    assert lib.bf_tile_emit(m.ctypes.data, None, 2, 2, ids.ctypes.data, ids.ctypes.data,
                            bfphast.INF, None, None, 0, 0, 0, ctypes.byref(tc),
                            None) == bfphast.BF_ERR_INVALID
    assert lib.bf_tile_emit(None, None, 2, 2, ids.ctypes.data, ids.ctypes.data, bfphast.INF,
                            None, None, 0, 0, 0, ctypes.byref(tc),
                            ctypes.byref(rows)) == bfphast.BF_ERR_INVALID
    # radius list offsets that decrease
    moff = np.array([0, 2, 1], np.uint64)
    mask = np.array([0, 1], np.uint32)
    assert lib.bf_tile_emit(m.ctypes.data, None, 2, 2, ids.ctypes.data, ids.ctypes.data,
                            bfphast.INF, moff.ctypes.data, mask.ctypes.data, 2, 1, 0,
                            ctypes.byref(tc), ctypes.byref(rows)) == bfphast.BF_ERR_INVALID
    assert b"radius list" in lib.bf_last_error()
    # geometry: decreasing polyline offsets, null output
    off = np.array([0, 2, 1], np.uint64)
    e7 = np.zeros(4, np.int32)
    w = np.ones(2, np.uint32)
    h = ctypes.c_void_p()
    assert lib.bf_geometry_create(2, off.ctypes.data_as(bfphast._u64p), e7.ctypes.data,
                                  w.ctypes.data_as(bfphast._u32p),
                                  ctypes.byref(h)) == bfphast.BF_ERR_INVALID
    assert lib.bf_geometry_create(2, off.ctypes.data_as(bfphast._u64p), e7.ctypes.data,
                                  w.ctypes.data_as(bfphast._u32p), None) == bfphast.BF_ERR_INVALID
    # polygons and settled sets without a graph
    ro = np.zeros(2, np.uint64)
    out = ctypes.POINTER(ctypes.c_double)()
    assert lib.bf_isochrone_polygons(None, None, ids.ctypes.data_as(bfphast._u32p),
                                     ids.ctypes.data_as(bfphast._u32p), None, 1, 0,
                                     ro.ctypes.data_as(bfphast._u64p), ctypes.byref(out),
                                     None) == bfphast.BF_ERR_INVALID
    r, d = ctypes.POINTER(ctypes.c_uint32)(), ctypes.POINTER(ctypes.c_uint32)()
    assert lib.bf_isochrone_settled(None, ids.ctypes.data_as(bfphast._u32p),
                                    ids.ctypes.data_as(bfphast._u32p), 1,
                                    ro.ctypes.data_as(bfphast._u64p), ctypes.byref(r),
                                    ctypes.byref(d), None) == bfphast.BF_ERR_INVALID
    # the tier table and projection are host functions: checked against known values
    c, dl, er, sm = bfphast.contour_config(bfphast.MODE_CAR, 1800)
    assert (c, dl, er, sm) == (60.0, 2, 2, 60.0)


def test_struct_layouts_match_header(built, tmp_path):
    # every public struct of the header against its ctypes mirror: size and
    # the offset of every field, from a C program compiled against the header
    import ctypes
    import shutil
    import subprocess
    import bfphast
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    pairs = {"bf_cch_csr": bfphast.CchCsr, "bf_config": bfphast.Config,
             "bf_graph_info": bfphast.GraphInfo, "bf_stats": bfphast.Stats,
             "bf_tune": bfphast.Tune, "bf_seed": bfphast.Seed, "bf_router": bfphast.Router,
             "bf_server_cfg": bfphast.ServerCfg, "bf_request": bfphast.Request,
             "bf_completion": bfphast.Completion, "bf_cch_topo": bfphast.CchTopo,
             "bf_cch_stats": bfphast.CchStats, "bf_raster": bfphast.Raster,
             "bf_tile_columns": bfphast.TileColumns}
    if hasattr(bfphast, "Seed2"):
        pairs["bf_seed2"] = bfphast.Seed2
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bf_phast.h"',
             'int main(void) {']
    for c, py in pairs.items():
        lines.append(f'  printf("{c} size %zu\\n", sizeof({c}));')
        for name, _ in py._fields_:
            lines.append(f'  printf("{c} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    root = pathlib.Path(__file__).resolve().parents[1]
    r = subprocess.run(["gcc", "-I", str(root / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out.splitlines()}
    for c, py in pairs.items():
        assert got[(c, "size")] == ctypes.sizeof(py), c
        for name, _ in py._fields_:
            assert got[(c, name)] == getattr(py, name).offset, (c, name)
