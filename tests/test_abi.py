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
