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
