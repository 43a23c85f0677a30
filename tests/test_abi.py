"""The C ABI library loads and exports every symbol include/diso_gb300.h declares;
argument errors come back as status codes without a GPU."""
import ctypes
import os
import re

import pytest

from helpers import ROOT

HEADER = os.path.join(ROOT, "include", "diso_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*[a-z_0-9 ]+[ \*]+(diso_[a-z_0-9]+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from diso_gb300.build import build

    build()
    from diso_gb300 import _native

    return _native.lib()


def test_header_declares_the_abi():
    names = declared_functions()
    for want in ("diso_create", "diso_destroy", "diso_forward_count", "diso_forward_emit", "diso_backward",
                 "diso_split_quads", "diso_segment_slots", "diso_last_error"):
        assert want in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} missing from libdiso_gb300.so"


def test_bindings_cover_the_header():
    from diso_gb300 import _native

    assert set(declared_functions()) <= set(_native.EXPORTS)


def test_argument_errors_are_status_codes(lib):
    h = ctypes.c_void_p()
    assert lib.diso_create(7, 0, ctypes.byref(h)) == 1
    assert b"unknown method" in lib.diso_last_error()
    assert lib.diso_create(0, 5, ctypes.byref(h)) == 1
    assert lib.diso_create(0, 0, ctypes.byref(h)) == 0 and h.value
    from diso_gb300._native import Counts

    c = Counts()
    # invalid dims are rejected before any CUDA call
    assert lib.diso_forward_count(h, ctypes.c_void_p(16), 0, 4, 4, 0.0, 1.0, ctypes.c_void_p(16), None,
                                  ctypes.byref(c)) == 1
    assert b"grid dims" in lib.diso_last_error()
    assert lib.diso_forward_count(h, None, 4, 4, 4, 0.0, 1.0, ctypes.c_void_p(16), None, ctypes.byref(c)) == 1
    n = ctypes.c_int64(5)
    assert lib.diso_split_quads(h, None, None, 3, None, ctypes.byref(n), None) == 1  # MC extractor
    lib.diso_destroy(h)


def test_segment_slots(lib):
    # cells (n+1)^3, rows cut into 32-cell chunks, the total slot, then two bytes per
    # 4x8x32-cell tile
    assert lib.diso_segment_slots(64, 64, 64) == 65 * 65 * 3 + 1 + (2 * 17 * 9 * 3 + 7) // 8
    assert lib.diso_segment_slots(31, 5, 7) == 32 * 6 * 1 + 1 + (2 * 8 * 1 * 1 + 7) // 8
    assert lib.diso_segment_slots(0, 5, 7) == 0


def test_edge_record_slots(lib):
    # adjoints (8 values per edge, in 8-byte slots), then for DMC 4 int32 patch ids per
    # edge, then the packed edge locations, then for DMC one byte per vertex
    mc, dmc, f32, f64 = 0, 1, 0, 1
    assert lib.diso_edge_record_slots(mc, f32, 10, 7) == 10 * 4 + 10
    assert lib.diso_edge_record_slots(mc, f64, 10, 7) == 10 * 8 + 10
    assert lib.diso_edge_record_slots(dmc, f32, 10, 7) == 7 * 4 + 7 * 2 + 7 + 2
    assert lib.diso_edge_record_slots(dmc, f64, 9, 7) == 7 * 8 + 7 * 2 + 7 + 2
    assert lib.diso_edge_record_slots(2, f32, 10, 7) == 0
    assert lib.diso_edge_record_slots(mc, f32, -1, 7) == 0


def test_backward_needs_an_aligned_edge_record(lib):
    h = ctypes.c_void_p()
    assert lib.diso_create(1, 0, ctypes.byref(h)) == 0
    p = ctypes.c_void_p(4096)
    args = (h, p, None, 4, 4, 4, 0.0, 1.0, p)
    tail = (1, 0, p, p, None, None)
    assert lib.diso_backward(*args, None, *tail) == 1
    assert b"null edge record" in lib.diso_last_error()
    assert lib.diso_backward(*args, ctypes.c_void_p(4096 + 8), *tail) == 1
    assert b"32-byte aligned" in lib.diso_last_error()
    lib.diso_destroy(h)


def test_recompute_backward_checks_its_arguments(lib):
    h = ctypes.c_void_p()
    assert lib.diso_create(1, 0, ctypes.byref(h)) == 0
    p = ctypes.c_void_p(4096)
    # (ex, sdf, deform, nx, ny, nz, iso, pad, seg, normalize, flags, grad_verts, grad_sdf, grad_deform, stream)
    assert lib.diso_backward_recompute(h, p, None, 4, 4, 4, 0.0, 1.0, None, 1, 0, p, p, None, None) == 1
    assert b"null seg" in lib.diso_last_error()
    assert lib.diso_backward_recompute(h, p, None, 4, 4, 4, 0.0, 1.0, p, 1, 0, None, p, None, None) == 1
    assert b"null grad_verts" in lib.diso_last_error()
    assert lib.diso_backward_recompute(h, p, p, 4, 4, 4, 0.0, 1.0, p, 1, 0, p, p, None, None) == 1
    assert b"without grad_deform" in lib.diso_last_error()
    assert lib.diso_backward_recompute(h, p, None, 0, 4, 4, 0.0, 1.0, p, 1, 0, p, p, None, None) == 1
    assert b"grid dims" in lib.diso_last_error()
    lib.diso_destroy(h)


def test_scan_wait_probe_checks_its_arguments(lib):
    assert lib.diso_scan_wait_probe(None, 16, None) == 1
    h = ctypes.c_void_p()
    assert lib.diso_create(0, 0, ctypes.byref(h)) == 0
    assert lib.diso_scan_wait_probe(h, 0, None) == 1
    assert b"spin limit" in lib.diso_last_error()
    assert lib.diso_scan_wait_probe(h, (1 << 22) + 1, None) == 1
    lib.diso_destroy(h)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from diso_gb300 import _native

    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(RuntimeError, match="missing"):
        _native.lib()


def test_field_entry_points_check_their_arguments(lib):
    import ctypes

    from diso_gb300 import _native as N

    c = N.Counts()
    d = N.SphereFieldDesc()
    assert lib.diso_forward_field(None, None, 4, 4, 4, 0.0, 1.0, None, 1, None, 0, None, 0, None, ctypes.byref(c)) == 1
    assert lib.diso_field_materialize(7, ctypes.byref(d), 4, 4, 4, None, None) == 1
    d.count = 0
    assert lib.diso_field_materialize(0, ctypes.byref(d), 4, 4, 4, None, None) == 1


def test_isovalue_grad_checks_its_arguments(lib):
    h = ctypes.c_void_p()
    assert lib.diso_create(0, 0, ctypes.byref(h)) == 0 and h.value
    out = ctypes.c_void_p(16)
    # rejected before any CUDA call: no extractor, no gradient, no output, bad dims
    assert lib.diso_isovalue_grad(None, ctypes.c_void_p(16), 4, 4, 4, None, out, None) == 1
    assert lib.diso_isovalue_grad(h, None, 4, 4, 4, None, out, None) == 1
    assert lib.diso_isovalue_grad(h, ctypes.c_void_p(16), 4, 4, 4, None, None, None) == 1
    assert b"grad_iso" in lib.diso_last_error()
    assert lib.diso_isovalue_grad(h, ctypes.c_void_p(16), 4, 0, 4, None, out, None) == 1
    assert b"grid dims" in lib.diso_last_error()
    lib.diso_destroy(h)


def _declarations():
    """{name: (return type, [parameter declarations])} from the header."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*([a-z_0-9 ]+?[ \*]+)(diso_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", src, flags=re.M):
        ret, name, params = m.groups()
        ps = [] if params.strip() in ("", "void") else [p.strip() for p in params.split(",")]
        out[name] = (ret.strip(), ps)
    return out


def _c_kind(decl):
    decl = re.sub(r"\b(const|struct)\b", " ", decl)
    if "*" in decl:
        return "pointer"
    return {"int": "int", "unsigned": "uint", "int64_t": "int64", "uint64_t": "int64", "double": "double",
            "void": "void"}[decl.split()[0]]


def _ctypes_kind(t):
    if t is None:
        return "void"
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return "pointer"
    return {ctypes.c_int: "int", ctypes.c_uint: "uint", ctypes.c_int64: "int64", ctypes.c_uint64: "int64",
            ctypes.c_double: "double"}[t]


def test_bindings_match_the_header_signatures():
    # a binding whose argument list differs from the C declaration would pass
    # garbage silently: every parameter's kind (pointer, int, int64, double) and the
    # return kind must agree
    from diso_gb300 import _native

    decls = _declarations()
    assert set(decls) == set(declared_functions())
    for name, (ret, params) in decls.items():
        restype, argtypes = _native.EXPORTS[name]
        assert _ctypes_kind(restype) == _c_kind(ret), (name, "return", ret, restype)
        assert len(argtypes) == len(params), (name, len(argtypes), len(params))
        for i, (p, t) in enumerate(zip(params, argtypes)):
            assert _ctypes_kind(t) == _c_kind(p), (name, i, p, t)
