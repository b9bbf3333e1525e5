"""CPU: the C-ABI library builds, loads, exports every declared symbol, and
rejects bad arguments on the host (no GPU call is made by these checks)."""

import ctypes
import os
import re

import numpy as np
import pytest

from serinv_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "serinv_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sgb_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("sgb_pobtaf", "sgb_pobtasi", "sgb_pobtas"):
        assert s in syms


def test_every_declared_symbol_is_exported(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _lib.exported_symbols(), f"{s} has no ctypes signature"


def test_version_and_strerror(lib):
    assert lib.sgb_version() >= 100
    for code in range(0, 9):
        assert len(lib.sgb_strerror(code)) > 0


def _desc(n=4, b=8, a=2, dtype=_lib.SGB_F64):
    m = _lib.SgbBta()
    m.dtype = dtype
    m.n, m.b, m.a = n, b, a
    # dummy non-null pointers: never dereferenced by the host-side checks
    m.diag = m.lower = m.arrow = m.tip = 0x1000
    return m


def test_workspace_queries(lib):
    m = _desc(n=4, b=64, a=16)
    sz = ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(m), 0, ctypes.byref(sz)) == 0
    assert sz.value >= 32 * 32 * 8
    assert lib.sgb_pobtasi_workspace_size(ctypes.byref(m), 0, ctypes.byref(sz)) == 0
    assert sz.value >= 4 * 64 * 64 * 8
    assert lib.sgb_pobtas_workspace_size(ctypes.byref(m), 16, 0, ctypes.byref(sz)) == 0
    assert sz.value % 256 == 0


@pytest.mark.parametrize("field,value,code", [
    ("dtype", 7, _lib.SGB_ERR_DTYPE),
    ("n", 0, _lib.SGB_ERR_SHAPE),
    ("b", 0, _lib.SGB_ERR_SHAPE),
    ("a", -1, _lib.SGB_ERR_SHAPE),
    ("diag", 0, _lib.SGB_ERR_ARG),
])
def test_bad_descriptor_rejected(lib, field, value, code):
    m = _desc()
    setattr(m, field, value)
    sz = ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(m), 0, ctypes.byref(sz)) == code
    assert lib.sgb_pobtaf(ctypes.byref(m), 1, 0, None, 0, None, None) == code


def test_null_and_workspace_errors(lib):
    assert lib.sgb_pobtaf(None, 1, 0, None, 0, None, None) == _lib.SGB_ERR_ARG
    m = _desc()
    # workspace missing / too small / misaligned: rejected before any launch
    assert lib.sgb_pobtaf(ctypes.byref(m), 1, 0, None, 0, None, None) == _lib.SGB_ERR_WORKSPACE
    assert lib.sgb_pobtasi(ctypes.byref(m), 1, 0, 0x1000, 8, None) == _lib.SGB_ERR_WORKSPACE
    assert lib.sgb_pobtas(ctypes.byref(m), 0x1000, 2, 2, b"N", 0, 0, 0x1001, 1 << 30, None) == \
        _lib.SGB_ERR_WORKSPACE
    assert lib.sgb_pobtas(ctypes.byref(m), 0x1000, 2, 2, b"X", 0, 0, 0x1000, 1 << 30, None) == _lib.SGB_ERR_ARG
    assert lib.sgb_pobtas(ctypes.byref(m), 0x1000, 2, 1, b"N", 0, 0, 0x1000, 1 << 30, None) == \
        _lib.SGB_ERR_SHAPE
    assert lib.sgb_pobtaf(ctypes.byref(m), 1, 9, 0x1000, 1 << 20, None, None) == _lib.SGB_ERR_ARG


def test_permuted_entry_points_host_checks(lib):
    """The buffer= entry points validate on the host before any launch."""
    m = _desc(n=4, b=8, a=2)
    sz = ctypes.c_size_t(0)
    assert lib.sgb_pobtasi_permuted_workspace_size(ctypes.byref(m), 0, ctypes.byref(sz)) == 0
    assert sz.value % 256 == 0 and sz.value >= 4 * 8 * 8 * 8
    mixed = _lib.SGB_PREC_MIXED
    plain = sz.value
    assert lib.sgb_pobtasi_permuted_workspace_size(ctypes.byref(m), mixed, ctypes.byref(sz)) == 0
    assert sz.value > plain  # slice scratch of the mixed form
    m32 = _desc(n=4, b=8, a=2, dtype=_lib.SGB_F32)
    assert lib.sgb_pobtaf_permuted(ctypes.byref(m32), 0x1000, mixed, 0x1000, 1 << 30, None, None) == \
        _lib.SGB_ERR_UNSUPPORTED
    assert lib.sgb_pobtaf_permuted(ctypes.byref(m), None, 0, 0x1000, 1 << 30, None, None) == _lib.SGB_ERR_ARG
    assert lib.sgb_pobtaf_permuted(ctypes.byref(m), 0x1000, 0, None, 0, None, None) == _lib.SGB_ERR_WORKSPACE
    assert lib.sgb_pobtasi_permuted(ctypes.byref(m), 0x1000, 0, 0x1000, 8, None) == _lib.SGB_ERR_WORKSPACE
    assert lib.sgb_pobtas_permuted(ctypes.byref(m), 0x1000, 0x1000, 2, 2, b"X", 0, 0x1000, 1 << 30, None) == \
        _lib.SGB_ERR_ARG
    assert lib.sgb_pobtas_permuted(ctypes.byref(m), 0x1000, 0x1000, 2, 1, b"N", 0, 0x1000, 1 << 30, None) == \
        _lib.SGB_ERR_SHAPE
    one = _desc(n=1, b=8, a=2)
    assert lib.sgb_pobtaf_permuted(ctypes.byref(one), 0x1000, 0, 0x1000, 1 << 30, None, None) == \
        _lib.SGB_ERR_SHAPE


def test_symv_and_refine_host_checks(lib):
    m = _desc(n=4, b=8, a=2)
    # x and y overlapping are rejected; bad leading dimensions too
    assert lib.sgb_bta_symv(ctypes.byref(m), 0x1000, 2, 0x1008, 2, 2, 1.0, 0.0, None) == _lib.SGB_ERR_ARG
    assert lib.sgb_bta_symv(ctypes.byref(m), 0x1000, 1, 0x100000, 2, 2, 1.0, 0.0, None) == _lib.SGB_ERR_SHAPE
    sz = ctypes.c_size_t(0)
    assert lib.sgb_pobtas_refine_workspace_size(ctypes.byref(m), 3, ctypes.byref(sz)) == 0
    assert sz.value >= 2 * (4 * 8 + 2) * 3 * 8
    other = _desc(n=4, b=8, a=3)
    assert lib.sgb_pobtas_refine(ctypes.byref(m), ctypes.byref(other), 0x1000, 1, 1, 2, 0x1000, 1 << 30,
                                 None) == _lib.SGB_ERR_SHAPE
    assert lib.sgb_pobtas_refine(ctypes.byref(m), ctypes.byref(m), 0x1000, 1, 1, -1, 0x1000, 1 << 30,
                                 None) == _lib.SGB_ERR_ARG
    assert lib.sgb_pobtas_refine(ctypes.byref(m), ctypes.byref(m), 0x1000, 1, 1, 2, None, 0,
                                 None) == _lib.SGB_ERR_WORKSPACE


def test_complex_and_host_entry_points_host_checks(lib):
    m = _desc(n=4, b=8, a=2)
    c = _desc(n=4, b=8, a=2, dtype=_lib.SGB_C128)
    real, cx = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(m), 0, ctypes.byref(real)) == 0
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(c), 0, ctypes.byref(cx)) == 0
    # the embedded stacks (blocks 2b, arrow 2a) follow the real workspace
    assert cx.value >= real.value + 8 * (4 * 16 * 16 + 3 * 16 * 16 + 4 * 4 * 16 + 4 * 4)
    perm = ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_permuted_workspace_size(ctypes.byref(c), 0, ctypes.byref(perm)) == 0
    assert perm.value > cx.value  # plus the embedded buffer
    assert lib.sgb_pobtaf(ctypes.byref(c), 1, 0, None, 0, None, None) == _lib.SGB_ERR_WORKSPACE
    c64 = _desc(n=4, b=8, a=2, dtype=_lib.SGB_C64)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(c64), _lib.SGB_PREC_MIXED, ctypes.byref(cx)) == \
        _lib.SGB_ERR_UNSUPPORTED
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(c), _lib.SGB_PREC_MIXED, ctypes.byref(cx)) == 0
    # host-resident entries: shapes must match, workspace checked before any launch
    other = _desc(n=4, b=8, a=3)
    assert lib.sgb_pobtaf_host(ctypes.byref(m), ctypes.byref(other), 1, 0, 0x1000, 1 << 30, None, None) == \
        _lib.SGB_ERR_SHAPE
    assert lib.sgb_pobtaf_host(ctypes.byref(m), ctypes.byref(m), 1, 0, None, 0, None, None) == \
        _lib.SGB_ERR_WORKSPACE
    assert lib.sgb_pobtasi_host(ctypes.byref(m), ctypes.byref(m), 1, 0, None, 0, None) == _lib.SGB_ERR_WORKSPACE


def test_error_mapping():
    with pytest.raises(ValueError):
        _lib.raise_for(_lib.SGB_ERR_SHAPE, "x")
    with pytest.raises(TypeError):
        _lib.raise_for(_lib.SGB_ERR_DTYPE, "x")
    with pytest.raises(np.linalg.LinAlgError):
        _lib.raise_for(_lib.SGB_ERR_NOT_SPD, "x")
    with pytest.raises(NotImplementedError):
        _lib.raise_for(_lib.SGB_ERR_UNSUPPORTED, "x")
    _lib.raise_for(_lib.SGB_OK, "x")


def test_precision_strings():
    assert _lib.precision_code("fp64") == _lib.SGB_PREC_NATIVE
    assert _lib.precision_code("mixed") == _lib.SGB_PREC_MIXED
    assert _lib.precision_code("mixed:5") == _lib.SGB_PREC_MIXED | (5 << 8)
    assert _lib.precision_code("mixed:6:7") == _lib.SGB_PREC_MIXED | (6 << 8) | (7 << 16)
    for bad in ("mixed:2", "mixed:6:8", "mixed:6:7:7", "half"):
        with pytest.raises(ValueError):
            _lib.precision_code(bad)


def test_inverse_slice_count_workspace_and_range(lib):
    m = _desc(n=4, b=512, a=64)
    sz6, sz67 = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(m), _lib.precision_code("mixed:6"), ctypes.byref(sz6)) == 0
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(m), _lib.precision_code("mixed:6:7"),
                                         ctypes.byref(sz67)) == 0
    assert sz67.value > sz6.value  # slice scratch for 7 slices
    bad = _lib.SGB_PREC_MIXED | (6 << 8) | (9 << 16)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(m), bad, ctypes.byref(sz6)) == _lib.SGB_ERR_ARG
    assert lib.sgb_pobtasi_workspace_size(ctypes.byref(m), 1 << 24 | 1, ctypes.byref(sz6)) == _lib.SGB_ERR_ARG


def test_spin_limit_hook_roundtrip(lib):
    prev = _lib.spin_limit()
    assert prev == 1 << 22
    assert _lib.spin_limit(5) == prev
    assert _lib.spin_limit(prev) == 5
    assert _lib.spin_limit() == prev


def test_stream_workspace_does_not_grow_with_n(lib):
    """The streamed ring's device footprint depends on the ring, not on n."""
    sizes = []
    for n in (10, 1000, 1_000_000):
        m = _desc(n=n, b=512, a=64)
        for q, ring in ((lib.sgb_pobtaf_stream_workspace_size, 4), (lib.sgb_pobtasi_stream_workspace_size, 32)):
            sz = ctypes.c_size_t(0)
            assert q(ctypes.byref(m), 0, ring, ctypes.byref(sz)) == 0
            sizes.append((q.__name__, sz.value))
    by = {}
    for name, v in sizes[2:]:  # n = 10 may be smaller (pobtasi chunk shrinks with n)
        by.setdefault(name, set()).add(v)
    assert all(len(v) == 1 for v in by.values()), by
    m = _desc(n=100, b=512, a=64)
    sz = ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_stream_workspace_size(ctypes.byref(m), 0, 1, ctypes.byref(sz)) == _lib.SGB_ERR_SHAPE
    cm = _desc(n=100, b=64, a=8, dtype=_lib.SGB_C128)
    assert lib.sgb_pobtaf_stream_workspace_size(ctypes.byref(cm), 0, 4, ctypes.byref(sz)) == _lib.SGB_ERR_UNSUPPORTED


def test_batch_plan_ex_rejects_bad_panel_ctas(lib):
    m = _desc(n=4, b=8, a=2)
    plan = ctypes.c_void_p(0)
    ns = (ctypes.c_int64 * 1)(0)
    rhs = (ctypes.c_void_p * 1)(None)
    assert lib.sgb_batch_plan_create_ex(ctypes.byref(m), rhs, ns, 1, 1, None, 1, -1, 0, 0x1000, 1 << 20,
                                        ctypes.byref(plan)) == _lib.SGB_ERR_ARG
    assert lib.sgb_batch_plan_create_ex(ctypes.byref(m), rhs, ns, 1, 1, None, 0, 24, 0, 0x1000, 1 << 20,
                                        ctypes.byref(plan)) == _lib.SGB_ERR_ARG
    assert lib.sgb_batch_plan_create_ex(ctypes.byref(m), rhs, ns, 1, 1, None, 1, 24, 2, 0x1000, 1 << 20,
                                        ctypes.byref(plan)) == _lib.SGB_ERR_ARG


def test_logdet_grad_host_checks(lib):
    m = _desc(n=4, b=8, a=2)
    assert lib.sgb_bta_logdet_quad_grad(ctypes.byref(m), None, 1, 1, 0x1000, None) == _lib.SGB_ERR_ARG
    assert lib.sgb_bta_logdet_quad_grad(ctypes.byref(m), 0x1000, 0, 1, 0x1000, None) == _lib.SGB_ERR_SHAPE
    assert lib.sgb_bta_logdet_quad_grad(ctypes.byref(m), 0x1000, 2, 1, 0x1000, None) == _lib.SGB_ERR_SHAPE
    c = _desc(n=4, b=8, a=2, dtype=_lib.SGB_C128)
    assert lib.sgb_bta_logdet_quad_grad(ctypes.byref(c), 0x1000, 1, 1, 0x1000, None) == _lib.SGB_ERR_DTYPE
