"""The C-ABI library builds, loads and exports every symbol include/mepgl.h
declares (no GPU calls)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "mepgl.h")).read()
    return sorted(set(re.findall(r"\b(mepgl_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "mepgl_create" in syms and "mepgl_nlcg_steps" in syms and len(syms) >= 19


def test_library_exports_every_declared_symbol():
    from mepgl_gb300 import build as B
    lib = B.build()
    L = ctypes.CDLL(lib)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from mepgl_gb300 import native
    assert set(declared_symbols()) <= set(native.exported_symbols())


def test_default_options_are_reference_semantics():
    from mepgl_gb300 import build as B, native
    B.build()
    o = native.default_options()
    assert (o.line_search, o.line_polynomial, o.spline, o.metric) == (
        native.LS_COMPAT, native.POLY_COMPAT, native.SPLINE_COMPAT, native.METRIC_JB)
