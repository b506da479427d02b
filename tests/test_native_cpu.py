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


_CTYPE_OF = {"double": ctypes.c_double, "int32_t": ctypes.c_int32, "uint64_t": ctypes.c_uint64}


def header_struct(name):
    """(field, C type) pairs of `typedef struct name {...} name;` in include/mepgl.h."""
    text = open(os.path.join(ROOT, "include", "mepgl.h")).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        fields += [(n.strip(), ctype) for n in names.split(",")]
    return fields


def test_refinement_structs_match_the_header():
    from mepgl_gb300 import native
    for name, cls in (("mepgl_refine_options", native.MepglRefineOptions),
                      ("mepgl_refine_report", native.MepglRefineReport)):
        want = [(f, _CTYPE_OF[t]) for f, t in header_struct(name)]
        assert list(cls._fields_) == want, (name, cls._fields_, want)


def test_default_refine_options():
    from mepgl_gb300 import build as B, native
    B.build()
    o = native.MepglRefineOptions()
    native.lib().mepgl_default_refine_options(ctypes.byref(o))
    assert (o.g_tol, o.max_newton, o.max_cg, o.lanczos_steps, o.gauge_degree) == (1e-8, 40, 3000, 12, -1)
    assert (o.mu0, o.cg_eta, o.max_retries, o.gauge_refresh, o.precondition, o.forcing) == (1e-3, 0.1, 8, 0, 1, 0)
