"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares (no compute calls here)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(jgb_[A-Za-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("jgb_create", "jgb_destroy", "jgb_formod", "jgb_formod_batch",
                     "jgb_formod_batch_dev", "jgb_set_table", "jgb_set_filter"):
        assert required in names


def test_library_exports_all_declared_symbols(built_lib):
    lib = ctypes.CDLL(os.path.join(ROOT, "jurassic_gb300", "libjurassic_gb300.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, "not exported: %s" % missing


def test_python_binding_covers_header(built_lib):
    from jurassic_gb300 import native
    missing = [n for n in declared_functions() if n not in native.SIGNATURES]
    assert not missing, "no ctypes signature for: %s" % missing


def test_invalid_control_is_rejected_without_gpu(built_lib):
    """Argument checks run before any device work: a bad control set returns
    JGB_ERR_ARG (the reference would exit())."""
    from jurassic_gb300 import native
    L = native.load()
    c = native._Ctl(ng=-1, nd=0)
    h = ctypes.c_void_p()
    assert L.jgb_create(ctypes.byref(c), 0, ctypes.byref(h)) == 1
    assert not h.value
