"""The C-ABI library loads, exports every entry point declared in
include/mdet_tnf.h and rejects bad arguments without touching a GPU."""
import ctypes
import os
import re

import mdet_gb300 as m
from mdet_gb300 import tnf as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "mdet_tnf.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mdet_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol():
    lib = T.load_library()
    names = header_functions()
    assert len(names) >= 13
    for nm in names:
        assert hasattr(lib, nm), nm
    # the Python bindings cover the same set
    assert sorted(n for n, _, _ in T.SIGNATURES) == names


def test_version_string():
    assert "sm_103a" in m.version()


def test_null_context_is_rejected():
    lib = T.load_library()
    assert lib.mdet_tnf_count(None, None, 0, None, None, 0, None, None) == T.ERR_INVALID
    ne = ctypes.c_uint64(0)
    assert lib.mdet_tnf_graph(None, None, None, 0, 0.9, 200, 0, None, None, None, 0, ctypes.byref(ne),
                              None) == T.ERR_INVALID
    assert lib.mdet_tnf_max_prob(None, None, None, 0, None, 0, 0, 0.7, None) == T.ERR_INVALID
    assert lib.mdet_last_error(None) == b"null context"
    assert lib.mdet_ctx_destroy(None) == T.OK


def test_bad_device_fails_cleanly():
    lib = T.load_library()
    h = ctypes.c_void_p()
    rc = lib.mdet_ctx_create(1 << 20, ctypes.byref(h))
    assert rc in (T.ERR_INVALID, T.ERR_CUDA)
    assert not h.value
