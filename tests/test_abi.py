"""The C ABI library: it builds, loads without a GPU, and exports every declared symbol."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "anneal_gb300.h")


@pytest.fixture(scope="module")
def lib_path():
    from anneal_gb300 import build
    return build.build()


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(anl_[A-Za-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    from anneal_gb300 import _native as N
    assert declared_symbols() == sorted(N.EXPORTS)


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_text_need_no_gpu(lib_path):
    from anneal_gb300 import _native as N
    lib = N.load()
    assert lib.anl_version() >= 100
    assert isinstance(N.last_error(), str)


def test_bad_arguments_are_rejected_before_any_device_work(lib_path):
    from anneal_gb300 import _native as N
    lib = N.load()
    h = ctypes.c_void_p()
    st = lib.anl_ctx_create(ctypes.byref(h), 0, 4, 4, 1.0, 0.3, 0)
    assert st == N.ANL_ERR_BADARG
    assert "bad arguments" in N.last_error()
    assert lib.anl_apply_K(None, None, None, None, None) == N.ANL_ERR_BADARG


def test_release_build_has_no_bounds_checks(lib_path):
    from anneal_gb300 import _native as N
    if N.DEBUG_LIB:
        pytest.skip("the debug library is loaded")
    lib = N.load()
    count, first = ctypes.c_longlong(0), (ctypes.c_longlong * 3)()
    assert lib.anl_debug_oob(ctypes.byref(count), first) == N.ANL_OK
    assert count.value == -1 and list(first) == [0, 0, 0]


def test_debug_build_compiles_and_exports_every_declared_symbol():
    from anneal_gb300 import build
    path = build.build(debug=True)
    assert path.endswith(os.path.join("_lib_debug", "libanneal_gb300.so"))
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
