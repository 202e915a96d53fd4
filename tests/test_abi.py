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
