"""The C ABI library exists, loads and exports every declared symbol (CPU).

No compute call is made here: this machine may have no GPU.
"""
import ctypes
import os
import re

import pytest

from tskit_gb300 import _build, _native

HEADER = os.path.join(_build.INCLUDE, "tskit_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(tsg_\w+)\s*\(", src)
    return sorted(set(n for n in names if not n.endswith("_t")))


@pytest.fixture(scope="module")
def lib():
    _build.build_cuda()
    return ctypes.CDLL(_native.lib_path())


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


def test_bindings_cover_header():
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_strerror_matches_reference_messages(lib):
    lib.tsg_strerror.restype = ctypes.c_char_p
    assert lib.tsg_strerror(-901).decode() == "Windows must be increasing list [0, ..., L]"
    assert lib.tsg_strerror(-600).decode() == "Duplicate sample value"
