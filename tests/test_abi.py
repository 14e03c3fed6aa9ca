"""The C-ABI library builds, loads and exports every declared entry point (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from picgo_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "medyan_mech.h")


def declared_functions(path=HEADER):
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mech_[a-z_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "mech_minimize" in names and "mech_set_networks" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.EXPORTS) | {n for n in names if n.startswith("mech_")}


def test_abi_version_and_struct_sizes(lib):
    assert lib.mech_abi_version() == 1
    # the ctypes mirrors must have the C layout: pointer-aligned network, 48-byte int head of MechResult
    assert C.sizeof(_lib.MechResult) == 48 + 8 * 4 + 8 * 7 * 2 + 8
    assert C.sizeof(_lib.MechCGParams) == 56
    assert _lib.MechNetwork.box.offset % 8 == 0


def test_context_without_device_fails_loudly(lib):
    ctx = C.c_void_p()
    rc = lib.mech_ctx_create(0, 0, C.byref(ctx))
    if rc == 0:          # a GPU is visible: the call must have produced a context
        assert ctx.value
        assert lib.mech_ctx_destroy(ctx) == 0
    else:
        assert rc == -8, rc
        assert b"device" in lib.mech_last_error()


def test_bad_arguments_are_rejected(lib):
    assert lib.mech_ctx_create(7, 0, C.byref(C.c_void_p())) == -1
    assert lib.mech_minimize(None, None, None) == -1
