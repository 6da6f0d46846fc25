"""CPU-side checks of the C ABI: the built library loads without a GPU and
exports every function include/*.h declares; argument validation returns
RTA_ERR_INVALID without touching a device."""
import ctypes as C
import glob
import os
import re

import pytest

from rta_gb300 import lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w \*]*?\b(rta_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(L.LIB_PATH):
        from rta_gb300 import build as B
        B.build()
    return L.load()


def test_header_declares_the_binding_list():
    assert declared_functions() == sorted(L.SYMBOLS)


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing


def test_invalid_arguments_are_rejected_without_a_device(lib):
    h = C.c_void_p()
    assert lib.rta_lbvh_create(C.byref(h)) == L.OK
    try:
        assert lib.rta_lbvh_build(h, None, 10, 30, None, None) == L.ERR_INVALID
        assert lib.rta_lbvh_build(h, C.c_void_p(16), 0, 30, None, None) == L.ERR_INVALID
        assert lib.rta_lbvh_build(h, C.c_void_p(16), 10, 31, None, None) == L.ERR_INVALID
        too_many = lib.rta_lbvh_max_triangles() + 1
        assert lib.rta_lbvh_build(h, C.c_void_p(16), too_many, 30, None, None) == L.ERR_INVALID
        v = L.LbvhView()
        assert lib.rta_lbvh_get(h, C.byref(v)) == L.ERR_INVALID   # nothing built yet
        for bad in (0, 7, 12):
            assert lib.rta_lbvh_set_digit_bits(h, bad) == L.ERR_INVALID
        for good in (8, 9, 10, 11):
            assert lib.rta_lbvh_set_digit_bits(h, good) == L.OK
        ms = C.c_float(0)
        assert lib.rta_frame_set_timing(None, 1) == L.ERR_INVALID
        assert lib.rta_frame_trace_ms(None, C.byref(ms)) == L.ERR_INVALID
    finally:
        assert lib.rta_lbvh_destroy(h) == L.OK
    assert lib.rta_trace(None, None, None, None, 0, None, None, 0, None, None) == L.ERR_INVALID
    assert lib.rta_setup_shirley_rays(None, None, None, 0.5, 1.0, 0, 0, None, None, None, 1.0,
                                      None) == L.ERR_INVALID
    assert lib.rta_frame_create(None, 10) == L.ERR_INVALID
    assert lib.rta_selftest_bounded_wait(None, None) == L.ERR_INVALID


def test_max_triangles_matches_link_encoding(lib):
    # leaf links carry 25-bit first-triangle offsets
    assert lib.rta_lbvh_max_triangles() == 1 << 25
