"""The encoder autotuner's choice rule and its C API (no GPU): candidates
whose output is at most 1 % above the preferred one's are eligible, the
cost of a candidate is
max(encode, copy-out) + 1/4 min(encode, copy-out) per input byte, and a
candidate within 1 % of the best cost loses to the preferred one."""
import ctypes as C

import pytest

from chucky_gb300 import capi, load


@pytest.fixture(scope="module")
def lib():
    lib = load()
    lib.chucky_autotune_pick.restype = C.c_int
    lib.chucky_autotune_pick.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.c_int, C.c_double, C.c_double, C.c_int]
    lib.chucky_autotune_entries.restype = C.c_size_t
    lib.chucky_autotune_entries.argtypes = [C.c_void_p, C.c_size_t]
    lib.chucky_autotune_enabled.restype = C.c_int
    return lib


def _pick(lib, enc_s, out_bytes, in_bytes=1e9, d2h=100.0, preferred=0):
    n = len(enc_s)
    e = (C.c_double * n)(*enc_s)
    o = (C.c_double * n)(*out_bytes)
    return lib.chucky_autotune_pick(e, o, n, in_bytes, d2h, preferred)


def test_only_the_best_compressing_are_eligible(lib):
    # 1 GB in, copy-out at 100 GB/s; the fast candidates compress 10 % worse
    # than the preferred (first) one: the other is slower but compresses
    # better, and is cheaper than the preferred
    assert _pick(lib, [0.030, 0.002, 0.020], [1.0e9, 1.1e9, 0.9e9]) == 2
    assert _pick(lib, [0.002, 0.020, 0.030], [1.0e9, 0.9e9, 0.905e9], preferred=-1) == 1


def test_fastest_of_equal_outputs(lib):
    # outputs within 1 % of each other: the least cost
    assert _pick(lib, [0.040, 0.020, 0.030], [0.9e9, 0.905e9, 0.9e9]) == 1


def test_copy_bound_cost(lib):
    # equal outputs, copy-out (9 ms) above every encode: the 1/4 overlap term
    assert _pick(lib, [0.004, 0.002, 0.003], [0.9e9, 0.9e9, 0.9e9]) == 1


def test_near_tie_keeps_the_preferred(lib):
    assert _pick(lib, [0.0200, 0.0199], [1e9, 1e9], preferred=0) == 0
    assert _pick(lib, [0.0200, 0.0150], [1e9, 1e9], preferred=0) == 1
    assert _pick(lib, [0.0150, 0.0200, 0.0151], [1e9, 1e9, 1e9], preferred=2) == 2
    # a faster candidate that compresses worse than the preferred one
    assert _pick(lib, [0.0200, 0.0100], [1e9, 1.1e9], preferred=0) == 0


def test_switch_and_empty_table(lib):
    was = lib.chucky_autotune_enabled()
    try:
        lib.chucky_autotune_set_enabled(1)
        assert lib.chucky_autotune_enabled() == 1
        lib.chucky_autotune_set_enabled(0)
        assert lib.chucky_autotune_enabled() == 0
    finally:
        lib.chucky_autotune_set_enabled(was)
    lib.chucky_autotune_clear()
    assert lib.chucky_autotune_entries(None, 0) == 0
