"""The CPU oracle, pinned against the reference CPU backend (compiled here
from the reference sources into oracle/_ref when that tree is present) and
against known answers from the reference's own tests."""
import ctypes as C

import numpy as np
import pytest

import cases
import harness as H
from chucky_gb300 import capi

needs_ref = pytest.mark.skipif(H.reference() is None,
                               reason="reference build (oracle/_ref) not present")


def _pieces(nbytes, seed):
    rng = np.random.default_rng(seed)
    return sorted(rng.integers(1, max(2, nbytes), size=5).tolist())


@needs_ref
@pytest.mark.parametrize("case", cases.CASES, ids=[c[0] for c in cases.CASES])
@pytest.mark.parametrize("dtype", ["u16", "i8", "f32", "u64"])
def test_oracle_matches_reference(case, dtype):
    cfg, epochs = cases.build(case, dtype)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=7)
    bpe = capi.BPE[dtype]
    pieces = [p - p % bpe for p in _pieces(n * bpe, 3)]
    a, ca = H.run_oracle(cfg, data, pieces)
    b, cb = H.run_reference(cfg, data, pieces)
    assert ca == cb
    assert a == b, H.diff_shards(a, b)


@needs_ref
@pytest.mark.parametrize("method", ["mean", "min", "max", "median", "max_sup", "min_sup"])
@pytest.mark.parametrize("dtype", cases.DTYPES_ALL)
def test_oracle_lod_methods_match_reference(method, dtype):
    case = cases.CASES[[c[0] for c in cases.CASES].index("sensor_dim0")]
    app = method if method in ("mean", "min", "max") else "mean"
    cfg, epochs = cases.build(case, dtype, reduce=method, append_reduce=app)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=11)
    a, _ = H.run_oracle(cfg, data)
    b, _ = H.run_reference(cfg, data)
    assert a == b, H.diff_shards(a, b)


def test_crc32c_known_answer():
    lib = H.oracle()
    buf = C.create_string_buffer(b"123456789", 9)
    assert lib.oracle_crc32c(buf, 9) == 0xE3069283


def test_morton_rank_power_of_two_is_z_order():
    lib = H.oracle()
    shape = (C.c_uint64 * 2)(4, 4)
    for y in range(4):
        for x in range(4):
            c = (C.c_uint64 * 2)(x, y)
            z = 0
            for b in range(2):
                z |= ((x >> b) & 1) << (2 * b) | ((y >> b) & 1) << (2 * b + 1)
            assert lib.oracle_morton_rank(2, shape, c, 0) == z


def test_morton_rank_is_a_bijection_on_ragged_shapes():
    lib = H.oracle()
    for shp in [(3, 5), (5, 3, 2), (7,), (6, 10)]:
        n = int(np.prod(shp))
        shape = (C.c_uint64 * len(shp))(*shp)
        ranks = set()
        for idx in np.ndindex(*shp):
            c = (C.c_uint64 * len(shp))(*idx)
            ranks.add(lib.oracle_morton_rank(len(shp), shape, c, 0))
        assert ranks == set(range(n))


def _f16_window(vals, method):
    lib = H.oracle()
    src = np.asarray(vals, dtype="<f2")
    out = np.zeros(1, dtype="<f2")
    assert lib.oracle_reduce_window(out.ctypes.data, src.ctypes.data, len(src),
                                    capi.DTYPE["f16"], capi.REDUCE[method]) == 0
    return float(out[0])


def test_f16_reduce_known_windows():
    # 8 -> 2 windows of tests/test_lod_dtypes.cu:290-360 (f16 mean/min/max)
    src = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0]
    for w in range(2):
        win = src[4 * w:4 * w + 4]
        assert _f16_window(win, "mean") == pytest.approx(sum(win) / 4, abs=1e-3)
        assert _f16_window(win, "min") == min(win)
        assert _f16_window(win, "max") == max(win)


def _fold(dtype, epochs, method, level):
    lib = H.oracle()
    npd = capi.NUMPY_DTYPE[dtype]
    acc = np.zeros(len(epochs[0]), dtype=npd)
    for i, e in enumerate(epochs):
        x = np.asarray(e, dtype=npd)
        lib.oracle_fold(acc.ctypes.data, x.ctypes.data, len(x), i, level,
                        capi.DTYPE[dtype], capi.REDUCE[method])
    out = np.zeros_like(acc)
    lib.oracle_emit(out.ctypes.data, acc.ctypes.data, len(acc), len(epochs),
                    capi.DTYPE[dtype], capi.REDUCE[method])
    return out


def test_dim0_integer_mean_shifts_at_every_fold():
    # tests/test_lod.c:574-612 and tests/test_lod_dtypes.cu:196-206: the
    # integer mean applies (a>>s)+(b>>s)+(((a&m)+(b&m))>>s) with s = level at
    # every fold step.
    vals = [[100], [200], [300], [400]]
    acc = 100
    for v in (200, 300, 400):
        acc = (acc >> 2) + (v >> 2) + (((acc & 3) + (v & 3)) >> 2)
    assert _fold("u16", vals, "mean", 2)[0] == acc
    assert _fold("u16", [[10], [20]], "mean", 1)[0] == 15


def test_dim0_float_mean_divides_at_emit():
    out = _fold("f32", [[1.0], [2.0], [4.0], [5.0]], "mean", 2)
    assert out[0] == np.float32(12.0) / np.float32(4)
    out = _fold("f16", [[1.0], [2.0], [4.0], [5.0]], "mean", 2)
    assert float(out[0]) == 3.0


def test_dim0_min_max_fold():
    assert _fold("i16", [[5], [-3], [7]], "min", 2)[0] == -3
    assert _fold("u8", [[5], [3], [7]], "max", 2)[0] == 7
