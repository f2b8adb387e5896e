"""The C-ABI library: it builds, loads without a GPU, exports every entry
point declared in include/*.h, and its host-only helpers agree with the
reference (dimension helpers, planner through the memory estimate)."""
import ctypes as C
import os
import re

import pytest

import cases
import harness as H
import chucky_gb300 as cg
from chucky_gb300 import build as cgbuild
from chucky_gb300 import capi

INCLUDE = os.path.join(H.ROOT, "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(INCLUDE, f)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b([a-z_][a-z0-9_]*)\s*\((?!\s*\*)", txt):
            name = m.group(1)
            before = txt[:m.start()].rstrip()
            if before.endswith(("static inline", "return", "if", "switch", "sizeof")):
                continue
            if name in ("if", "switch", "return", "sizeof", "while", "for"):
                continue
            names.add(name)
    # static inline helpers defined in headers are not exported
    return {n for n in names if n not in ("dtype_bpe", "dtype_zarr_string",
                                          "dtype_accum_bpe")}


@pytest.fixture(scope="module")
def lib():
    cgbuild.build()
    return cg.load()


def test_every_declared_symbol_is_exported(lib):
    decl = declared_functions()
    assert "tile_stream_gpu_create" in decl and "writer_append" in decl
    missing = [n for n in sorted(decl) if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_list_matches_headers(lib):
    assert set(cg.EXPORTS) <= declared_functions()


@pytest.mark.parametrize("case", cases.CASES, ids=[c[0] for c in cases.CASES])
def test_memory_estimate_plans_like_the_oracle(lib, case):
    cfg, _ = cases.build(case)
    info = capi.MemoryInfo()
    assert lib.tile_stream_gpu_memory_estimate(C.byref(cfg), C.byref(info)) == 0
    o = H.oracle()
    sink = H.MemSink()
    s = o.oracle_stream_create(C.byref(cfg), sink.base)
    try:
        class Info(C.Structure):
            _fields_ = [("nlod", C.c_int), ("append_downsample", C.c_int),
                        ("epochs_per_batch", C.c_uint32), ("total_chunks", C.c_uint64),
                        ("chunk_elements", C.c_uint64), ("epoch_elements", C.c_uint64),
                        ("max_output_size", C.c_uint64)]
        oi = Info()
        o.oracle_stream_info.argtypes = [C.c_void_p, C.c_void_p]
        buf = C.create_string_buffer(4096)
        o.oracle_stream_info(s, buf)
        oi = Info.from_buffer_copy(buf.raw[:C.sizeof(Info)])
        assert info.nlod == oi.nlod
        assert info.epochs_per_batch == oi.epochs_per_batch
        assert info.total_chunks == oi.total_chunks
    finally:
        o.oracle_stream_destroy(s)
        sink.close()


def test_invalid_configs_are_rejected(lib):
    case = cases.CASES[0]
    cfg, _ = cases.build(case, codec="lz4", level=0)  # LZ4 needs level >= 1
    info = capi.MemoryInfo()
    assert lib.tile_stream_gpu_memory_estimate(C.byref(cfg), C.byref(info)) != 0
    cfg, _ = cases.build(case, codec=capi.CODEC_BLOSC_LZ4)
    assert lib.tile_stream_gpu_memory_estimate(C.byref(cfg), C.byref(info)) != 0
    assert lib.codec_is_gpu_supported(capi.CODEC_ZSTD) == 1
    assert lib.codec_is_gpu_supported(capi.CODEC_BLOSC_ZSTD) == 0


@pytest.mark.skipif(H.reference() is None, reason="reference build not present")
def test_dims_helpers_match_reference(lib):
    ref = H.reference()
    for name in ("dims_budget_chunk_size", "dims_n_append", "dims_set_shard_counts"):
        getattr(ref, name)
    specs = [[1, 1, 0], [1, 2, 2], [0, 1, 3, 1], [2, 1, 1, 1, 1]]
    for ratios in specs:
        rank = len(ratios)
        for nelem in (1, 7, 4096, 1 << 20, 12345):
            a = capi.make_dims([dict(size=1024, chunk=1) for _ in range(rank)])
            b = capi.make_dims([dict(size=1024, chunk=1) for _ in range(rank)])
            r = (C.c_uint8 * rank)(*ratios)
            lib.dims_budget_chunk_size(a, rank, C.c_uint64(nelem), r)
            ref.dims_budget_chunk_size(b, rank, C.c_uint64(nelem), r)
            assert [a[i].chunk_size for i in range(rank)] == \
                   [b[i].chunk_size for i in range(rank)]
    for chunks in ([1, 1, 4], [1, 4, 4], [2, 1, 1], [1, 1, 1]):
        for ds in ([0, 0, 0], [0, 1, 0], [1, 1, 1]):
            a = capi.make_dims([dict(size=8, chunk=c, downsample=d)
                                for c, d in zip(chunks, ds)])
            assert lib.dims_n_append(a, 3) == ref.dims_n_append(a, 3)
