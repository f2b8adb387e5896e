"""GPU multi-array writer (include/multiarray.gpu.h) against single-array
ingestion through the oracle.

Three arrays of different shapes, dtypes, codecs and pyramids are fed
through one multiarray writer, epoch by epoch in turns, with the
reference's switching rule exercised (a switch away from an array in the
middle of an epoch is refused as not flushable, src/multiarray/stream.c:
552-571).  Each array's shards must equal the oracle's shards of that array
ingested alone: byte for byte without compression, chunk by chunk after
decoding with compression.
"""
import ctypes as C

import numpy as np
import pytest

from chucky_gb300 import capi, load
from harness import MemSink, compare_decoded, epoch_elements, run_oracle

pytestmark = pytest.mark.gpu

D = dict


def _arrays():
    return [
        # bounded 3-D u16 cube with a mean pyramid, no compression
        ([D(size=24, chunk=8, cps=2, name="z", downsample=1),
          D(size=32, chunk=8, cps=2, name="y", downsample=1),
          D(size=32, chunk=8, cps=2, name="x", downsample=1)],
         dict(dtype="u16", reduce="mean", epochs_per_batch=2)),
        # unbounded u8 frames with a dim-0 max pyramid, no compression
        ([D(size=0, chunk=2, cps=1, name="t", downsample=1),
          D(size=40, chunk=16, cps=2, name="y", downsample=1),
          D(size=48, chunk=16, cps=2, name="x", downsample=1)],
         dict(dtype="u8", reduce="max", append_reduce="max")),
        # unbounded f32 stacks, zstd, no pyramid
        ([D(size=0, chunk=1, cps=2, name="t"), D(size=8, chunk=8, cps=1, name="z"),
          D(size=64, chunk=32, cps=2, name="y"), D(size=64, chunk=32, cps=2, name="x")],
         dict(dtype="f32", codec="zstd", level=1)),
    ]


def _config(spec, kw, **over):
    dims = capi.make_dims(spec)
    cfg = capi.make_config(dims, **dict(kw, **over))
    cfg._dims = dims
    return cfg


def _epoch_bytes(spec, kw):
    # the planner's epoch (inner dims in the lifted, chunk-padded space)
    return epoch_elements(_config(spec, kw)) * capi.BPE[kw["dtype"]]


def test_multiarray_matches_single_arrays():
    lib = load()
    P = C.c_void_p
    lib.multiarray_tile_stream_gpu_create.restype = P
    lib.multiarray_tile_stream_gpu_create.argtypes = [C.c_int, P, P, C.c_int]
    lib.multiarray_tile_stream_gpu_writer.restype = C.POINTER(capi.MultiarrayWriter)
    lib.multiarray_tile_stream_gpu_writer.argtypes = [P]
    lib.multiarray_tile_stream_gpu_destroy.argtypes = [P]

    arrays = _arrays()
    rng = np.random.default_rng(31)
    epochs = [3, 5, 4]  # array 0 is bounded at 3 epochs (24 / 8)
    data = []
    for (spec, kw), ne in zip(arrays, epochs):
        nb = _epoch_bytes(spec, kw) * ne
        if kw["dtype"] == "f32":
            x = rng.normal(0, 1, size=nb // 4).astype("<f4").view(np.uint8)
        else:
            x = rng.integers(0, 255, size=nb, dtype=np.uint8)
        data.append(np.ascontiguousarray(x))
    cfgs = [_config(spec, kw) for spec, kw in arrays]
    sinks = [MemSink() for _ in arrays]
    try:
        carr = (capi.StreamConfiguration * 3)(*cfgs)
        sarr = (P * 3)(*[s.base for s in sinks])
        ms = lib.multiarray_tile_stream_gpu_create(3, carr, sarr, 1)
        assert ms
        try:
            w = lib.multiarray_tile_stream_gpu_writer(ms)
            wc = w.contents

            def update(i, a, b):
                buf = data[i]
                base = buf.ctypes.data
                return wc.update(w, i, capi.Slice(base + a, base + b))

            pos = [0, 0, 0]
            ebytes = [_epoch_bytes(spec, kw) for spec, kw in arrays]
            # half an epoch into array 1, then a refused switch to array 2
            r = update(1, 0, ebytes[1] // 2)
            assert r.error == capi.MULTIARRAY_OK
            pos[1] = ebytes[1] // 2
            r = update(2, 0, ebytes[2])
            assert r.error == capi.MULTIARRAY_NOT_FLUSHABLE
            assert r.rest.beg == data[2].ctypes.data
            r = update(1, pos[1], ebytes[1])
            assert r.error == capi.MULTIARRAY_OK
            pos[1] = ebytes[1]
            base = data[0].ctypes.data
            assert wc.update(w, 7, capi.Slice(base, base)).error == capi.MULTIARRAY_FAIL
            # the rest in turns, one epoch at a time
            while any(p < d.size for p, d in zip(pos, data)):
                for i in range(3):
                    if pos[i] < data[i].size:
                        b = min(data[i].size, pos[i] + ebytes[i])
                        r = update(i, pos[i], b)
                        assert r.error == capi.MULTIARRAY_OK, (i, r.error)
                        pos[i] = b
            # array 0 is bounded and full: more data is refused as finished
            extra = update(0, 0, ebytes[0])
            assert extra.error == capi.MULTIARRAY_FINISHED
            assert wc.flush(w).error == capi.MULTIARRAY_OK
        finally:
            lib.multiarray_tile_stream_gpu_destroy(ms)
        got = [s.shards() for s in sinks]
    finally:
        for s in sinks:
            s.close()
    for i, ((spec, kw), cfg) in enumerate(zip(arrays, cfgs)):
        if kw.get("codec", "none") == "none":
            want, _ = run_oracle(cfg, data[i], quirks=False)
            assert got[i].keys() == want.keys(), i
            for k in want:
                assert got[i][k] == want[k], (i, k)
        else:
            raw_cfg = _config(spec, kw, codec="none", level=0)
            want, _ = run_oracle(raw_cfg, data[i], quirks=False)
            n, _, _ = compare_decoded(cfg, got[i], want, kw["codec"])
            assert n > 0
