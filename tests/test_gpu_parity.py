"""GPU stream vs the CPU oracle: whole shard files, byte for byte.

CODEC_NONE makes every chunk byte visible, so these compare the transpose,
the LOD pyramid (every level, every reduce method, dim-0 folds), the shard
aggregation, the index and its crc32c, and the shard keys.  The oracle runs
with reference quirks off: a partial final epoch is zero-filled and a dim-0
drain delivers the drained data (the two places where the reference CPU
backend delivers stale buffer contents)."""
import numpy as np
import pytest

import cases
import harness as H
from chucky_gb300 import capi

pytestmark = pytest.mark.gpu


def _pieces(nbytes, bpe, seed):
    rng = np.random.default_rng(seed)
    cuts = rng.integers(1, max(2, nbytes), size=6).tolist()
    return sorted(c - c % bpe for c in cuts)


@pytest.mark.parametrize("case", cases.CASES, ids=[c[0] for c in cases.CASES])
@pytest.mark.parametrize("dtype", ["u16", "u8", "f32", "i64"])
def test_gpu_matches_oracle(case, dtype):
    cfg, epochs = cases.build(case, dtype)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=5)
    pieces = _pieces(n * capi.BPE[dtype], capi.BPE[dtype], 9)
    a, ca = H.run_gpu(cfg, data, pieces)
    b, cb = H.run_oracle(cfg, data, pieces, quirks=False)
    assert ca == cb
    assert a == b, H.diff_shards(a, b)


@pytest.mark.parametrize("method", ["mean", "min", "max", "median", "max_sup", "min_sup"])
@pytest.mark.parametrize("dtype", cases.DTYPES_ALL + ["f16"])
def test_gpu_lod_methods(method, dtype):
    case = cases.CASES[[c[0] for c in cases.CASES].index("sensor_dim0")]
    app = method if method in ("mean", "min", "max") else "max"
    cfg, epochs = cases.build(case, dtype, reduce=method, append_reduce=app)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=13)
    a, _ = H.run_gpu(cfg, data)
    b, _ = H.run_oracle(cfg, data, quirks=False)
    assert a == b, H.diff_shards(a, b)


@pytest.mark.parametrize("case", cases.CASES, ids=[c[0] for c in cases.CASES])
@pytest.mark.parametrize("dtype", ["u16", "f32"])
def test_gpu_device_pointer_appends(case, dtype):
    """Appends of device memory (the copy to the epoch buffer is then a
    device-to-device copy) in arbitrary pieces: the same shards."""
    import torch
    import chucky_gb300 as cg
    cfg, epochs = cases.build(case, dtype)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=21)
    bpe = capi.BPE[dtype]
    cuts = [0] + _pieces(n * bpe, bpe, 4) + [n * bpe]
    dev = torch.from_numpy(data.view(np.uint8).reshape(-1).copy()).cuda()
    torch.cuda.synchronize()
    sink = H.MemSink()
    try:
        s = cg.GpuStream(cfg, sink.base)
        try:
            base = dev.data_ptr()
            for a, b in zip(cuts[:-1], cuts[1:]):
                assert s.append(base + a, b - a).error == 0
            assert s.flush().error == 0
            cursor = s.cursor()
        finally:
            s.close()
        got = sink.shards()
    finally:
        sink.close()
    want, cw = H.run_oracle(cfg, data, quirks=False)
    assert cursor == cw
    assert got == want, H.diff_shards(got, want)


def _append_device_fn():
    import ctypes as C
    import chucky_gb300 as cg
    lib = cg.load()
    f = lib.tile_stream_gpu_append_device
    f.restype = capi.WriterResult
    f.argtypes = [C.c_void_p, capi.Slice, C.c_void_p]
    return f


@pytest.mark.parametrize("name,dtype", [("sensor_dim0", "u16"), ("lod2d_tiles", "f32"),
                                        ("rank5_batched", "u16")])
def test_gpu_append_device_is_stream_ordered(name, dtype):
    """tile_stream_gpu_append_device with the caller's stream: one device
    buffer is refilled on that stream before each append (by an
    asynchronous copy) and overwritten right after it; the copies must see
    each fill and finish before the overwrite."""
    import torch
    import chucky_gb300 as cg
    case = cases.CASES[[c[0] for c in cases.CASES].index(name)]
    cfg, epochs = cases.build(case, dtype)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=31)
    raw = data.view(np.uint8).reshape(-1)
    bpe = capi.BPE[dtype]
    cuts = [0] + _pieces(raw.size, bpe, 8) + [raw.size]
    host = torch.from_numpy(raw.copy()).pin_memory()
    buf = torch.empty(max(b - a for a, b in zip(cuts[:-1], cuts[1:])) + 16,
                      dtype=torch.uint8, device="cuda")
    side = torch.cuda.Stream()
    append_device = _append_device_fn()
    sink = H.MemSink()
    try:
        s = cg.GpuStream(cfg, sink.base)
        try:
            for a, b in zip(cuts[:-1], cuts[1:]):
                with torch.cuda.stream(side):
                    buf[:b - a].copy_(host[a:b], non_blocking=True)
                r = append_device(s.h, capi.Slice(buf.data_ptr(), buf.data_ptr() + b - a),
                                  side.cuda_stream)
                assert r.error == 0
                with torch.cuda.stream(side):
                    buf.fill_(0xAB)
            assert s.flush().error == 0
            side.synchronize()
        finally:
            s.close()
        got = sink.shards()
    finally:
        sink.close()
    want, _ = H.run_oracle(cfg, data, quirks=False)
    assert got == want, H.diff_shards(got, want)


def test_gpu_append_device_rejects_host_memory():
    import torch
    import chucky_gb300 as cg
    case = cases.CASES[[c[0] for c in cases.CASES].index("xval_basic")]
    cfg, _ = cases.build(case, "u16")
    append_device = _append_device_fn()
    host = np.zeros(64, dtype=np.uint8)
    sink = H.MemSink()
    side = torch.cuda.Stream()
    try:
        s = cg.GpuStream(cfg, sink.base)
        try:
            r = append_device(s.h, capi.Slice(host.ctypes.data, host.ctypes.data + 64),
                              side.cuda_stream)
            assert r.error == 1
        finally:
            s.close()
    finally:
        sink.close()


@pytest.mark.parametrize("pieces", ["frames", "whole"])
@pytest.mark.parametrize("name", ["cube_multiscale", "unbounded_frames", "lod2d_tiles"])
def test_gpu_pinned_appends(name, pieces):
    """Pinned host memory: frame-sized appends go through the staging ring,
    whole-array appends straight to the epoch buffer."""
    import torch
    import chucky_gb300 as cg
    case = cases.CASES[[c[0] for c in cases.CASES].index(name)]
    cfg, epochs = cases.build(case, "u16")
    ee = H.epoch_elements(cfg)
    n = int(epochs * ee)
    data = cases.make_data("u16", n, seed=41)
    host = torch.from_numpy(data.view(np.uint8).reshape(-1).copy()).pin_memory()
    frame = int(np.prod([cfg.dimensions[d].size or 1 for d in range(1, cfg.rank)])) * 2
    step = frame if pieces == "frames" else host.numel()
    sink = H.MemSink()
    try:
        s = cg.GpuStream(cfg, sink.base)
        try:
            base = host.data_ptr()
            for a in range(0, host.numel(), step):
                b = min(host.numel(), a + step)
                assert s.append(base + a, b - a).error == 0
            assert s.flush().error == 0
        finally:
            s.close()
        got = sink.shards()
    finally:
        sink.close()
    want, _ = H.run_oracle(cfg, data, quirks=False)
    assert got == want, H.diff_shards(got, want)
