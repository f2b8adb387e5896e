"""The allocation-free LZ4 entry point (chucky_lz4_encode_chunks_static)
against the stream's own LZ4 output.

A 2-D u16 array whose chunks span whole rows (x is one chunk wide) has each
chunk's bytes contiguous in the input, so the stream's compressed chunks
(read back from its shards) and the static entry point run on the raw input
must agree byte for byte.  Calls run back to back on one CUDA stream with
different inputs and chunk sizes: stale scratch from one call must not leak
into the next.  This file sorts last so that it also runs after every other
GPU test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

from chucky_gb300 import capi, load
from harness import decode, parse_shard, run_gpu

CPS = 4  # chunks per shard along t
PAD = 256  # readable bytes required after the last chunk


def _lib():
    lib = load()
    f = lib.chucky_lz4_encode_chunks_static
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t,
                  C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    lib.chucky_lz4_static_scratch_bytes.restype = C.c_size_t
    return lib


def _bound(n):
    return n + n // 255 + 16


def _data(seed, rows, width):
    """Sensor-like u16 rows: Poisson noise, flat runs, a ramp, a zero band."""
    rng = np.random.default_rng(seed)
    x = rng.poisson(100, size=(rows, width)).astype("<u2")
    x[:, : width // 8] = 7
    x[rows // 3: rows // 3 + 2] = 0
    x[:, width - width // 16:] = (np.arange(width // 16, dtype="<u2") * 3)[None, :]
    return x


def _stream_chunks(x, chunk_rows):
    """Compressed chunks in t order, from the stream's shards."""
    rows, width = x.shape
    dims = capi.make_dims([dict(size=rows, chunk=chunk_rows, cps=CPS, name="t"),
                           dict(size=width, chunk=width, cps=1, name="x")])
    cfg = capi.make_config(dims, dtype="u16", codec="lz4", level=1)
    cfg._dims = dims
    shards, _ = run_gpu(cfg, x)
    n_chunks = rows // chunk_rows
    out = []
    for s in range((n_chunks + CPS - 1) // CPS):
        blob, _ = shards[(0, s)]
        index, ok = parse_shard(blob, CPS)
        assert ok
        for j in range(min(CPS, n_chunks - s * CPS)):
            off, nb = (int(v) for v in index[j])
            out.append(blob[off: off + nb])
    return out


def _static_chunks(lib, d_in, chunk_bytes, n_chunks, torch, offset=0, in_stride=None):
    in_stride = in_stride or chunk_bytes
    out_stride = (_bound(chunk_bytes) + 255) // 256 * 256
    d_out = torch.empty(n_chunks * out_stride, dtype=torch.uint8, device="cuda")
    d_sizes = torch.zeros(n_chunks, dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream()
    rc = lib.chucky_lz4_encode_chunks_static(
        d_in.data_ptr() + offset, chunk_bytes, in_stride, n_chunks,
        d_out.data_ptr(), out_stride, d_sizes.data_ptr(), st.cuda_stream)
    assert rc == 0
    st.synchronize()
    out = d_out.cpu().numpy()
    sizes = d_sizes.cpu().numpy()
    return [out[i * out_stride: i * out_stride + int(sizes[i])].tobytes()
            for i in range(n_chunks)]


def _device_input(x, torch):
    raw = np.concatenate([x.view(np.uint8).reshape(-1), np.zeros(PAD, np.uint8)])
    return torch.from_numpy(raw).cuda()


@pytest.mark.gpu
def test_static_lz4_matches_stream_back_to_back():
    torch = pytest.importorskip("torch")
    lib = _lib()
    # (seed, rows, width, chunk rows): 256 KiB chunks, and 49156-byte
    # chunks (not a multiple of the 16 KiB segment or of 256 bytes)
    cases = [(11, 128, 8192, 16), (12, 40, 24578, 1)]
    expect, inputs = [], []
    for seed, rows, width, cr in cases:
        x = _data(seed, rows, width)
        expect.append(_stream_chunks(x, cr))
        inputs.append((x, cr))
    # two calls in a row per input, alternating inputs and chunk sizes
    for k in (0, 1, 0, 1):
        x, cr = inputs[k]
        chunk_bytes = cr * x.shape[1] * 2
        n_chunks = x.shape[0] // cr
        got = _static_chunks(lib, _device_input(x, torch), chunk_bytes, n_chunks, torch)
        assert len(got) == len(expect[k])
        for i, (g, e) in enumerate(zip(got, expect[k])):
            assert g == e, f"input {k} chunk {i}: {len(g)} vs {len(e)} bytes"
        raw = x.view(np.uint8).reshape(-1)
        assert decode("lz4", got[-1], chunk_bytes) == \
            raw[(n_chunks - 1) * chunk_bytes: n_chunks * chunk_bytes].tobytes()


@pytest.mark.gpu
def test_static_lz4_gapped_input_at_a_4_byte_offset():
    """Chunks 4 bytes past a 16-byte boundary with 12 bytes of other data
    between them (in_stride = chunk_bytes + 12): the encoder's 4-byte input
    path, checked against the stream's output for the same chunk bytes."""
    torch = pytest.importorskip("torch")
    lib = _lib()
    x = _data(12, 40, 24578)  # 49156-byte chunks, one row each
    expect = _stream_chunks(x, 1)
    chunk_bytes = x.shape[1] * 2
    n_chunks = x.shape[0]
    stride = chunk_bytes + 12
    rng = np.random.default_rng(3)
    raw = rng.integers(0, 256, size=4 + n_chunks * stride + PAD, dtype=np.uint8)
    rows = x.view(np.uint8).reshape(n_chunks, chunk_bytes)
    for i in range(n_chunks):
        raw[4 + i * stride: 4 + i * stride + chunk_bytes] = rows[i]
    d_in = torch.from_numpy(raw).cuda()
    for _ in range(2):
        got = _static_chunks(lib, d_in, chunk_bytes, n_chunks, torch, offset=4,
                             in_stride=stride)
        assert len(got) == len(expect)
        for i, (g, e) in enumerate(zip(got, expect)):
            assert g == e, f"chunk {i}: {len(g)} vs {len(e)} bytes"


def test_static_lz4_rejects_requests_beyond_the_fixed_scratch():
    lib = _lib()
    cap = lib.chucky_lz4_static_scratch_bytes()
    assert cap == 32 << 20
    chunk = 1 << 20
    fake = 1 << 20  # never dereferenced: the request is rejected first
    # 64 MiB of input needs far more scratch than the fixed array
    assert lib.chucky_lz4_encode_chunks_static(
        fake, chunk, chunk, 64, fake, _bound(chunk), fake, None) == 2
    assert lib.chucky_lz4_encode_chunks_static(
        fake, chunk, chunk, 1, fake, chunk, fake, None) == 1  # out_stride too small
    assert lib.chucky_lz4_encode_chunks_static(
        fake + 1, chunk, chunk, 1, fake, _bound(chunk), fake, None) == 1  # misaligned
    assert lib.chucky_lz4_encode_chunks_static(
        fake, chunk, chunk, 0, fake, _bound(chunk), fake, None) == 0  # nothing to do
    # chunk counts whose scratch size overflows 64 bits are rejected too
    for n in (1 << 44, 1 << 50, (1 << 64) - 1):
        assert lib.chucky_lz4_encode_chunks_static(
            fake, chunk, chunk, n, fake, _bound(chunk), fake, None) == 2
