"""The device decoders.

* LZ4 (chucky_lz4_decode_chunks): blocks written by this library's GPU
  encoder and by the stock liblz4 (LZ4_compress_default) decode on the GPU
  to the original chunk bytes; a block cut short reports an error status.
* zstd (chucky_zstd_decode_chunks): frames written by this library's GPU
  encoder and by the stock libzstd at levels 1, 3 and 19 (and two frames
  one after another, a skippable frame before one) decode to the original
  chunk bytes; frames cut short or with bytes flipped report an error
  status instead of a result."""
import ctypes as C

import numpy as np
import pytest

from chucky_gb300 import load

pytestmark = pytest.mark.gpu


def _lib():
    lib = load()
    lib.chucky_lz4_encode_chunks_static.argtypes = [
        C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t,
        C.c_void_p, C.c_void_p]
    lib.chucky_lz4_decode_chunks.argtypes = [
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
        C.c_size_t, C.c_void_p, C.c_void_p]
    return lib


def _chunks(n, chunk, seed):
    """Poisson noise, flat runs, zeros and a repeating ramp, per chunk."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, chunk), dtype=np.uint8)
    for i in range(n):
        k = i % 4
        if k == 0:
            out[i] = rng.poisson(100, size=chunk // 2).astype("<u2").view(np.uint8)
        elif k == 1:
            out[i] = 0
        elif k == 2:
            out[i] = np.arange(chunk) % 13
        else:
            out[i] = rng.integers(0, 256, size=chunk, dtype=np.uint8)
            out[i, : chunk // 3] = 5
    return out


def _decode(lib, blob_dev, offs, lens, n, chunk):
    import torch
    d_off = torch.tensor(offs, dtype=torch.int64, device="cuda")
    d_len = torch.tensor(lens, dtype=torch.int64, device="cuda")
    out = torch.zeros(n * chunk, dtype=torch.uint8, device="cuda")
    st = torch.full((n,), 99, dtype=torch.int32, device="cuda")
    rc = lib.chucky_lz4_decode_chunks(blob_dev.data_ptr(), d_off.data_ptr(), d_len.data_ptr(),
                                      n, out.data_ptr(), chunk, chunk, st.data_ptr(),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(n, chunk), st.cpu().numpy()


def test_decodes_own_encoder_output():
    import torch
    lib = _lib()
    n, chunk = 16, 65536
    x = _chunks(n, chunk, 1)
    d_in = torch.zeros(n * chunk + 256, dtype=torch.uint8, device="cuda")
    d_in[: n * chunk] = torch.from_numpy(x.reshape(-1)).cuda()
    stride = (chunk + chunk // 255 + 16 + 15) // 16 * 16
    d_out = torch.empty(n * stride, dtype=torch.uint8, device="cuda")
    d_sizes = torch.zeros(n, dtype=torch.int64, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.chucky_lz4_encode_chunks_static(d_in.data_ptr(), chunk, chunk, n,
                                               d_out.data_ptr(), stride,
                                               d_sizes.data_ptr(), s) == 0
    torch.cuda.synchronize()
    sizes = d_sizes.cpu().numpy().tolist()
    got, st = _decode(lib, d_out, [i * stride for i in range(n)], sizes, n, chunk)
    assert (st == 0).all()
    assert np.array_equal(got, x)


def test_decodes_stock_lz4_blocks_and_rejects_a_cut_block():
    import torch
    lib = _lib()
    lz4 = C.CDLL("liblz4.so.1")
    lz4.LZ4_compress_default.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int]
    n, chunk = 8, 100000
    x = _chunks(n, chunk, 2)
    blobs = []
    for i in range(n):
        cap = chunk + chunk // 255 + 16
        buf = C.create_string_buffer(cap)
        k = lz4.LZ4_compress_default(x[i].tobytes(), buf, chunk, cap)
        assert k > 0
        blobs.append(buf.raw[:k])
    offs, pos = [], 0
    for b in blobs:
        offs.append(pos)
        pos += len(b)
    flat = np.frombuffer(b"".join(blobs), dtype=np.uint8)
    dev = torch.from_numpy(flat.copy()).cuda()
    lens = [len(b) for b in blobs]
    got, st = _decode(lib, dev, offs, lens, n, chunk)
    assert (st == 0).all()
    assert np.array_equal(got, x)
    # the same blocks, each one byte short: every one must fail
    _, st = _decode(lib, dev, offs, [m - 1 for m in lens], n, chunk)
    assert (st != 0).all()


def _zstd_lib():
    lib = load()
    lib.chucky_zstd_decode_chunks.argtypes = [
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
        C.c_size_t, C.c_void_p, C.c_void_p]
    lib.chucky_encode_chunks.argtypes = [
        C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_void_p,
        C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.chucky_encode_bound.restype = C.c_size_t
    lib.chucky_encode_bound.argtypes = [C.c_int, C.c_size_t]
    lib.chucky_encode_scratch_bytes.restype = C.c_size_t
    lib.chucky_encode_scratch_bytes.argtypes = [C.c_int, C.c_int, C.c_size_t, C.c_size_t]
    return lib


def _zstd_decode(lib, blobs, chunk):
    import torch
    offs, pos = [], 0
    for b in blobs:
        offs.append(pos)
        pos += len(b)
    flat = np.frombuffer(b"".join(blobs) + b"\0" * 8, dtype=np.uint8)
    dev = torch.from_numpy(flat.copy()).cuda()
    n = len(blobs)
    d_off = torch.tensor(offs, dtype=torch.int64, device="cuda")
    d_len = torch.tensor([len(b) for b in blobs], dtype=torch.int64, device="cuda")
    out = torch.zeros(n * chunk, dtype=torch.uint8, device="cuda")
    st = torch.full((n,), 99, dtype=torch.int32, device="cuda")
    rc = lib.chucky_zstd_decode_chunks(dev.data_ptr(), d_off.data_ptr(), d_len.data_ptr(),
                                       n, out.data_ptr(), chunk, chunk, st.data_ptr(),
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(n, chunk), st.cpu().numpy()


def _zstd_compress(x, level):
    z = C.CDLL("libzstd.so.1")
    z.ZSTD_compressBound.restype = C.c_size_t
    z.ZSTD_compressBound.argtypes = [C.c_size_t]
    z.ZSTD_compress.restype = C.c_size_t
    z.ZSTD_compress.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.c_int]
    cap = z.ZSTD_compressBound(len(x))
    buf = C.create_string_buffer(cap)
    k = z.ZSTD_compress(buf, cap, x, len(x), level)
    assert k < cap
    return buf.raw[:k]


@pytest.mark.parametrize("level", [1, 3])
def test_zstd_decodes_own_encoder_output(level):
    """Level 3 frames carry FSE-described sequence tables in the first
    block with sequences and repeat them in later blocks."""
    import torch
    lib = _zstd_lib()
    n, chunk = 16, 200000  # several 8 KiB zstd blocks and Huffman streams per chunk
    x = _chunks(n, chunk, 3)
    d_in = torch.zeros(n * chunk + 256, dtype=torch.uint8, device="cuda")
    d_in[: n * chunk] = torch.from_numpy(x.reshape(-1)).cuda()
    bound = lib.chucky_encode_bound(2, chunk)
    stride = (bound + 15) // 16 * 16
    d_out = torch.empty(n * stride, dtype=torch.uint8, device="cuda")
    d_sizes = torch.zeros(n, dtype=torch.int64, device="cuda")
    sb = lib.chucky_encode_scratch_bytes(2, level, chunk, n)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.chucky_encode_chunks(2, level, d_in.data_ptr(), chunk, chunk, n,
                                    d_out.data_ptr(), stride, d_sizes.data_ptr(),
                                    scratch.data_ptr(), sb, s) == 0
    torch.cuda.synchronize()
    sizes = d_sizes.cpu().numpy().tolist()
    raw = d_out.cpu().numpy()
    blobs = [raw[i * stride: i * stride + sizes[i]].tobytes() for i in range(n)]
    got, st = _zstd_decode(lib, blobs, chunk)
    assert (st == 0).all(), st
    assert np.array_equal(got, x)


@pytest.mark.parametrize("level", [1, 3, 19])
def test_zstd_decodes_stock_frames(level):
    lib = _zstd_lib()
    n, chunk = 8, 150000
    x = _chunks(n, chunk, 4 + level)
    blobs = [_zstd_compress(x[i].tobytes(), level) for i in range(n)]
    got, st = _zstd_decode(lib, blobs, chunk)
    assert (st == 0).all(), st
    assert np.array_equal(got, x)


def test_zstd_frame_sequences_and_skippable_frames():
    lib = _zstd_lib()
    chunk = 120000
    x = _chunks(2, chunk // 2, 9).reshape(-1)  # two halves
    a = _zstd_compress(x[: chunk // 2].tobytes(), 3)
    b = _zstd_compress(x[chunk // 2:].tobytes(), 1)
    skip = (0x184D2A53).to_bytes(4, "little") + (5).to_bytes(4, "little") + b"hello"
    got, st = _zstd_decode(lib, [a + b, skip + a + b], chunk)
    assert (st == 0).all(), st
    assert np.array_equal(got[0], x) and np.array_equal(got[1], x)


def test_zstd_rejects_malformed_frames():
    lib = _zstd_lib()
    chunk = 100000
    x = _chunks(4, chunk, 5)
    good = [_zstd_compress(x[i].tobytes(), 3) for i in range(4)]
    rng = np.random.default_rng(1)
    bad = [g[: len(g) - 1] for g in good] + [g[: len(g) // 2] for g in good]
    bad.append(rng.integers(0, 256, size=5000, dtype=np.uint8).tobytes())
    _, st = _zstd_decode(lib, bad, chunk)
    assert (st != 0).all(), st
    assert (st <= 5).all()
    # bytes flipped: any status, never a fault (decoded frames are checked)
    flipped = []
    for t in range(64):
        g = bytearray(good[t % 4])
        g[int(rng.integers(0, len(g)))] ^= int(rng.integers(1, 256))
        flipped.append(bytes(g))
    got, st = _zstd_decode(lib, flipped, chunk)
    assert (st <= 5).all()
