"""The device LZ4 decoder (chucky_lz4_decode_chunks): blocks written by this
library's GPU encoder and blocks written by the stock liblz4
(LZ4_compress_default) decode on the GPU to the original chunk bytes; a
block cut short reports an error status instead of a result."""
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
