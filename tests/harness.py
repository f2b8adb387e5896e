"""Test-side helpers: run the CPU oracle, the reference CPU backend (when it
was built here) and this library's GPU stream on the same input, and collect
the shard files each of them delivers.

Only tests import this module.  It reads the oracle as the checker.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from chucky_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libchucky_ref.so")

_oracle = None
_ref = None


def oracle():
    """The C restatement (built on demand with make)."""
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"],
                           check=True)
        lib = C.CDLL(ORACLE_SO)
        P = C.c_void_p
        lib.oracle_stream_create.restype = P
        lib.oracle_stream_create.argtypes = [C.POINTER(capi.StreamConfiguration), P]
        lib.oracle_stream_writer.restype = C.POINTER(capi.Writer)
        lib.oracle_stream_writer.argtypes = [P]
        lib.oracle_stream_destroy.argtypes = [P]
        lib.oracle_stream_cursor.restype = C.c_uint64
        lib.oracle_stream_cursor.argtypes = [P]
        lib.oracle_stream_layout.restype = C.POINTER(capi.StreamLayout)
        lib.oracle_stream_layout.argtypes = [P]
        lib.oracle_mem_sink_create.restype = P
        lib.oracle_mem_sink_destroy.argtypes = [P]
        lib.oracle_mem_sink_base.restype = P
        lib.oracle_mem_sink_base.argtypes = [P]
        lib.oracle_mem_sink_count.restype = C.c_size_t
        lib.oracle_mem_sink_count.argtypes = [P]
        lib.oracle_mem_sink_at.argtypes = [
            P, C.c_size_t, C.POINTER(C.c_uint8), C.POINTER(C.c_uint64),
            C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_size_t),
            C.POINTER(C.c_int)]
        lib.oracle_null_sink_create.restype = P
        lib.oracle_null_sink_destroy.argtypes = [P]
        lib.oracle_null_sink_bytes.restype = C.c_uint64
        lib.oracle_null_sink_bytes.argtypes = [P]
        lib.oracle_crc32c.restype = C.c_uint32
        lib.oracle_crc32c.argtypes = [P, C.c_size_t]
        for f in (lib.oracle_zstd_decompress, lib.oracle_lz4_decompress):
            f.restype = C.c_size_t
            f.argtypes = [P, C.c_size_t, P, C.c_size_t]
        lib.oracle_morton_rank.restype = C.c_uint64
        lib.oracle_morton_rank.argtypes = [C.c_int, C.POINTER(C.c_uint64),
                                           C.POINTER(C.c_uint64), C.c_int]
        lib.oracle_reduce_window.argtypes = [P, P, C.c_uint64, C.c_int, C.c_int]
        lib.oracle_fold.argtypes = [P, P, C.c_uint64, C.c_uint32, C.c_int,
                                    C.c_int, C.c_int]
        lib.oracle_emit.argtypes = [P, P, C.c_uint64, C.c_uint32, C.c_int, C.c_int]
        lib.oracle_set_reference_quirks.argtypes = [C.c_int]
        _oracle = lib
    return _oracle


def reference():
    """The reference CPU backend compiled from its own sources, or None."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        lib = C.CDLL(REF_SO)
        P = C.c_void_p
        lib.tile_stream_cpu_create.restype = P
        lib.tile_stream_cpu_create.argtypes = [C.POINTER(capi.StreamConfiguration), P]
        lib.tile_stream_cpu_writer.restype = C.POINTER(capi.Writer)
        lib.tile_stream_cpu_writer.argtypes = [P]
        lib.tile_stream_cpu_destroy.argtypes = [P]
        lib.tile_stream_cpu_cursor.restype = C.c_uint64
        lib.tile_stream_cpu_cursor.argtypes = [P]
        lib.tile_stream_cpu_layout.restype = C.POINTER(capi.StreamLayout)
        lib.tile_stream_cpu_layout.argtypes = [P]
        _ref = lib
    return _ref


class MemSink:
    """The oracle's in-memory shard sink (works with any implementation of
    the shard_sink ABI)."""

    def __init__(self):
        self.lib = oracle()
        self.h = self.lib.oracle_mem_sink_create()
        self.base = self.lib.oracle_mem_sink_base(self.h)

    def shards(self):
        out = {}
        n = self.lib.oracle_mem_sink_count(self.h)
        lv, idx = C.c_uint8(), C.c_uint64()
        data, size, fin = C.POINTER(C.c_uint8)(), C.c_size_t(), C.c_int()
        for i in range(n):
            self.lib.oracle_mem_sink_at(self.h, i, C.byref(lv), C.byref(idx),
                                        C.byref(data), C.byref(size), C.byref(fin))
            if size.value == 0:
                continue
            out[(lv.value, idx.value)] = (C.string_at(data, size.value), bool(fin.value))
        return out

    def close(self):
        if self.h:
            self.lib.oracle_mem_sink_destroy(self.h)
            self.h = None


def _drive(writer, data, pieces):
    """Append `data` (bytes-like numpy array) in `pieces` slices, then flush."""
    buf = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
    base = buf.ctypes.data
    n = buf.size
    if pieces is None:
        cuts = [0, n]
    else:
        cuts = sorted(set([0, n] + [int(c) for c in pieces if 0 < c < n]))
    w = writer.contents
    for a, b in zip(cuts[:-1], cuts[1:]):
        r = w.append(writer, capi.Slice(base + a, base + b))
        if r.error != 0:
            raise RuntimeError(f"append failed error={r.error}")
    r = w.flush(writer)
    if r.error != 0:
        raise RuntimeError(f"flush failed error={r.error}")


def run_oracle(cfg, data, pieces=None, quirks=True):
    lib = oracle()
    lib.oracle_set_reference_quirks(1 if quirks else 0)
    sink = MemSink()
    try:
        s = lib.oracle_stream_create(C.byref(cfg), sink.base)
        if not s:
            raise RuntimeError("oracle_stream_create failed")
        try:
            _drive(lib.oracle_stream_writer(s), data, pieces)
            cursor = lib.oracle_stream_cursor(s)
        finally:
            lib.oracle_stream_destroy(s)
        return sink.shards(), cursor
    finally:
        sink.close()
        lib.oracle_set_reference_quirks(1)


def run_reference(cfg, data, pieces=None):
    lib = reference()
    sink = MemSink()
    try:
        s = lib.tile_stream_cpu_create(C.byref(cfg), sink.base)
        if not s:
            raise RuntimeError("tile_stream_cpu_create failed")
        try:
            _drive(lib.tile_stream_cpu_writer(s), data, pieces)
            cursor = lib.tile_stream_cpu_cursor(s)
        finally:
            lib.tile_stream_cpu_destroy(s)
        return sink.shards(), cursor
    finally:
        sink.close()


def parse_shard(blob, n_slots, alignment=0):
    """Split a shard file into (index entries, crc ok).  The index is the
    trailing 16*n_slots bytes + crc32c (little endian)."""
    lib = oracle()
    idx_bytes = 16 * n_slots
    tail = blob[-(idx_bytes + 4):]
    index = np.frombuffer(tail[:idx_bytes], dtype="<u8").reshape(-1, 2)
    crc = int.from_bytes(tail[idx_bytes:], "little")
    buf = C.create_string_buffer(tail[:idx_bytes], idx_bytes)
    ok = lib.oracle_crc32c(buf, idx_bytes) == crc
    return index, ok


def run_gpu(cfg, data, pieces=None, deadline_ms=None):
    """This library's GPU stream on the same input (needs a GPU); with
    `deadline_ms`, the stream's batch deadline (partial batches)."""
    import chucky_gb300 as cg
    sink = MemSink()
    try:
        s = cg.GpuStream(cfg, sink.base)
        if deadline_ms is not None:
            s.lib.tile_stream_gpu_set_batch_deadline.argtypes = [C.c_void_p, C.c_double]
            if s.lib.tile_stream_gpu_set_batch_deadline(s.h, float(deadline_ms)) != 0:
                raise RuntimeError("tile_stream_gpu_set_batch_deadline failed")
        try:
            _drive(s.writer, data, pieces)
            cursor = s.cursor()
        finally:
            s.close()
        return sink.shards(), cursor
    finally:
        sink.close()


def epoch_elements(cfg):
    """Elements per epoch, from the oracle's plan."""
    lib = oracle()
    sink = MemSink()
    try:
        s = lib.oracle_stream_create(C.byref(cfg), sink.base)
        if not s:
            raise RuntimeError("invalid config")
        ee = lib.oracle_stream_layout(s).contents.epoch_elements
        lib.oracle_stream_destroy(s)
        return ee
    finally:
        sink.close()


def diff_shards(a, b):
    """Human-readable list of differing shard keys."""
    out = []
    for k in sorted(set(a) | set(b)):
        x, y = a.get(k), b.get(k)
        if x != y:
            if x is None or y is None:
                out.append(f"{k}: present only in {'b' if x is None else 'a'}")
            elif x[0] != y[0]:
                n = min(len(x[0]), len(y[0]))
                first = next((i for i in range(n) if x[0][i] != y[0][i]), n)
                out.append(f"{k}: sizes {len(x[0])}/{len(y[0])} first diff at {first}")
            else:
                out.append(f"{k}: finalized {x[1]}/{y[1]}")
    return out


class _Info(C.Structure):
    _fields_ = [("nlod", C.c_int), ("append_downsample", C.c_int),
                ("epochs_per_batch", C.c_uint32), ("total_chunks", C.c_uint64),
                ("chunk_elements", C.c_uint64), ("epoch_elements", C.c_uint64),
                ("max_output_size", C.c_uint64),
                ("lod_nelem", C.c_uint64 * 32), ("level_chunks", C.c_uint64 * 32),
                ("shard_inner_count", C.c_uint64 * 32),
                ("chunks_per_shard_total", C.c_uint64 * 32),
                ("chunks_per_shard_append", C.c_uint64 * 32),
                ("fixed_dims_count", C.c_uint64)]


def plan_info(cfg):
    lib = oracle()
    lib.oracle_stream_info.argtypes = [C.c_void_p, C.POINTER(_Info)]
    sink = MemSink()
    try:
        s = lib.oracle_stream_create(C.byref(cfg), sink.base)
        info = _Info()
        lib.oracle_stream_info(s, C.byref(info))
        lib.oracle_stream_destroy(s)
        return info
    finally:
        sink.close()


def decode(codec, blob, raw_size):
    lib = oracle()
    src = C.create_string_buffer(blob, len(blob))
    dst = C.create_string_buffer(raw_size + 64)
    if codec == "zstd":
        n = lib.oracle_zstd_decompress(dst, raw_size + 64, src, len(blob))
    else:
        n = lib.oracle_lz4_decompress(dst, raw_size, src, len(blob))
    if n == C.c_size_t(-1).value:
        raise ValueError(f"{codec} decode failed")
    return dst.raw[:n]


def compare_decoded(cfg_codec, shards_codec, shards_raw, codec):
    """Decode every chunk of the compressed shards with the stock library and
    compare with the raw chunk bytes of the CODEC_NONE shards.  Returns
    (number of chunks checked, compressed bytes, raw bytes)."""
    info = plan_info(cfg_codec)
    chunk_bytes = info.chunk_elements * {1: 1}.get(0, 1)
    assert set(shards_codec) == set(shards_raw), (sorted(shards_codec), sorted(shards_raw))
    checked = comp_total = raw_total = 0
    for key, (blob, fin) in shards_codec.items():
        raw_blob, raw_fin = shards_raw[key]
        assert fin and raw_fin
        nslots = info.chunks_per_shard_total[key[0]]
        idx_c, ok_c = parse_shard(blob, nslots)
        idx_r, ok_r = parse_shard(raw_blob, nslots)
        assert ok_c and ok_r, "index crc32c mismatch"
        for (oc, nc), (orr, nr) in zip(idx_c.tolist(), idx_r.tolist()):
            empty_c = oc == 0xFFFFFFFFFFFFFFFF and nc == 0xFFFFFFFFFFFFFFFF
            empty_r = orr == 0xFFFFFFFFFFFFFFFF and nr == 0xFFFFFFFFFFFFFFFF
            assert empty_c == empty_r
            if empty_c:
                continue
            raw = raw_blob[orr:orr + nr]
            got = decode(codec, blob[oc:oc + nc], len(raw))
            assert got == raw, f"chunk mismatch in shard {key}"
            checked += 1
            comp_total += nc
            raw_total += nr
    return checked, comp_total, raw_total


def run_into(impl, cfg, data, sink_base, pieces=None, quirks=True):
    """Drive implementation `impl` ("oracle", "reference" or "gpu") into an
    arbitrary shard_sink; returns the stream's final cursor."""
    if impl == "oracle":
        lib = oracle()
        lib.oracle_set_reference_quirks(1 if quirks else 0)
        try:
            s = lib.oracle_stream_create(C.byref(cfg), sink_base)
            if not s:
                raise RuntimeError("oracle_stream_create failed")
            try:
                _drive(lib.oracle_stream_writer(s), data, pieces)
                return lib.oracle_stream_cursor(s)
            finally:
                lib.oracle_stream_destroy(s)
        finally:
            lib.oracle_set_reference_quirks(1)
    if impl == "reference":
        lib = reference()
        s = lib.tile_stream_cpu_create(C.byref(cfg), sink_base)
        if not s:
            raise RuntimeError("tile_stream_cpu_create failed")
        try:
            _drive(lib.tile_stream_cpu_writer(s), data, pieces)
            return lib.tile_stream_cpu_cursor(s)
        finally:
            lib.tile_stream_cpu_destroy(s)
    import chucky_gb300 as cg
    s = cg.GpuStream(cfg, sink_base)
    try:
        _drive(s.writer, data, pieces)
        return s.cursor()
    finally:
        s.close()
