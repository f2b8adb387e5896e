"""Failure handling, driven from the host (no GPU fault is ever made).

* Sinks that fail: `open` returns NULL, or `write` / `finalize` returns an
  error at its N-th call.  The stream must report `writer_error_fail` from an
  append or the flush (never a clean flush), and destroy cleanly afterwards.
  The reference CPU backend (src/zarr/shard_delivery.c:133-135 checks
  `open`; writes and finalize propagate their return codes,
  src/zarr/shard_delivery.c:36-102, 145-170) fixes the contract; the oracle
  and the GPU stream are held to it.
* Appending after the flush returns `writer_error_finished` with the whole
  input as `rest` (src/gpu/stream.c:71-72, src/cpu/stream.c:530-531).
* A bounded array stops at its capacity: the append that crosses it is cut
  at the last element that fits, the stream flushes itself and the result is
  `writer_error_finished` with the unconsumed input as `rest`
  (src/gpu/stream.c:83-88); the shards equal those of exactly the array's
  elements.
* `writer_append_wait` backs off while a writer consumes nothing and gives
  up after 10 stalls in a row (src/writer.c:19-45).

The CPU implementations (oracle, reference build) run everywhere; the GPU
stream's cases are marked gpu.
"""
import ctypes as C
import time

import numpy as np
import pytest

import cases
import harness as H
from chucky_gb300 import capi

IMPLS = [
    pytest.param("oracle", id="oracle"),
    pytest.param("reference", id="reference",
                 marks=pytest.mark.skipif(H.reference() is None,
                                          reason="reference build not present")),
    pytest.param("gpu", id="gpu", marks=pytest.mark.gpu),
]

OPEN_FN = C.CFUNCTYPE(C.c_void_p, C.c_void_p, C.c_uint8, C.c_uint64)
WRITE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p)
FIN_FN = C.CFUNCTYPE(C.c_int, C.c_void_p)


class _ShardWriter(C.Structure):
    _fields_ = [("write", WRITE_FN), ("write_direct", C.c_void_p), ("finalize", FIN_FN)]


class _ShardSink(C.Structure):
    _fields_ = [("open", OPEN_FN), ("update_append", C.c_void_p),
                ("record_fence", C.c_void_p), ("wait_fence", C.c_void_p)]


class FaultySink:
    """A shard_sink whose `fail` operation ("open", "write" or "finalize")
    fails at its `at`-th call (1-based) and every call after it.  Counts
    the calls of each operation."""

    def __init__(self, fail=None, at=1):
        self.fail, self.at = fail, at
        self.calls = {"open": 0, "write": 0, "finalize": 0}
        self._open = OPEN_FN(self._on_open)
        self._write = WRITE_FN(self._on_write)
        self._fin = FIN_FN(self._on_finalize)
        self.writer = _ShardWriter(self._write, None, self._fin)
        self.sink = _ShardSink(self._open, None, None, None)

    def _hit(self, op):
        self.calls[op] += 1
        return self.fail == op and self.calls[op] >= self.at

    def _on_open(self, _sink, _level, _index):
        if self._hit("open"):
            return None
        return C.addressof(self.writer)

    def _on_write(self, _w, _off, _beg, _end):
        return 1 if self._hit("write") else 0

    def _on_finalize(self, _w):
        return 1 if self._hit("finalize") else 0

    @property
    def base(self):
        return C.addressof(self.sink)


class Stream:
    """One stream of the given implementation over a shard_sink address."""

    def __init__(self, impl, cfg, sink_base):
        self.impl, self.cfg = impl, cfg
        if impl == "oracle":
            self.lib = H.oracle()
            self.lib.oracle_set_reference_quirks(1)
            self.h = self.lib.oracle_stream_create(C.byref(cfg), sink_base)
            self.w = self.lib.oracle_stream_writer(self.h) if self.h else None
            self._destroy = self.lib.oracle_stream_destroy
        elif impl == "reference":
            self.lib = H.reference()
            self.h = self.lib.tile_stream_cpu_create(C.byref(cfg), sink_base)
            self.w = self.lib.tile_stream_cpu_writer(self.h) if self.h else None
            self._destroy = self.lib.tile_stream_cpu_destroy
        else:
            import chucky_gb300 as cg
            self.g = cg.GpuStream(cfg, sink_base)
            self.h, self.w = self.g.h, self.g.writer
            self._destroy = lambda h: self.g.close()
        assert self.h, f"{impl}: create failed"

    def append(self, buf, beg=0, end=None):
        end = buf.size if end is None else end
        base = buf.ctypes.data
        r = self.w.contents.append(self.w, capi.Slice(base + int(beg), base + int(end)))
        rest = (0 if r.rest.beg is None else r.rest.beg - base,
                0 if r.rest.end is None else r.rest.end - base)
        return r.error, rest

    def flush(self):
        return self.w.contents.flush(self.w).error

    def destroy(self):
        if self.h:
            self._destroy(self.h)
            self.h = None


def _small_case(codec="none"):
    """A 3-D u16 stream of 6 epochs, 2 epochs per batch, 4 shards per
    epoch, a 2-level pyramid: every shard is opened, written and
    finalized several times."""
    D = dict
    dims = capi.make_dims([D(size=0, chunk=2, cps=2, downsample=1),
                           D(size=16, chunk=8, cps=1, downsample=1),
                           D(size=32, chunk=8, cps=2, downsample=1)])
    cfg = capi.make_config(dims, dtype="u16", codec=codec, level=1, reduce="mean",
                           append_reduce="mean", max_nlod=2, epochs_per_batch=2)
    cfg._dims = dims
    n = 12 * 16 * 32
    data = cases.make_data("u16", n, seed=5).view(np.uint8).reshape(-1)
    return cfg, data


def _run_to_end(s, data, pieces=4):
    """Append in `pieces` slices, stopping at the first error, then flush.
    Returns the errors seen: [(call, code)]."""
    errs = []
    cuts = np.linspace(0, data.size, pieces + 1).astype(int)
    cuts -= cuts % 2
    for a, b in zip(cuts[:-1], cuts[1:]):
        e, _ = s.append(data, a, b)
        if e:
            errs.append(("append", e))
            break
    e = s.flush()
    errs.append(("flush", e))
    return errs


@pytest.mark.parametrize("impl", IMPLS)
@pytest.mark.parametrize("fail,at", [("open", 1), ("open", 5), ("write", 1),
                                     ("write", 7), ("finalize", 1), ("finalize", 3)])
def test_failing_sink_is_reported(impl, fail, at):
    cfg, data = _small_case()
    sink = FaultySink(fail, at)
    s = Stream(impl, cfg, sink.base)
    try:
        errs = _run_to_end(s, data)
    finally:
        s.destroy()  # must not crash with shards left open
    assert sink.calls[fail] >= at, f"{fail} was called only {sink.calls[fail]} times"
    # the failure surfaces as writer_error_fail, at an append or the flush
    assert any(code == 1 for _, code in errs), errs
    assert all(code in (0, 1) for _, code in errs), errs


@pytest.mark.parametrize("impl", IMPLS)
def test_healthy_sink_sees_every_shard_finalized(impl):
    cfg, data = _small_case()
    sink = FaultySink()
    s = Stream(impl, cfg, sink.base)
    try:
        errs = _run_to_end(s, data)
    finally:
        s.destroy()
    assert errs == [("flush", 0)]
    assert sink.calls["open"] == sink.calls["finalize"] > 0


@pytest.mark.parametrize("impl", IMPLS)
def test_append_after_flush_is_finished(impl):
    cfg, data = _small_case()
    sink = H.MemSink()
    s = Stream(impl, cfg, sink.base)
    try:
        e, _ = s.append(data, 0, 1024)
        assert e == 0
        assert s.flush() == 0
        e, rest = s.append(data, 1024, 2048)
        assert e == 2
        assert rest == (1024, 2048)  # nothing consumed
        assert s.flush() in (0, 2)  # a second flush changes nothing
    finally:
        s.destroy()
        sink.close()


@pytest.mark.parametrize("impl", IMPLS)
def test_bounded_array_stops_at_capacity(impl):
    """dim 0 of size 10 (chunk 2): an append of 13 frames consumes 10, the
    stream flushes itself and reports finished with the 3 frames left."""
    D = dict
    dims = capi.make_dims([D(size=10, chunk=2, cps=2), D(size=8, chunk=4, cps=2),
                           D(size=16, chunk=8, cps=1)])
    cfg = capi.make_config(dims, dtype="u16", epochs_per_batch=2)
    cfg._dims = dims
    frame = 8 * 16 * 2
    data = cases.make_data("u16", 13 * 8 * 16, seed=9).view(np.uint8).reshape(-1)
    sink = H.MemSink()
    s = Stream(impl, cfg, sink.base)
    try:
        e, rest = s.append(data)
        assert e == 2
        assert rest == (10 * frame, 13 * frame)
        e, rest = s.append(data, 10 * frame)  # still finished
        assert e == 2 and rest == (10 * frame, 13 * frame)
        got = sink.shards()
    finally:
        s.destroy()
        sink.close()
    want, _ = H.run_oracle(cfg, data[:10 * frame].view("<u2"))
    assert got == want, H.diff_shards(got, want)


# ---- writer_append_wait ----------------------------------------------------

class StallingWriter:
    """The oracle library's test writer (see oracle/oracle.h): consumes
    nothing for its first `stalls` calls, then `chunk` bytes per call (all
    when 0), or fails after the stalls."""

    def __init__(self, stalls, chunk=0, error=False):
        self.lib = H.oracle()
        L = self.lib
        L.oracle_stalling_writer_create.restype = C.c_void_p
        L.oracle_stalling_writer_create.argtypes = [C.c_int, C.c_size_t, C.c_int]
        L.oracle_stalling_writer_destroy.argtypes = [C.c_void_p]
        L.oracle_stalling_writer_base.restype = C.c_void_p
        L.oracle_stalling_writer_base.argtypes = [C.c_void_p]
        L.oracle_stalling_writer_calls.argtypes = [C.c_void_p]
        L.oracle_stalling_writer_time.restype = C.c_double
        L.oracle_stalling_writer_time.argtypes = [C.c_void_p, C.c_int]
        self.h = L.oracle_stalling_writer_create(min(stalls, 1 << 30), chunk, int(error))
        self.base = L.oracle_stalling_writer_base(self.h)

    @property
    def calls(self):
        return self.lib.oracle_stalling_writer_calls(self.h)

    def times(self, n):
        return [self.lib.oracle_stalling_writer_time(self.h, i) for i in range(n)]

    def close(self):
        self.lib.oracle_stalling_writer_destroy(self.h)


def _append_wait(which):
    if which == "ours":
        import chucky_gb300 as cg
        lib = cg.load()
    else:
        lib = H.reference()
        if lib is None:
            pytest.skip("reference build not present")
    f = lib.writer_append_wait
    f.restype = capi.WriterResult
    f.argtypes = [C.c_void_p, capi.Slice]
    return f


@pytest.mark.parametrize("which", ["ours", "reference"])
def test_append_wait_backs_off_then_succeeds(which):
    append_wait = _append_wait(which)
    buf = (C.c_uint8 * 1000)()
    base = C.addressof(buf)
    w = StallingWriter(stalls=4, chunk=300)
    try:
        r = append_wait(w.base, capi.Slice(base, base + 1000))
        assert r.error == 0
        # 4 stalls, then calls of 300, 300, 300 and 100 bytes
        assert w.calls == 8
        gaps = np.diff(w.times(5)) * 1e3
    finally:
        w.close()
    # back-off of 2, 4, 8, 16 ms after stalls 1..4 (1 ms << stalls)
    for g, want in zip(gaps, (2, 4, 8, 16)):
        assert g >= 0.8 * want, (gaps, want)


@pytest.mark.parametrize("which", ["ours", "reference"])
def test_append_wait_gives_up_after_ten_stalls(which):
    append_wait = _append_wait(which)
    buf = (C.c_uint8 * 64)()
    base = C.addressof(buf)
    w = StallingWriter(stalls=1 << 30)
    try:
        r = append_wait(w.base, capi.Slice(base, base + 64))
        assert r.error == 1
        assert w.calls == 10
        assert (r.rest.beg, r.rest.end) == (base, base + 64)
    finally:
        w.close()


@pytest.mark.parametrize("which", ["ours", "reference"])
def test_append_wait_returns_the_writers_error(which):
    append_wait = _append_wait(which)
    buf = (C.c_uint8 * 64)()
    base = C.addressof(buf)
    w = StallingWriter(stalls=2, error=True)
    try:
        r = append_wait(w.base, capi.Slice(base, base + 64))
        assert r.error == 1
        assert w.calls == 3
    finally:
        w.close()
