"""Served form: many concurrent ingest streams on one GPU.

A request is one array ingested through its own GPU stream (its own CUDA
streams, pools, LOD accumulators and shard state resident on the device).
The server admits requests while their memory estimate
(`tile_stream_gpu_memory_estimate`) fits an HBM budget, runs every admitted
request on its own host thread -- appends arrive as a Poisson process, the
stream flushes at the end -- and starts queued requests as soon as slots
and memory free up (continuous admission).  Idle streams of a finished
request are kept and re-used (`tile_stream_gpu_restart`) by later requests
with the same configuration, so device buffers are not re-allocated.

Both forms start from a pool of idle streams created before the clock
starts, as a server does at start-up (`setup_s` reports that time): one
per request as far as the budget allows for the concurrent form, one per
distinct configuration for the sequential one.  Reported: aggregate input GB/s
over the whole run and the p50/p99 of the append-to-delivered latency of
every epoch (`tile_stream_gpu_latencies`).  `run_plain` processes the same
requests one at a time, appending as fast as possible, for comparison.
"""
import ctypes as C
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import capi, load


@dataclass
class Request:
    name: str
    cfg_kwargs: dict
    dims: list            # capi.make_dims spec
    data: object          # host or device buffer exposing data_ptr()/numel() (bytes)
    frame_bytes: int      # append granularity
    arrival_s: float = 0.0       # arrival time after the server starts
    mean_gap_s: float = 0.0      # mean gap between appends (Poisson)
    key: tuple = field(default=None)
    sink: int = None             # this request's shard_sink*, else the server's

    def config(self):
        dims = capi.make_dims(self.dims)
        cfg = capi.make_config(dims, **self.cfg_kwargs)
        cfg._dims = dims
        return cfg


class StreamPool:
    """GPU streams resident on the device, by configuration.

    A finished request's stream stays resident (idle) and is restarted for
    the next request with the same configuration; idle streams of other
    configurations are evicted when a new stream would exceed the budget.
    `resident` counts the estimated device bytes of every stream alive."""

    def __init__(self, lib, sink, budget):
        self.lib, self.sink, self.budget = lib, sink, budget
        self.idle = {}  # key -> [(stream, bytes)]
        self.resident = 0

    @staticmethod
    def key(req):
        return req.key or (tuple(sorted(req.cfg_kwargs.items())), repr(req.dims))

    def try_acquire(self, req, need):
        """A stream for req, or None when it does not fit yet (caller waits)."""
        from . import GpuStream
        k = self.key(req)
        sink = req.sink or self.sink
        lst = self.idle.get(k)
        if lst:
            s, nb = lst.pop()
            if self.lib.tile_stream_gpu_restart(s.h, sink) == 0:
                return s, nb
            s.close()
            self.resident -= nb
        while self.resident + need > self.budget and self._evict_one():
            pass
        if self.resident + need > self.budget:
            return None
        self.resident += need
        return GpuStream(req.config(), sink), need

    def prewarm(self, requests, need, per_request=False):
        """Create idle streams at server start-up, as far as the budget
        allows: one per distinct configuration, or one per request
        (`per_request`, for requests that will run concurrently).  Returns
        the seconds it took."""
        t0 = time.perf_counter()
        seen, made = set(), []
        for r, m in zip(requests, need):
            k = self.key(r)
            if (k in seen and not per_request) or self.resident + m > self.budget:
                continue
            seen.add(k)
            from . import GpuStream
            self.resident += m
            made.append((r, GpuStream(r.config(), r.sink or self.sink), m))
        for r, st, m in made:
            self.release(r, st, m)
        return time.perf_counter() - t0

    def _evict_one(self):
        for k, lst in self.idle.items():
            if lst:
                s, nb = lst.pop()
                s.close()
                self.resident -= nb
                return True
        return False

    def release(self, req, s, nb):
        self.idle.setdefault(self.key(req), []).append((s, nb))

    def close(self):
        while self._evict_one():
            pass


def _setup(lib):
    lib.chucky_discard_sink_create.restype = C.c_void_p
    lib.chucky_discard_sink_bytes.restype = C.c_uint64
    lib.chucky_discard_sink_bytes.argtypes = [C.c_void_p]
    lib.chucky_discard_sink_destroy.argtypes = [C.c_void_p]
    lib.tile_stream_gpu_restart.argtypes = [C.c_void_p, C.c_void_p]
    lib.tile_stream_gpu_latencies.restype = C.c_size_t
    lib.tile_stream_gpu_latencies.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                              C.c_size_t]
    lib.tile_stream_gpu_clear_latencies.argtypes = [C.c_void_p]


def _latencies(lib, s):
    n = lib.tile_stream_gpu_latencies(s.h, None, 0)
    buf = (C.c_double * max(1, n))()
    lib.tile_stream_gpu_latencies(s.h, buf, n)
    lib.tile_stream_gpu_clear_latencies(s.h)
    return list(buf[:n])


def _ingest(s, req, rng, paced):
    """Append the request's data frame by frame, then flush."""
    base = req.data.data_ptr()
    total = req.data.numel()
    off = 0
    while off < total:
        n = min(req.frame_bytes, total - off)
        if paced and req.mean_gap_s > 0:
            time.sleep(rng.exponential(req.mean_gap_s))
        r = s.append(base + off, n)
        if r.error:
            raise RuntimeError(f"{req.name}: append failed ({r.error})")
        off += n
    r = s.flush()
    if r.error:
        raise RuntimeError(f"{req.name}: flush failed ({r.error})")
    return total


def memory_estimate(lib, req):
    info = capi.MemoryInfo()
    cfg = req.config()
    if lib.tile_stream_gpu_memory_estimate(C.byref(cfg), C.byref(info)) != 0:
        raise ValueError(f"{req.name}: invalid configuration")
    return info.device_bytes


def run_served(requests, hbm_budget=48 << 30, max_streams=16, seed=0, sink=None):
    """Run requests concurrently (arrival times honoured, Poisson appends)."""
    lib = load()
    _setup(lib)
    own_sink = sink is None
    sink = sink or lib.chucky_discard_sink_create()
    pool = StreamPool(lib, sink, hbm_budget)
    need = [memory_estimate(lib, r) for r in requests]
    for r, m in zip(requests, need):
        if m > hbm_budget:
            raise ValueError(f"{r.name}: needs {m} bytes, above the budget")
    setup_s = pool.prewarm(requests, need, per_request=True)
    lock = threading.Condition()
    state = {"active": 0, "bytes": 0, "lat": [], "err": [], "peak": 0}
    t0 = time.perf_counter()

    def worker(i, req, s, nb):
        rng = np.random.default_rng(seed + i)
        try:
            nbytes = _ingest(s, req, rng, paced=True)
            lat = _latencies(lib, s)
            with lock:
                state["bytes"] += nbytes
                state["lat"].extend(lat)
        except Exception as e:  # reported after the run
            with lock:
                state["err"].append(str(e))
        finally:
            with lock:
                pool.release(req, s, nb)
                state["active"] -= 1
                lock.notify_all()

    threads = []
    order = sorted(range(len(requests)), key=lambda i: requests[i].arrival_s)
    for i in order:
        req = requests[i]
        delay = req.arrival_s - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        with lock:  # admission: a free slot and room in the HBM budget
            while True:
                got = None
                if state["active"] < max_streams:
                    got = pool.try_acquire(req, need[i])
                if got:
                    break
                lock.wait()
            state["active"] += 1
            state["peak"] = max(state["peak"], pool.resident)
        th = threading.Thread(target=worker, args=(i, req) + got)
        th.start()
        threads.append(th)
    for th in threads:
        th.join()
    wall = time.perf_counter() - t0
    pool.close()
    if own_sink:
        lib.chucky_discard_sink_destroy(sink)
    if state["err"]:
        raise RuntimeError("; ".join(state["err"]))
    lat = np.array(state["lat"]) if state["lat"] else np.zeros(1)
    return {"gbs": state["bytes"] / wall / 1e9, "bytes": state["bytes"],
            "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "epochs": int(len(lat)),
            "peak_resident_bytes": int(state["peak"]), "setup_s": setup_s}


def run_plain(requests, sink=None):
    """The same requests one at a time, appended as fast as possible."""
    lib = load()
    _setup(lib)
    own_sink = sink is None
    sink = sink or lib.chucky_discard_sink_create()
    pool = StreamPool(lib, sink, 1 << 62)
    need = [memory_estimate(lib, r) for r in requests]
    setup_s = pool.prewarm(requests, need)
    lat, nbytes = [], 0
    t0 = time.perf_counter()
    rng = np.random.default_rng(0)
    per = []
    for req, m in zip(requests, need):
        t1 = time.perf_counter()
        s, nb = pool.try_acquire(req, m)
        n = _ingest(s, req, rng, paced=False)
        nbytes += n
        lat.extend(_latencies(lib, s))
        pool.release(req, s, nb)
        per.append([req.name, round(n / 1e6, 1), round((time.perf_counter() - t1) * 1e3, 2)])
    wall = time.perf_counter() - t0
    pool.close()
    if own_sink:
        lib.chucky_discard_sink_destroy(sink)
    lat = np.array(lat) if lat else np.zeros(1)
    return {"gbs": nbytes / wall / 1e9, "bytes": nbytes, "wall_s": wall,
            "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "epochs": int(len(lat)),
            "setup_s": setup_s, "requests_mb_ms": per}


# ---------------------------------------------------------------------------
# The served-form workload: 16 requests drawn from four shapes
# ---------------------------------------------------------------------------

def _shapes():
    D = dict
    return {
        # 256^3 u16 cube, appended along z
        "cube": dict(dims=[D(size=256, chunk=64, cps=4, name="z"),
                           D(size=256, chunk=64, cps=4, name="y"),
                           D(size=256, chunk=64, cps=4, name="x")],
                     lod="zyx", dtype="u16", frame=256 * 256 * 2, frames=256,
                     extra=dict(epochs_per_batch=4)),
        # 2304 x 4096 u16 sensor frames, unbounded time
        "sensor": dict(dims=[D(size=0, chunk=32, cps=1, name="t"),
                             D(size=2304, chunk=256, cps=8, name="y"),
                             D(size=4096, chunk=256, cps=8, name="x")],
                       lod="yx", dtype="u16", frame=2304 * 4096 * 2, frames=32,
                       extra=dict(epochs_per_batch=2)),
        # 512^2 x 64 f32 stacks, unbounded stack index
        "stack": dict(dims=[D(size=0, chunk=1, cps=1, name="t"),
                            D(size=64, chunk=64, cps=1, name="z"),
                            D(size=512, chunk=128, cps=4, name="y"),
                            D(size=512, chunk=128, cps=4, name="x")],
                      lod="yx", dtype="f32", frame=64 * 512 * 512 * 4, frames=4,
                      extra=dict(epochs_per_batch=2)),
        # 1024^2 u8 frames, unbounded time
        "frames8": dict(dims=[D(size=0, chunk=64, cps=1, name="t"),
                              D(size=1024, chunk=256, cps=4, name="y"),
                              D(size=1024, chunk=256, cps=4, name="x")],
                        lod="yx", dtype="u8", frame=1024 * 1024, frames=256,
                        extra=dict(epochs_per_batch=2)),
    }


def _make_data(kind, spec, rng):
    n = spec["frame"] * spec["frames"]
    if spec["dtype"] == "f32":
        x = (rng.normal(0, 1, size=n // 4)).astype("<f4").view(np.uint8)
    elif spec["dtype"] == "u16":
        base = rng.poisson(100, size=n // 2).astype("<u2")
        x = np.minimum(base, 4095).astype("<u2").view(np.uint8)
    else:
        x = rng.integers(0, 64, size=n, dtype=np.uint8)
    return x


def c5_requests(seed=5, n=16, mean_gap_s=0.0005, arrival_gap_s=0.02, device_data=False):
    """16 requests (seeded) from the four shapes, LZ4 / zstd alternating,
    every other one with a mean LOD pyramid (at most 4 levels)."""
    import torch
    rng = np.random.default_rng(seed)
    shapes = _shapes()
    names = list(shapes)
    data = {}
    reqs = []
    t = 0.0
    for i in range(n):
        kind = names[int(rng.integers(0, len(names)))]
        spec = shapes[kind]
        if kind not in data:
            arr = torch.from_numpy(_make_data(kind, spec, rng))
            data[kind] = arr.cuda() if device_data else arr.pin_memory()
        lod = i % 2 == 1
        dims = [dict(d) for d in spec["dims"]]
        for d in dims:
            d["downsample"] = 1 if (lod and d["name"] in spec["lod"]) else 0
        kw = dict(dtype=spec["dtype"], codec="lz4" if i % 2 == 0 else "zstd", level=1,
                  reduce="mean", append_reduce="mean", max_nlod=4 if lod else 0)
        kw.update(spec.get("extra", {}))
        reqs.append(Request(name=f"{i}:{kind}", cfg_kwargs=kw, dims=dims,
                            data=data[kind], frame_bytes=spec["frame"],
                            arrival_s=t, mean_gap_s=mean_gap_s))
        t += float(rng.exponential(arrival_gap_s))
    return reqs


def main():
    import json
    from . import build
    build.build()
    reqs = c5_requests()
    run_plain(reqs[:2])  # warm up (module load, first allocations)
    plain = run_plain(reqs)
    # the same 16 requests all queued at once, appended as fast as possible
    burst = c5_requests(mean_gap_s=0.0, arrival_gap_s=0.0)
    served = run_served(burst)
    # Poisson arrivals and appends: latency under an open load
    paced = run_served(reqs)
    out = {"workload": "16 requests from {256^3 u16 cube, 2304x4096 u16 frames, "
                       "512^2x64 f32 stacks, 1024^2 u8 frames}, LZ4/zstd alternating, "
                       "half with 4-level mean LOD, 48 GB admission",
           "plain": plain, "served": served, "served_paced": paced,
           "served_over_plain": served["gbs"] / plain["gbs"]}
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
