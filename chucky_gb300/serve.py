"""Served form from Python: a binding of the C server (include/chucky_serve.h)
and the served workload.

A request is one array ingested by a resident GPU stream.  The server admits
requests while their device-memory estimate fits an HBM budget and fewer
than `max_streams` are open, keeps finished streams resident for the next
request of the same configuration, and (batch_encoders) encodes the ready
batches of all open requests together in a shared encoder engine.  The
request loop itself -- one host thread per admitted request, Poisson-paced
appends, flush, close -- runs in C (`chucky_server_replay`), so nothing here
is on the data path.

Two forms over the same requests:
  * plain  -- one request at a time (max_streams 1), each stream encoding
    on its own, appended as fast as possible;
  * served -- up to 16 requests at once under a 48 GB budget, encoders
    batched across streams.
Both are timed after the server's start-up (resident streams created: one
per configuration for the plain form, one per request as far as the budget
allows for the served form) and a warm-up pass, and report aggregate input
GB/s and the p50 / p99 of the append-to-delivered latency of every epoch.
"""
import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi, load


@dataclass
class Request:
    name: str
    cfg_kwargs: dict
    dims: list            # capi.make_dims spec
    data: object          # host or device buffer (torch tensor or numpy array), bytes
    frame_bytes: int      # append granularity
    arrival_s: float = 0.0       # arrival time after the server starts
    mean_gap_s: float = 0.0      # mean gap between appends (Poisson)
    sink: int = None             # this request's shard_sink*, else the server's
    seed: int = 0
    _cfg: object = field(default=None, repr=False)

    def config(self):
        if self._cfg is None:
            dims = capi.make_dims(self.dims)
            cfg = capi.make_config(dims, **self.cfg_kwargs)
            cfg._dims = dims
            self._cfg = cfg
        return self._cfg

    def buffer(self):
        d = self.data
        if hasattr(d, "data_ptr"):
            return d.data_ptr(), d.numel() * d.element_size()
        return d.ctypes.data, d.nbytes


def _lib():
    lib = capi.bind_server(load())
    lib.chucky_discard_sink_create.restype = C.c_void_p
    lib.chucky_discard_sink_destroy.argtypes = [C.c_void_p]
    lib.chucky_discard_sink_bytes.restype = C.c_uint64
    lib.chucky_discard_sink_bytes.argtypes = [C.c_void_p]
    lib.tile_stream_gpu_memory_estimate.restype = C.c_int
    return lib


class Server:
    """Owner of one chucky_server."""

    def __init__(self, hbm_budget=48 << 30, max_streams=16, batch_encoders=True,
                 wave_bytes=0, lanes=0, autotune=False, batch_deadline_ms=0.0):
        self.lib = _lib()
        cfg = capi.ServerConfig(hbm_budget, max_streams, 1 if batch_encoders else 0,
                                wave_bytes, lanes, 1 if autotune else 0,
                                float(batch_deadline_ms))
        self.h = self.lib.chucky_server_create(C.byref(cfg))
        if not self.h:
            raise RuntimeError("chucky_server_create failed")

    def replay(self, requests, sink, paced=True):
        """Run the requests through the C request loop; returns wall seconds."""
        arr = (capi.ReplayRequest * len(requests))()
        for i, r in enumerate(requests):
            ptr, nbytes = r.buffer()
            arr[i].config = C.pointer(r.config())
            arr[i].sink = r.sink or sink
            arr[i].data = ptr
            arr[i].bytes = nbytes
            arr[i].append_bytes = r.frame_bytes
            arr[i].arrival_s = r.arrival_s if paced else 0.0
            arr[i].mean_gap_s = r.mean_gap_s if paced else 0.0
            arr[i].seed = r.seed + i
        wall = C.c_double()
        if self.lib.chucky_server_replay(self.h, arr, len(requests), C.byref(wall)):
            raise RuntimeError("a request failed")
        return wall.value

    def prewarm(self, requests, sink, per_request=True):
        """Create idle streams at start-up: one per request (`per_request`,
        for requests that may run concurrently) or one per configuration,
        as far as the budget allows.  Returns the number created."""
        cfgs, seen = [], set()
        for r in requests:
            key = (tuple(sorted(r.cfg_kwargs.items())), repr(r.dims))
            if per_request or key not in seen:
                cfgs.append(r.config())
                seen.add(key)
        arr = (C.POINTER(capi.StreamConfiguration) * len(cfgs))(
            *[C.pointer(c) for c in cfgs])
        return self.lib.chucky_server_prewarm(self.h, arr, len(cfgs), sink)

    def stats(self):
        st = capi.ServerStats()
        self.lib.chucky_server_get_stats(self.h, C.byref(st))
        return {k: getattr(st, k) for k, _ in capi.ServerStats._fields_}

    def reset_stats(self):
        self.lib.chucky_server_reset_stats(self.h)

    def close(self):
        if self.h:
            self.lib.chucky_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_form(requests, hbm_budget, max_streams, batch_encoders, paced, sink=None,
             warmup=True, batch_deadline_ms=0.0):
    """Warm-up pass (creates the resident streams), then the timed pass."""
    lib = _lib()
    own = sink is None
    sink = sink or lib.chucky_discard_sink_create()
    try:
        with Server(hbm_budget, max_streams, batch_encoders,
                    batch_deadline_ms=batch_deadline_ms) as srv:
            srv.prewarm(requests, sink, per_request=max_streams > 1)
            if warmup:
                srv.replay(requests, sink, paced=False)
            srv.reset_stats()
            wall = srv.replay(requests, sink, paced=paced)
            st = srv.stats()
    finally:
        if own:
            lib.chucky_discard_sink_destroy(sink)
    st["wall_s"] = wall
    st["gbs"] = st["input_bytes"] / wall / 1e9 if wall > 0 else 0.0
    return st


def run_plain(requests, sink=None, warmup=True):
    """One request at a time, each stream encoding on its own, appended as
    fast as possible."""
    return run_form(requests, 1 << 62, 1, False, paced=False, sink=sink, warmup=warmup)


def run_served(requests, hbm_budget=48 << 30, max_streams=16, batch_encoders=True,
               paced=True, sink=None, warmup=True, batch_deadline_ms=0.0):
    return run_form(requests, hbm_budget, max_streams, batch_encoders, paced, sink=sink,
                    warmup=warmup, batch_deadline_ms=batch_deadline_ms)


def memory_estimate(req):
    lib = _lib()
    info = capi.MemoryInfo()
    if lib.tile_stream_gpu_memory_estimate(C.byref(req.config()), C.byref(info)) != 0:
        raise ValueError(f"{req.name}: invalid configuration")
    return info.device_bytes


# ---------------------------------------------------------------------------
# The served workload: 16 requests drawn from four shapes
# ---------------------------------------------------------------------------

def shapes():
    D = dict
    return {
        # 256^3 u16 cube, appended frame by frame along z
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


def make_data(spec, rng, frames=None):
    n = spec["frame"] * (frames or spec["frames"])
    if spec["dtype"] == "f32":
        return rng.normal(0, 1, size=n // 4).astype("<f4").view(np.uint8)
    if spec["dtype"] == "u16":
        return np.minimum(rng.poisson(100, size=n // 2), 4095).astype("<u2").view(np.uint8)
    return rng.integers(0, 64, size=n, dtype=np.uint8)


def c5_requests(seed=5, n=16, mean_gap_s=0.0005, arrival_gap_s=0.02, device=None,
                pinned=True, frames=None):
    """`n` requests (seeded) from the four shapes, LZ4 / zstd alternating,
    every other one with a mean pyramid (at most 4 levels), arrivals with
    exponential gaps of mean `arrival_gap_s`.  Data: one buffer per shape,
    pinned host memory, or device memory when `device` is given.  `frames`
    ({shape: frames}) shortens requests."""
    import torch
    rng = np.random.default_rng(seed)
    sh = shapes()
    names = list(sh)
    data = {}
    reqs = []
    t = 0.0
    for i in range(n):
        kind = names[int(rng.integers(0, len(names)))]
        spec = sh[kind]
        if kind not in data:
            arr = torch.from_numpy(make_data(spec, rng, (frames or {}).get(kind)))
            data[kind] = arr.to(device) if device is not None else (
                arr.pin_memory() if pinned else arr)
        lod = i % 2 == 1
        dims = [dict(d) for d in spec["dims"]]
        for d in dims:
            d["downsample"] = 1 if (lod and d["name"] in spec["lod"]) else 0
        kw = dict(dtype=spec["dtype"], codec="lz4" if i % 2 == 0 else "zstd", level=1,
                  reduce="mean", append_reduce="mean", max_nlod=4 if lod else 0)
        kw.update(spec.get("extra", {}))
        reqs.append(Request(name=f"{i}:{kind}", cfg_kwargs=kw, dims=dims,
                            data=data[kind], frame_bytes=spec["frame"],
                            arrival_s=t, mean_gap_s=mean_gap_s, seed=seed * 1000 + i))
        t += float(rng.exponential(arrival_gap_s))
    return reqs


C5_WORKLOAD = ("16 requests drawn (seeded) from {256^3 u16 cube appended frame by frame, "
               "2304x4096 u16 frames x32, 512^2x64 f32 stacks x4, 1024^2 u8 frames x256}, "
               "LZ4 / zstd-1 alternating, every other request with a 4-level mean pyramid, "
               "48 GB HBM admission budget, 16 streams")


def main():
    import json
    from . import build
    build.build()
    reqs = c5_requests()
    plain = run_plain(reqs)
    served = run_served(reqs, paced=False)
    paced = run_served(reqs, paced=True)
    out = {"workload": C5_WORKLOAD, "plain": plain, "served": served,
           "served_paced": paced, "served_over_plain": served["gbs"] / plain["gbs"]}
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
