"""Served form through the C server (include/chucky_serve.h): a request's
shards are the same whether it runs alone or concurrently with others.

Requests of the four served shapes -- the 256^3 u16 cube appended frame by
frame, 2304 x 4096 u16 sensor frames, 512^2 x 64 f32 stacks, 1024^2 u8
frames (shortened to one or two epochs each) -- with LZ4 / zstd and half of
them with a mean pyramid, each writing into its own memory sink.  They run
first one at a time (max_streams 1, every stream encoding on its own), then
all together with Poisson-paced appends, encoders batched across streams by
the shared engine, and a memory budget that admits only some of them at once
(admission waits, restarted streams).  Every shard must match byte for
byte, and every chunk of one request per shape must decode to the oracle's
raw chunk bytes.
"""
import numpy as np
import pytest

from harness import MemSink, compare_decoded, run_oracle

pytestmark = pytest.mark.gpu

FRAMES = {"cube": 256, "sensor": 32, "stack": 2, "frames8": 64}


def _requests(sinks):
    from chucky_gb300 import serve
    reqs = serve.c5_requests(seed=21, n=len(sinks), mean_gap_s=0.0003,
                             arrival_gap_s=0.002, frames=FRAMES)
    for r, s in zip(reqs, sinks):
        r.sink = s.base
    return reqs


@pytest.mark.parametrize("deadline_ms", [0.0, 2.0])
def test_served_matches_alone(deadline_ms):
    """With a batch deadline the mixed pass also starts partial batches
    (paced appends) and delivers finished ones at each append."""
    from chucky_gb300 import serve
    n = 8
    alone_sinks = [MemSink() for _ in range(n)]
    mix_sinks = [MemSink() for _ in range(n)]
    try:
        reqs = _requests(alone_sinks)
        serve.run_plain(reqs, warmup=False)
        alone = [s.shards() for s in alone_sinks]
        reqs = _requests(mix_sinks)
        # a budget for about three requests at a time: admission waits and
        # restarted (reused) streams both happen
        budget = 3 * max(serve.memory_estimate(r) for r in reqs)
        st = serve.run_served(reqs, hbm_budget=budget, max_streams=4, paced=True,
                              warmup=False, batch_deadline_ms=deadline_ms)
        assert st["requests"] == n and st["epochs"] > 0
        assert st["engine_rounds"] > 0 and st["engine_jobs"] >= st["engine_rounds"]
        assert st["streams_reused"] + st["streams_created"] == n
        mixed = [s.shards() for s in mix_sinks]
        for i, (a, m) in enumerate(zip(alone, mixed)):
            assert a.keys() == m.keys(), f"request {reqs[i].name}: shard sets differ"
            for k in a:
                assert a[k] == m[k], f"request {reqs[i].name} shard {k} differs"
        # the data itself: every chunk decodes to the oracle's bytes (one
        # request of each shape)
        seen = set()
        for i, r in enumerate(reqs):
            kind = r.name.split(":")[1]
            if kind in seen:
                continue
            seen.add(kind)
            raw_kw = dict(r.cfg_kwargs, codec="none")
            cfg = serve.Request(name="raw", cfg_kwargs=raw_kw, dims=r.dims,
                                data=None, frame_bytes=0).config()
            data = r.data.numpy() if hasattr(r.data, "numpy") else r.data
            shards_raw, _ = run_oracle(cfg, data, quirks=False)
            checked, _, _ = compare_decoded(r.config(), mixed[i], shards_raw,
                                            r.cfg_kwargs["codec"])
            assert checked > 0
    finally:
        for s in alone_sinks + mix_sinks:
            s.close()


def test_admission_respects_the_budget():
    """Three requests of one configuration and a budget for one stream of it
    (each stream with its own encoders, charged its full estimate): they
    are served one at a time on one resident stream."""
    from chucky_gb300 import serve
    sinks = [MemSink() for _ in range(3)]
    try:
        first = _requests(sinks[:1])[0]
        reqs = [serve.Request(name=f"{i}:{first.name}", cfg_kwargs=first.cfg_kwargs,
                              dims=first.dims, data=first.data,
                              frame_bytes=first.frame_bytes, sink=s.base)
                for i, s in enumerate(sinks)]
        budget = serve.memory_estimate(reqs[0])
        st = serve.run_served(reqs, hbm_budget=budget, max_streams=16, paced=False,
                              batch_encoders=False, warmup=False)
        # (the server's start-up created the one stream that fits)
        assert st["streams_created"] + st["streams_reused"] == 3
        assert st["streams_reused"] >= 2
        assert st["requests"] == 3
        assert st["peak_open"] == 1
        assert st["peak_resident_bytes"] <= budget
    finally:
        for s in sinks:
            s.close()
