"""Served form: a request's shards are the same whether it runs alone or
concurrently with others on resident, restarted streams.

Each request writes into its own memory sink.  The requests run first one at
a time (run_plain) and then all together with Poisson-paced appends and a
memory budget that admits only some of them at once (run_served), which
also exercises stream reuse through tile_stream_gpu_restart.  Every shard
must match byte for byte, and every chunk must decode to the oracle's raw
chunk bytes.
"""
import numpy as np
import pytest

from harness import MemSink, compare_decoded, run_oracle

pytestmark = pytest.mark.gpu

D = dict


def _requests(torch, sinks):
    from chucky_gb300 import serve
    rng = np.random.default_rng(21)
    specs = [
        # (dims, kwargs, frame bytes, frames)
        ([D(size=64, chunk=16, cps=2, name="z", downsample=1),
          D(size=64, chunk=16, cps=2, name="y", downsample=1),
          D(size=64, chunk=16, cps=2, name="x", downsample=1)],
         dict(dtype="u16", codec="lz4", level=1, reduce="mean", append_reduce="mean",
              max_nlod=3, epochs_per_batch=2), 64 * 64 * 2, 64),
        ([D(size=0, chunk=4, cps=1, name="t"),
          D(size=96, chunk=32, cps=2, name="y", downsample=1),
          D(size=128, chunk=32, cps=2, name="x", downsample=1)],
         dict(dtype="u16", codec="zstd", level=1, reduce="max", append_reduce="max",
              max_nlod=3, epochs_per_batch=2), 96 * 128 * 2, 22),
        ([D(size=0, chunk=8, cps=1, name="t"),
          D(size=128, chunk=64, cps=2, name="y"),
          D(size=128, chunk=64, cps=2, name="x")],
         dict(dtype="u8", codec="lz4", level=1), 128 * 128, 40),
        ([D(size=0, chunk=1, cps=1, name="t"),
          D(size=16, chunk=16, cps=1, name="z"),
          D(size=64, chunk=32, cps=2, name="y", downsample=1),
          D(size=64, chunk=32, cps=2, name="x", downsample=1)],
         dict(dtype="f32", codec="zstd", level=1, reduce="mean", append_reduce="mean",
              max_nlod=2), 16 * 64 * 64 * 4, 5),
    ]
    reqs, raw = [], []
    for i, (dims, kw, frame, frames) in enumerate(specs * 2):
        n = frame * frames
        if kw["dtype"] == "f32":
            x = rng.normal(0, 1, size=n // 4).astype("<f4").view(np.uint8)
        else:
            x = (rng.integers(0, 32, size=n, dtype=np.uint8) | (np.arange(n) % 7 == 0))
            x = x.astype(np.uint8)
        raw.append(x)
        reqs.append(serve.Request(name=f"r{i}", cfg_kwargs=dict(kw), dims=dims,
                                  data=torch.from_numpy(x), frame_bytes=frame,
                                  arrival_s=0.002 * i, mean_gap_s=0.0005,
                                  sink=sinks[i].base))
    return reqs, raw


def _shards(sinks):
    return [s.shards() for s in sinks]


def test_served_matches_alone():
    torch = pytest.importorskip("torch")
    from chucky_gb300 import serve
    alone_sinks = [MemSink() for _ in range(8)]
    mix_sinks = [MemSink() for _ in range(8)]
    try:
        reqs, raw = _requests(torch, alone_sinks)
        serve.run_plain(reqs)
        alone = _shards(alone_sinks)
        reqs, _ = _requests(torch, mix_sinks)
        # a budget for about three requests at a time: admission waits and
        # restarted (reused) streams both happen
        budget = 3 * max(serve.memory_estimate(serve.load(), r) for r in reqs)
        out = serve.run_served(reqs, hbm_budget=budget, max_streams=4)
        assert out["epochs"] > 0
        mixed = _shards(mix_sinks)
        for i, (a, m) in enumerate(zip(alone, mixed)):
            assert a.keys() == m.keys(), f"request {i}: shard sets differ"
            for k in a:
                assert a[k] == m[k], f"request {i} shard {k} differs"
        # and the data itself: every chunk decodes to the oracle's bytes
        for i in range(4):
            raw_kw = dict(reqs[i].cfg_kwargs, codec="none")
            cfg = serve.Request(name="raw", cfg_kwargs=raw_kw, dims=reqs[i].dims,
                                data=None, frame_bytes=0).config()
            shards_raw, _ = run_oracle(cfg, raw[i], quirks=False)
            n, _, _ = compare_decoded(reqs[i].config(), mixed[i], shards_raw,
                                      reqs[i].cfg_kwargs["codec"])
            assert n > 0
    finally:
        for s in alone_sinks + mix_sinks:
            s.close()
