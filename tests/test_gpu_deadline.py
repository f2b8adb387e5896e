"""Batch deadline (tile_stream_gpu_set_batch_deadline): a stream that
starts partial batches as soon as an epoch has waited -- here at almost
every append -- writes the same shard bytes as one that waits for full
batches of K epochs (where no shard alignment pads each batch's chunks),
and every chunk decodes to the oracle's bytes."""
import numpy as np
import pytest

import cases
import harness as H

pytestmark = pytest.mark.gpu

NAMES = ["cube_multiscale", "sensor_dim0", "rank5_batched", "partial_epoch",
         "unbounded_frames", "aligned_shards"]


@pytest.mark.parametrize("codec,level", [("none", 0), ("lz4", 1), ("zstd", 1)])
@pytest.mark.parametrize("name", NAMES)
def test_partial_batches_write_the_same_shards(name, codec, level):
    case = cases.CASES[[c[0] for c in cases.CASES].index(name)]
    cfg, epochs = cases.build(case, "u16", codec=codec, level=level)
    cfg_r, _ = cases.build(case, "u16")
    ee = H.epoch_elements(cfg_r)
    n = int(epochs * ee)
    data = cases.make_data("u16", n, seed=5)
    # appends of a third of an epoch (in bytes, u16)
    step = max(1, ee // 3) * 2
    pieces = list(range(step, n * 2, step))
    base, c0 = H.run_gpu(cfg, data, pieces)
    fast, c1 = H.run_gpu(cfg, data, pieces, deadline_ms=1e-6)
    assert c0 == c1
    if not cfg.shard_alignment:
        assert fast == base, H.diff_shards(fast, base)
    want, _ = H.run_oracle(cfg_r, data, quirks=False)
    if codec == "none":
        if not cfg.shard_alignment:
            assert fast == want, H.diff_shards(fast, want)
    else:
        checked, _, _ = H.compare_decoded(cfg, fast, want, codec)
        assert checked > 0
