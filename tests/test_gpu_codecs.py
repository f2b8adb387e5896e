"""GPU encoders: every chunk written by the GPU stream with LZ4 or zstd
decodes with the stock liblz4 / libzstd to exactly the chunk bytes the
oracle writes with CODEC_NONE; shard indexes and crc32c stay valid."""
import numpy as np
import pytest

import cases
import harness as H
from chucky_gb300 import capi

pytestmark = pytest.mark.gpu

CODEC_CASES = ["cube_small_lz4geom", "cube_multiscale", "sensor_dim0",
               "rank5_batched", "aligned_shards", "partial_epoch", "unbounded_frames"]


def _data(kind, dtype, n, seed):
    rng = np.random.default_rng(seed)
    npd = capi.NUMPY_DTYPE[dtype]
    if kind == "random":
        return cases.make_data(dtype, n, seed)
    if kind == "zeros":
        return np.zeros(n, dtype=npd)
    if kind == "ramp":
        return (np.arange(n) % 251).astype(npd)
    # mixed: blocks of zeros, constants and noise
    out = np.zeros(n, dtype=npd)
    step = max(1, n // 17)
    for i in range(0, n, step):
        r = rng.integers(0, 4)
        if r == 1:
            out[i:i + step] = rng.integers(0, 100)
        elif r >= 2:
            out[i:i + step] = cases.make_data(dtype, min(step, n - i), seed + i)
    return out


@pytest.mark.parametrize("codec,level", [("lz4", 1), ("lz4", 2), ("zstd", 1), ("zstd", 3)])
@pytest.mark.parametrize("name", CODEC_CASES)
@pytest.mark.parametrize("kind", ["mixed", "random", "zeros", "ramp"])
def test_gpu_chunks_decode_to_oracle_bytes(codec, level, name, kind):
    case = cases.CASES[[c[0] for c in cases.CASES].index(name)]
    dtype = "u16"
    cfg_c, epochs = cases.build(case, dtype, codec=codec, level=level)
    cfg_r, _ = cases.build(case, dtype)
    n = int(epochs * H.epoch_elements(cfg_r))
    data = _data(kind, dtype, n, seed=3)
    got, _ = H.run_gpu(cfg_c, data)
    want, _ = H.run_oracle(cfg_r, data, quirks=False)
    checked, comp, raw = H.compare_decoded(cfg_c, got, want, codec)
    assert checked > 0
    if kind == "zeros":
        assert comp * 4 < raw
