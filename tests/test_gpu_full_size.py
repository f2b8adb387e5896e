"""The benchmark's workloads at their full sizes: every chunk the GPU stream
writes (every pyramid level) decodes with the stock liblz4 / libzstd to the
chunk bytes the oracle writes for the same input with CODEC_NONE, and the
shard indexes and their crc32c are valid.

  * the plain multiscale pair: 256^3 u16 (mean pyramid) and 256^3 f32
    (median pyramid), chunk 64^3, zstd-3;
  * the 256^3 u16 cube with LZ4 and no pyramid;
  * 2304 x 4096 u16 sensor frames, chunk 32 x 256 x 256, 5-level max
    pyramid with dim-0 downsampling: 64 frames (two epochs, so level 1 is
    folded and emitted), zstd-1 and LZ4; and 512 frames (16 epochs: every
    level 1..4 folds and emits in steady state, level 4 once per 16
    epochs), zstd-1, appended frame by frame;
  * the batched rank-5 (t, c, z, y, x) arrays t x 3 x 128 x 512 x 512 in
    all five dtypes (u8 t=8, i16 / u16 / f16 t=4, f32 t=2: 768 MiB each)
    with zero / constant / random chunks, max_sup / min_sup pyramid,
    zstd-1.
Inputs are the benchmark's own seeded generators."""
import os
import sys

import numpy as np
import pytest

import harness as H

pytestmark = pytest.mark.gpu

sys.path.insert(0, H.ROOT)
import bench  # noqa: E402

from chucky_gb300 import capi  # noqa: E402


def _raw_config(cfg_codec):
    """The same stream with CODEC_NONE (the oracle's reference bytes)."""
    import ctypes as C
    raw = capi.StreamConfiguration()
    C.memmove(C.byref(raw), C.byref(cfg_codec), C.sizeof(raw))
    raw.codec.id = capi.CODEC["none"]
    raw.codec.level = 0
    raw._dims = cfg_codec._dims
    return raw


def _check(cfg, data, codec):
    got, _ = H.run_gpu(cfg, data)
    want, _ = H.run_oracle(_raw_config(cfg), data, quirks=False)
    checked, comp, raw = H.compare_decoded(cfg, got, want, codec)
    assert checked > 0
    return comp, raw


def test_multiscale_pair_zstd3():
    u16, f32 = bench.make_cubes()
    for cube, cfg in ((u16, bench.make_config("u16", "mean")),
                      (f32, bench.make_config("f32", "median"))):
        comp, raw = _check(cfg, cube, "zstd")
        assert comp < raw


def test_cube_lz4():
    u16, _ = bench.make_cubes()
    _check(bench.cube_lz4_config(), u16, "lz4")


@pytest.mark.parametrize("codec", ["zstd", "lz4"])
def test_sensor_frames_two_epochs(codec):
    import torch
    frames = bench.sensor_frames(64, torch.device("cuda")).cpu().numpy().view("<u2")
    comp, raw = _check(bench.sensor_config(codec, "max"), frames, codec)
    assert comp < raw


def test_sensor_frames_sixteen_epochs():
    import torch
    frames = bench.sensor_frames(512, torch.device("cuda")).cpu().numpy().view("<u2")
    cfg = bench.sensor_config("zstd", "max")
    frame_bytes = 2304 * 4096 * 2
    pieces = list(range(frame_bytes, frames.nbytes, frame_bytes))
    got, _ = H.run_gpu(cfg, frames, pieces)
    want, _ = H.run_oracle(_raw_config(cfg), frames, quirks=False)
    checked, comp, raw = H.compare_decoded(cfg, got, want, "zstd")
    levels = {k[0] for k in want}
    assert levels == {0, 1, 2, 3, 4}, levels
    # level l emits 16 / 2^l epochs of ceil(9 / 2^l) x ceil(16 / 2^l)
    # chunks of 256 x 256: 16*144 + 8*40 + 4*12 + 2*4 + 1*1, all checked
    assert checked == 2681
    assert comp < raw


@pytest.mark.parametrize("dtype,t,reduce", bench.BATCHED_DTYPES,
                         ids=[d[0] for d in bench.BATCHED_DTYPES])
def test_batched_rank5(dtype, t, reduce):
    import torch
    arr = bench.batched_array(dtype, t, torch.device("cuda")).cpu().numpy()
    comp, raw = _check(bench.batched_config(dtype, t, reduce), arr, "zstd")
    assert comp * 2 < raw  # half the chunks are zero, a quarter constant
