"""GPU stream vs the CPU oracle: whole shard files, byte for byte.

CODEC_NONE makes every chunk byte visible, so these compare the transpose,
the LOD pyramid (every level, every reduce method, dim-0 folds), the shard
aggregation, the index and its crc32c, and the shard keys.  The oracle runs
with reference quirks off: a partial final epoch is zero-filled and a dim-0
drain delivers the drained data (the two places where the reference CPU
backend delivers stale buffer contents)."""
import numpy as np
import pytest

import cases
import harness as H
from chucky_gb300 import capi

pytestmark = pytest.mark.gpu


def _pieces(nbytes, bpe, seed):
    rng = np.random.default_rng(seed)
    cuts = rng.integers(1, max(2, nbytes), size=6).tolist()
    return sorted(c - c % bpe for c in cuts)


@pytest.mark.parametrize("case", cases.CASES, ids=[c[0] for c in cases.CASES])
@pytest.mark.parametrize("dtype", ["u16", "u8", "f32", "i64"])
def test_gpu_matches_oracle(case, dtype):
    cfg, epochs = cases.build(case, dtype)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=5)
    pieces = _pieces(n * capi.BPE[dtype], capi.BPE[dtype], 9)
    a, ca = H.run_gpu(cfg, data, pieces)
    b, cb = H.run_oracle(cfg, data, pieces, quirks=False)
    assert ca == cb
    assert a == b, H.diff_shards(a, b)


@pytest.mark.parametrize("method", ["mean", "min", "max", "median", "max_sup", "min_sup"])
@pytest.mark.parametrize("dtype", cases.DTYPES_ALL + ["f16"])
def test_gpu_lod_methods(method, dtype):
    case = cases.CASES[[c[0] for c in cases.CASES].index("sensor_dim0")]
    app = method if method in ("mean", "min", "max") else "max"
    cfg, epochs = cases.build(case, dtype, reduce=method, append_reduce=app)
    n = int(epochs * H.epoch_elements(cfg))
    data = cases.make_data(dtype, n, seed=13)
    a, _ = H.run_gpu(cfg, data)
    b, _ = H.run_oracle(cfg, data, quirks=False)
    assert a == b, H.diff_shards(a, b)
