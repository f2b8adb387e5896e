"""The encoder autotuner on the GPU: a stream tuned at its first batch
still writes chunks that decode to the oracle's bytes, the key's choice is
in the table, and a second stream of the same key (same process) writes
the same shard bytes."""
import ctypes as C

import numpy as np
import pytest

import cases
import harness as H
from chucky_gb300 import capi, load


pytestmark = pytest.mark.gpu


@pytest.fixture
def tuner():
    lib = load()
    lib.chucky_autotune_entries.restype = C.c_size_t
    lib.chucky_autotune_entries.argtypes = [C.c_void_p, C.c_size_t]
    lib.chucky_autotune_clear()
    lib.chucky_autotune_set_enabled(1)
    try:
        yield lib
    finally:
        lib.chucky_autotune_set_enabled(0)
        lib.chucky_autotune_clear()


def _entries(lib):
    return capi.autotune_entries(lib)


def _sensorish(n, seed):
    rng = np.random.default_rng(seed)
    return rng.poisson(100, size=n).astype(np.uint16)


@pytest.mark.parametrize("codec,level", [("lz4", 1), ("zstd", 1), ("zstd", 3)])
@pytest.mark.parametrize("name", ["sensor_dim0", "cube_multiscale"])
def test_tuned_stream_decodes_to_oracle_bytes(tuner, codec, level, name):
    case = cases.CASES[[c[0] for c in cases.CASES].index(name)]
    cfg_c, epochs = cases.build(case, "u16", codec=codec, level=level)
    cfg_r, _ = cases.build(case, "u16")
    n = int(epochs * H.epoch_elements(cfg_r))
    data = _sensorish(n, 11)
    got, _ = H.run_gpu(cfg_c, data)
    want, _ = H.run_oracle(cfg_r, data, quirks=False)
    checked, _, _ = H.compare_decoded(cfg_c, got, want, codec)
    assert checked > 0
    es = _entries(tuner)
    assert len(es) == 1
    e = es[0]
    assert e.candidates > 0, "tuning failed"
    assert e.level == level and e.rank == cfg_c.rank
    # the same key again: the cached choice, the same bytes
    again, _ = H.run_gpu(cfg_c, data)
    assert again == got
    assert len(_entries(tuner)) == 1
