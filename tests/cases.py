"""Stream configurations shared by the oracle pins and the GPU parity tests.

Shapes follow the reference's own tests (tests/test_cross_validate.c:177-191,
280-294, 375-397, 512-535; tests/test_lod_cpu.c:616-700) plus small versions
of the benchmark workloads (256^3 cube, sensor frames, rank-5 batched form).
Each case: name, dims spec, config kwargs, number of epochs (fractional =
partial final epoch), dtype list.
"""
import numpy as np

from chucky_gb300 import capi

D = dict

CASES = [
    ("xval_basic", [D(size=4, chunk=2, cps=2), D(size=4, chunk=2, cps=2),
                    D(size=6, chunk=3, cps=2)], {}, 2),
    ("xval_multishard", [D(size=6, chunk=2, cps=1), D(size=8, chunk=4, cps=1),
                         D(size=9, chunk=3, cps=1)], {}, 3),
    ("xval_lod", [D(size=4, chunk=2, cps=2), D(size=8, chunk=4, cps=2, downsample=1),
                  D(size=8, chunk=4, cps=2, downsample=1),
                  D(size=8, chunk=4, cps=2, downsample=1)],
     dict(epochs_per_batch=1), 2),
    ("xval_lod_dim0", [D(size=8, chunk=2, cps=2, downsample=1),
                       D(size=8, chunk=4, cps=2, downsample=1),
                       D(size=8, chunk=4, cps=2, downsample=1),
                       D(size=8, chunk=4, cps=2, downsample=1)],
     dict(epochs_per_batch=1), 4),
    ("unbounded_frames", [D(size=0, chunk=1, cps=4), D(size=24, chunk=8, cps=2),
                          D(size=40, chunk=16, cps=2)], {}, 11),
    ("cube_small_lz4geom", [D(size=32, chunk=8, cps=4, name="z"),
                            D(size=32, chunk=8, cps=4, name="y"),
                            D(size=32, chunk=8, cps=4, name="x")], {}, 4),
    ("cube_multiscale", [D(size=32, chunk=8, cps=4, downsample=1),
                         D(size=32, chunk=8, cps=4, downsample=1),
                         D(size=32, chunk=8, cps=4, downsample=1)],
     dict(reduce="median", append_reduce="mean"), 4),
    ("sensor_dim0", [D(size=0, chunk=4, cps=1, downsample=1),
                     D(size=36, chunk=8, cps=2, downsample=1),
                     D(size=64, chunk=8, cps=4, downsample=1)],
     dict(reduce="max", append_reduce="max"), 9),
    ("rank5_batched", [D(size=3, chunk=1, cps=1), D(size=2, chunk=1, cps=1),
                       D(size=16, chunk=4, cps=4, downsample=1),
                       D(size=16, chunk=8, cps=4, downsample=1),
                       D(size=16, chunk=8, cps=4, downsample=1)],
     dict(reduce="min_sup"), 6),
    ("storage_order", [D(size=6, chunk=2, cps=2), D(size=8, chunk=4, cps=1, pos=2),
                       D(size=12, chunk=4, cps=2, pos=1)], {}, 3),
    ("nondivisible_lod", [D(size=0, chunk=1, cps=2), D(size=10, chunk=8, cps=2, downsample=1),
                          D(size=6, chunk=4, cps=0, downsample=1)],
     dict(reduce="mean"), 5),
    ("partial_epoch", [D(size=7, chunk=2, cps=2), D(size=8, chunk=4, cps=1),
                       D(size=16, chunk=8, cps=2)], dict(epochs_per_batch=2), 3.5),
    ("lod4d_morton", [D(size=0, chunk=1, cps=2), D(size=6, chunk=2, cps=2, downsample=1),
                      D(size=5, chunk=2, cps=0, downsample=1),
                      D(size=4, chunk=2, cps=2, downsample=1),
                      D(size=8, chunk=4, cps=1, downsample=1)],
     dict(reduce="median"), 3),
    ("deep1d_morton", [D(size=0, chunk=1, cps=2, downsample=1), D(size=4100, chunk=2, cps=64, downsample=1)],
     dict(reduce="mean", append_reduce="max"), 5),
    ("aligned_shards", [D(size=8, chunk=2, cps=2), D(size=16, chunk=8, cps=1),
                        D(size=16, chunk=8, cps=2)], dict(shard_alignment=512), 4),
    # 64x64 LOD tiles inside 64-wide chunks (vector path) next to ragged
    # edge tiles (element path)
    ("lod2d_tiles", [D(size=0, chunk=2, cps=1), D(size=200, chunk=64, cps=2, downsample=1),
                     D(size=320, chunk=64, cps=2, downsample=1)], dict(reduce="mean"), 3),
    ("lod2d_dim0_tiles", [D(size=0, chunk=4, cps=1, downsample=1),
                          D(size=128, chunk=128, cps=1, downsample=1),
                          D(size=192, chunk=64, cps=2, downsample=1)],
     dict(reduce="max", append_reduce="mean"), 5),
]

DTYPES_ALL = ["u8", "u16", "u32", "u64", "i8", "i16", "i32", "i64", "f32", "f64"]


def make_data(dtype, n, seed=0):
    """Seeded synthetic values of `dtype` (numpy), n elements."""
    rng = np.random.default_rng(seed)
    npd = capi.NUMPY_DTYPE[dtype]
    if dtype in ("f16", "f32", "f64"):
        return (rng.normal(size=n) * 100).astype(npd)
    info = np.iinfo(np.dtype(npd))
    lo = max(info.min, -(1 << 40))
    hi = min(info.max, 1 << 40)
    return rng.integers(lo, hi, size=n, endpoint=True).astype(npd)


def build(case, dtype="u16", **over):
    name, spec, kw, epochs = case
    kw = dict(kw)
    kw.update(over)
    dims = capi.make_dims(spec)
    cfg = capi.make_config(dims, dtype=dtype, **kw)
    cfg._dims = dims  # keep alive
    return cfg, epochs
