"""Zarr v3 stores written through the filesystem sink, read back from disk.

* CPU: the reference CPU stream writes a store through the reference's own
  fs sink (src/zarr/zarr_fs_sink.c, src/zarr/zarr_metadata.c, compiled into
  oracle/_ref) and through this library's (`zarr_fs_sink.cpp`); the oracle
  writes one through this library's.  The three directory trees -- shard
  files under c/<i>/<j>/..., every zarr.json (array, group, OME-NGFF
  multiscales) -- are byte-identical, for every codec (the oracle and the
  reference compress with the same liblz4 / libzstd calls).
* Every store reads back (tests/zarr_read.py: the array's zarr.json, the
  shard index and its crc32c, stock-library decoding) to the appended
  array at level 0, like the reference's tests/test_zarr_readback.c.
* GPU: the GPU stream writes through this library's sink.  Uncompressed,
  its tree equals the oracle's byte for byte; compressed, the metadata
  files are identical and every level reads back to the oracle's arrays.
"""
import ctypes as C
import os

import numpy as np
import pytest

import cases
import harness as H
import zarr_read as Z
from chucky_gb300 import capi

needs_ref = pytest.mark.skipif(H.reference() is None,
                               reason="reference build (oracle/_ref) not present")

D = dict
# name, dims, stream kwargs, epochs, multiscale sink, sink kwargs
STORES = [
    # the reference readback test's shape (tests/test_zarr_readback.c:30-36)
    ("tyx_frames", [D(size=0, chunk=1, cps=4, name="t"), D(size=8, chunk=4, cps=2, name="y"),
                    D(size=12, chunk=6, cps=2, name="x")], {}, 4, False, {}),
    ("cube_multiscale", [D(size=32, chunk=8, cps=4, downsample=1, name="z"),
                         D(size=32, chunk=8, cps=4, downsample=1, name="y"),
                         D(size=32, chunk=8, cps=4, downsample=1, name="x")],
     dict(reduce="median", append_reduce="mean", max_nlod=4), 4, True, {}),
    ("sensor_dim0", [D(size=0, chunk=4, cps=1, downsample=1, name="t"),
                     D(size=32, chunk=8, cps=2, downsample=1, name="y"),
                     D(size=64, chunk=8, cps=4, downsample=1, name="x")],
     dict(reduce="max", append_reduce="max", max_nlod=5), 9, True, {}),
    # y = 36 is not a multiple of its chunk: the stream consumes epochs in
    # the lifted (padded) index space, as the reference does, so the input
    # is not a dense row-major array of the stored shape (trees only)
    ("sensor_dim0_ragged", [D(size=0, chunk=4, cps=1, downsample=1, name="t"),
                            D(size=36, chunk=8, cps=2, downsample=1, name="y"),
                            D(size=64, chunk=8, cps=4, downsample=1, name="x")],
     dict(reduce="mean", append_reduce="mean", max_nlod=5), 9, True, {}),
    ("aligned_unbuffered", [D(size=8, chunk=2, cps=2, name="z"), D(size=16, chunk=8, cps=1, name="y"),
                            D(size=16, chunk=8, cps=2, name="x")],
     dict(shard_alignment=4096), 4, False, dict(unbuffered=1)),
    ("storage_order", [D(size=6, chunk=2, cps=2, name="z"), D(size=8, chunk=4, cps=1, pos=2, name="y"),
                       D(size=12, chunk=4, cps=2, pos=1, name="x")], {}, 3, False, {}),
]
CODECS = [("none", 0), ("lz4", 1), ("zstd", 3)]


def _case(name, dtype, codec, level):
    spec = next(s for s in STORES if s[0] == name)
    _, dims_spec, kw, epochs, multiscale, sink_kw = spec
    dims = capi.make_dims(dims_spec)
    cfg = capi.make_config(dims, dtype=dtype, codec=codec, level=level, **kw)
    cfg._dims = dims
    return cfg, epochs, multiscale, sink_kw, dims_spec


class FsSink:
    """A zarr fs sink of `lib` (this library or the reference build)."""

    def __init__(self, lib, path, cfg, multiscale, nlod, unbuffered=0):
        self.lib = capi.bind_zarr_fs_sink(lib)
        self.pre = "zarr_fs_multiscale_sink_" if multiscale else "zarr_fs_sink_"
        if multiscale:
            z = capi.ZarrMultiscaleConfig()
            z.nlod = nlod
        else:
            z = capi.ZarrConfig()
            z.array_name = b"0"
        z.store_path = path.encode()
        z.data_type = cfg.dtype
        z.fill_value = 0.0
        z.rank = cfg.rank
        z.dimensions = cfg.dimensions
        z.unbuffered = unbuffered
        z.codec = cfg.codec
        self._z = z
        create = getattr(self.lib, self.pre + "create")
        self.h = create(C.byref(z))
        assert self.h, f"{self.pre}create failed for {path}"
        self.base = getattr(self.lib, self.pre + "as_shard_sink")(self.h)

    def close(self):
        if self.h:
            getattr(self.lib, self.pre + "flush")(self.h)
            getattr(self.lib, self.pre + "destroy")(self.h)
            self.h = None


def _ours():
    import chucky_gb300 as cg
    return cg.load()


def _write(impl, sink_lib, path, cfg, data, multiscale, sink_kw, quirks=True):
    os.makedirs(path, exist_ok=True)
    nlod = H.plan_info(cfg).nlod
    sink = FsSink(sink_lib, path, cfg, multiscale, nlod, **sink_kw)
    try:
        cursor = H.run_into(impl, cfg, data, sink.base, quirks=quirks)
    finally:
        sink.close()
    return cursor


def _input(cfg, epochs, dtype, dims_spec):
    ee = H.epoch_elements(cfg)
    n = int(epochs * ee)
    if dtype == "u16":  # the reference readback test's ramp, plus noise
        data = ((np.arange(n) + cases.make_data("u8", n, seed=2)) & 0xFFFF).astype("<u2")
    else:
        data = cases.make_data(dtype, n, seed=2)
    inner = [d["size"] for d in dims_spec[1:]]
    rows = n // int(np.prod(inner))
    return data, data.reshape([rows] + inner)


def _level0(path, multiscale):
    return os.path.join(path, "0")


def _mask_padding(blob, n_slots):
    """The shard file with every byte outside its indexed chunks and its
    index zeroed: page-alignment padding is not written by the reference
    (it holds whatever its buffer held), so only the rest is compared."""
    index, ok = H.parse_shard(blob, n_slots)
    assert ok
    keep = np.zeros(len(blob), dtype=bool)
    keep[len(blob) - (16 * n_slots + 4):] = True
    for off, nb in index.tolist():
        if off != 0xFFFFFFFFFFFFFFFF:
            keep[off:off + nb] = True
    out = np.frombuffer(blob, dtype=np.uint8).copy()
    out[~keep] = 0
    return out.tobytes()


def _same_file(key, a, b, cfg, spec):
    if cfg.shard_alignment and not key.endswith("zarr.json"):
        n_slots = int(np.prod([d["cps"] for d in spec]))
        return _mask_padding(a, n_slots) == _mask_padding(b, n_slots)
    return a == b


def _dense(name):
    """The appended bytes are the stored array in row-major order."""
    return name not in ("storage_order", "sensor_dim0_ragged")


@needs_ref
@pytest.mark.parametrize("codec,level", CODECS, ids=[c[0] for c in CODECS])
@pytest.mark.parametrize("name", [s[0] for s in STORES])
def test_store_identical_to_reference_sink(tmp_path, name, codec, level):
    cfg, epochs, multiscale, sink_kw, spec = _case(name, "u16", codec, level)
    data, arr = _input(cfg, epochs, "u16", spec)
    ref = H.reference()
    d_ref = str(tmp_path / "ref")
    d_ours_ref = str(tmp_path / "ours_sink_ref_stream")
    d_oracle = str(tmp_path / "ours_sink_oracle")
    _write("reference", ref, d_ref, cfg, data, multiscale, sink_kw)
    _write("reference", _ours(), d_ours_ref, cfg, data, multiscale, sink_kw)
    _write("oracle", _ours(), d_oracle, cfg, data, multiscale, sink_kw)
    t_ref, t_a, t_b = Z.tree(d_ref), Z.tree(d_ours_ref), Z.tree(d_oracle)
    assert sorted(t_a) == sorted(t_ref)
    for k in t_ref:
        assert t_a[k] == t_ref[k], f"{k} differs (this sink vs the reference sink)"
        assert _same_file(k, t_b[k], t_ref[k], cfg, spec), \
            f"{k} differs (oracle stream vs reference stream)"
    assert sorted(t_b) == sorted(t_ref)
    # the store reads back to the appended array
    if _dense(name):
        got = Z.read_array(_level0(d_oracle, multiscale))
        np.testing.assert_array_equal(got, arr)


def test_storage_order_reads_back_transposed(tmp_path):
    """Dims stored in the order (z, x, y).  The stream writes chunks in
    storage order; the fs sink takes its dims as given (neither sink reads
    `storage_position`, src/zarr/zarr_metadata.c:34-207), so a caller hands
    it the dims in storage order, and the store then reads back as the
    appended array with its axes permuted to that order."""
    cfg, epochs, multiscale, sink_kw, spec = _case("storage_order", "u16", "none", 0)
    data, arr = _input(cfg, epochs, "u16", spec)
    order = sorted(range(len(spec)), key=lambda i: spec[i].get("pos", i))
    sdims = capi.make_dims([dict(spec[i], pos=j) for j, i in enumerate(order)])
    d = str(tmp_path / "s")
    os.makedirs(d)
    lib = capi.bind_zarr_fs_sink(_ours())
    z = capi.ZarrConfig()
    z.store_path, z.array_name = d.encode(), b"0"
    z.data_type, z.rank, z.codec = cfg.dtype, cfg.rank, cfg.codec
    z.dimensions = C.cast(sdims, C.POINTER(capi.Dimension))
    h = lib.zarr_fs_sink_create(C.byref(z))
    assert h
    try:
        H.run_into("oracle", cfg, data, lib.zarr_fs_sink_as_shard_sink(h))
    finally:
        lib.zarr_fs_sink_flush(h)
        lib.zarr_fs_sink_destroy(h)
    meta = Z.read_json(_level0(d, multiscale))
    assert meta["dimension_names"] == [spec[i]["name"] for i in order]
    np.testing.assert_array_equal(Z.read_array(_level0(d, multiscale)),
                                  arr.transpose(order))


@pytest.mark.gpu
@pytest.mark.parametrize("codec,level", CODECS, ids=[c[0] for c in CODECS])
@pytest.mark.parametrize("name", [s[0] for s in STORES])
def test_gpu_store_reads_back(tmp_path, name, codec, level):
    cfg, epochs, multiscale, sink_kw, spec = _case(name, "u16", codec, level)
    data, arr = _input(cfg, epochs, "u16", spec)
    d_gpu = str(tmp_path / "gpu")
    d_ora = str(tmp_path / "oracle")
    _write("gpu", _ours(), d_gpu, cfg, data, multiscale, sink_kw)
    _write("oracle", _ours(), d_ora, cfg, data, multiscale, sink_kw, quirks=False)
    t_gpu, t_ora = Z.tree(d_gpu), Z.tree(d_ora)
    assert sorted(t_gpu) == sorted(t_ora)
    for k in t_ora:
        if codec == "none" or k.endswith("zarr.json"):
            assert t_gpu[k] == t_ora[k], f"{k} differs"
    # every chunk of every shard file decodes to the oracle's chunk bytes;
    # the slot count per shard comes from the planner: at levels >= 1 of a
    # bounded, downsampled append dim the reference's zarr.json declares
    # more inner chunks per shard than its epoch-split shard files hold
    # (reproduced byte for byte), so zarr.json is not used for them
    info = H.plan_info(cfg)
    for k in t_ora:
        if k.endswith("zarr.json"):
            continue
        lv = int(k.split(os.sep)[0]) if multiscale else 0
        n_slots = info.chunks_per_shard_total[lv]
        idx_g, ok_g = H.parse_shard(t_gpu[k], n_slots)
        idx_o, ok_o = H.parse_shard(t_ora[k], n_slots)
        assert ok_g and ok_o, k
        for (og, ng), (oo, no) in zip(idx_g.tolist(), idx_o.tolist()):
            assert (og == 0xFFFFFFFFFFFFFFFF) == (oo == 0xFFFFFFFFFFFFFFFF), k
            if oo == 0xFFFFFFFFFFFFFFFF:
                continue
            raw = t_ora[k][oo:oo + no]
            if codec != "none":
                raw = H.decode(codec, raw, info.chunk_elements * 2)
            got = t_gpu[k][og:og + ng]
            if codec != "none":
                got = H.decode(codec, got, info.chunk_elements * 2)
            assert got == raw, k
    if _dense(name):
        np.testing.assert_array_equal(Z.read_array(_level0(d_gpu, multiscale)), arr)
