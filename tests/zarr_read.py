"""A minimal reader of Zarr v3 sharded arrays, for the store tests.

It reads what a zarr v3 reader does for the layout both the reference's fs
sink and this library's write (src/zarr/zarr_metadata.c:34-207): the array's
zarr.json (shape, shard shape as the regular chunk grid, one
`sharding_indexed` codec whose inner chunks use `bytes` little endian and
optionally `lz4` / `zstd`, index codecs `bytes` + `crc32c` at the end),
shard files under `c/<i>/<j>/...`, and each shard's index of
(offset, nbytes) u64 pairs (all ones for an empty chunk) followed by the
index's crc32c.  Chunks are decoded with the stock liblz4 / libzstd the
oracle links.  Only tests import this module.
"""
import itertools
import json
import os

import numpy as np

import harness as H

ZARR_DTYPE = {"uint8": "<u1", "uint16": "<u2", "uint32": "<u4", "uint64": "<u8",
              "int8": "<i1", "int16": "<i2", "int32": "<i4", "int64": "<i8",
              "float16": "<f2", "float32": "<f4", "float64": "<f8"}


def read_json(path):
    with open(os.path.join(path, "zarr.json")) as fh:
        return json.load(fh)


def read_array(path, shape=None):
    """The array stored at `path` as a numpy array.  `shape` overrides the
    stored shape (an unbounded dim 0 whose metadata was not updated)."""
    meta = read_json(path)
    assert meta["zarr_format"] == 3 and meta["node_type"] == "array"
    shape = tuple(shape or meta["shape"])
    dt = np.dtype(ZARR_DTYPE[meta["data_type"]])
    shard = meta["chunk_grid"]["configuration"]["chunk_shape"]
    (codec,) = meta["codecs"]
    assert codec["name"] == "sharding_indexed"
    cfg = codec["configuration"]
    inner = cfg["chunk_shape"]
    names = [c["name"] for c in cfg["codecs"]]
    assert names[0] == "bytes" and cfg["codecs"][0]["configuration"]["endian"] == "little"
    comp = names[1] if len(names) > 1 else None
    assert [c["name"] for c in cfg["index_codecs"]] == ["bytes", "crc32c"]
    assert cfg["index_location"] == "end"
    sep = meta["chunk_key_encoding"]["configuration"]["separator"]
    out = np.full(shape, meta["fill_value"], dtype=dt)
    rank = len(shape)
    cps = [s // c for s, c in zip(shard, inner)]
    n_inner = int(np.prod(cps))
    chunk_bytes = int(np.prod(inner)) * dt.itemsize
    nshards = [-(-n // s) if n else 0 for n, s in zip(shape, shard)]
    for sc in itertools.product(*[range(n) for n in nshards]):
        f = os.path.join(path, "c" + "".join(sep + str(c) for c in sc))
        if not os.path.exists(f):
            continue
        with open(f, "rb") as fh:
            blob = fh.read()
        index, ok = H.parse_shard(blob, n_inner)
        assert ok, f"{f}: index crc32c mismatch"
        for j, (off, nb) in enumerate(index.tolist()):
            if off == 0xFFFFFFFFFFFFFFFF and nb == 0xFFFFFFFFFFFFFFFF:
                continue
            raw = blob[off:off + nb]
            if comp:
                raw = H.decode(comp, raw, chunk_bytes)
            assert len(raw) == chunk_bytes, (f, j, len(raw))
            cc = np.unravel_index(j, cps)
            block = np.frombuffer(raw, dtype=dt).reshape(inner)
            lo = [s * sh + c * i for s, sh, c, i in zip(sc, shard, cc, inner)]
            sl = tuple(slice(l, min(l + i, n)) for l, i, n in zip(lo, inner, shape))
            if any(s.start >= s.stop for s in sl):
                continue
            out[sl] = block[tuple(slice(0, s.stop - s.start) for s in sl)]
    return out


def tree(root):
    """{relative path: bytes} of every file under root."""
    out = {}
    for d, _, files in os.walk(root):
        for f in files:
            p = os.path.join(d, f)
            with open(p, "rb") as fh:
                out[os.path.relpath(p, root)] = fh.read()
    return out
