"""chucky_gb300: GB300-native streaming ingest (chunk transpose, LOD pyramid,
LZ4/zstd encoders, shard aggregation) behind the chucky C API.

The product is the C-ABI library libchucky_gb300.so (declared in include/*.h).
This package builds it (build.py) and exposes its entry points through
ctypes with the argument types of the C API (capi.py).  There is no CPU
fallback: load() raises if the CUDA library is missing.
"""
import ctypes as C
import os

from . import capi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libchucky_gb300.so")

_lib = None

# every exported entry point of include/*.h
EXPORTS = [
    "tile_stream_gpu_memory_estimate", "tile_stream_gpu_advise_chunk_sizes",
    "tile_stream_gpu_create", "tile_stream_gpu_destroy",
    "tile_stream_gpu_get_metrics", "tile_stream_gpu_layout",
    "tile_stream_gpu_writer", "tile_stream_gpu_cursor", "tile_stream_gpu_status",
    "writer_ok", "writer_error", "writer_error_at", "writer_finished_at",
    "writer_append", "writer_flush", "writer_append_wait",
    "dims_create", "dims_set_storage_order", "dims_set_downsample_by_name",
    "dims_set_chunk_sizes", "dims_budget_chunk_size", "dims_set_shard_counts",
    "dims_budget_chunk_bytes", "dims_n_append", "dims_validate", "dims_print",
    "codec_is_blosc", "codec_is_gpu_supported",
    "multiarray_tile_stream_gpu_create", "multiarray_tile_stream_gpu_destroy",
    "multiarray_tile_stream_gpu_writer", "multiarray_tile_stream_gpu_get_metrics",
]


def load():
    """Load libchucky_gb300.so (build it first with build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: run chucky_gb300.build.build() first "
            "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    cfgp = C.POINTER(capi.StreamConfiguration)
    lib.tile_stream_gpu_create.restype = P
    lib.tile_stream_gpu_create.argtypes = [cfgp, P]
    lib.tile_stream_gpu_destroy.argtypes = [P]
    lib.tile_stream_gpu_writer.restype = C.POINTER(capi.Writer)
    lib.tile_stream_gpu_writer.argtypes = [P]
    lib.tile_stream_gpu_cursor.restype = C.c_uint64
    lib.tile_stream_gpu_cursor.argtypes = [P]
    lib.tile_stream_gpu_layout.restype = C.POINTER(capi.StreamLayout)
    lib.tile_stream_gpu_layout.argtypes = [P]
    lib.tile_stream_gpu_status.restype = capi.StreamStatus
    lib.tile_stream_gpu_status.argtypes = [P]
    lib.tile_stream_gpu_get_metrics.restype = capi.StreamMetrics
    lib.tile_stream_gpu_get_metrics.argtypes = [P]
    lib.tile_stream_gpu_memory_estimate.restype = C.c_int
    lib.tile_stream_gpu_memory_estimate.argtypes = [cfgp, C.POINTER(capi.MemoryInfo)]
    lib.tile_stream_gpu_advise_chunk_sizes.restype = C.c_int
    lib.tile_stream_gpu_advise_chunk_sizes.argtypes = [
        cfgp, C.c_size_t, C.POINTER(C.c_uint8), C.c_size_t]
    lib.writer_append.restype = capi.WriterResult
    lib.writer_append.argtypes = [C.POINTER(capi.Writer), capi.Slice]
    lib.writer_flush.restype = capi.WriterResult
    lib.writer_flush.argtypes = [C.POINTER(capi.Writer)]
    lib.writer_append_wait.restype = capi.WriterResult
    lib.writer_append_wait.argtypes = [C.POINTER(capi.Writer), capi.Slice]
    lib.dims_n_append.restype = C.c_uint8
    lib.dims_n_append.argtypes = [C.POINTER(capi.Dimension), C.c_uint8]
    lib.dims_validate.argtypes = [C.POINTER(capi.Dimension), C.c_uint8]
    lib.dims_create.restype = C.c_uint8
    lib.dims_create.argtypes = [C.POINTER(capi.Dimension), C.c_char_p,
                                C.POINTER(C.c_uint64)]
    lib.chucky_crc32c.restype = C.c_uint32
    lib.chucky_crc32c.argtypes = [P, C.c_size_t]
    _lib = lib
    return lib


class GpuStream:
    """Thin owner of one tile_stream_gpu handle."""

    def __init__(self, cfg, sink_base):
        self.lib = load()
        self._cfg = cfg  # keeps the dimension array alive
        self.h = self.lib.tile_stream_gpu_create(C.byref(cfg), sink_base)
        if not self.h:
            raise RuntimeError("tile_stream_gpu_create failed")
        self.writer = self.lib.tile_stream_gpu_writer(self.h)

    def append(self, ptr, nbytes):
        r = self.lib.writer_append(self.writer, capi.Slice(ptr, ptr + nbytes))
        return r

    def flush(self):
        return self.lib.writer_flush(self.writer)

    def layout(self):
        return self.lib.tile_stream_gpu_layout(self.h).contents

    def status(self):
        return self.lib.tile_stream_gpu_status(self.h)

    def metrics(self):
        return self.lib.tile_stream_gpu_get_metrics(self.h)

    def cursor(self):
        return self.lib.tile_stream_gpu_cursor(self.h)

    def close(self):
        if self.h:
            self.lib.tile_stream_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
