"""ctypes mirror of the public C API structs (include/*.h).

The layouts follow the reference's public headers (src/types.stream.h,
src/dimension.h, src/types.codec.h, src/writer.h, src/stream.gpu.h), so the
same Python structures drive this library and any other implementation of
the same C ABI.
"""
import ctypes as C

MAX_RANK = 64
HALF_MAX_RANK = MAX_RANK // 2
LOD_MAX_LEVELS = 32
MAX_BATCH_EPOCHS = 128

# enum dtype
DTYPES = ["u8", "u16", "u32", "u64", "i8", "i16", "i32", "i64", "f16", "f32", "f64"]
DTYPE = {n: i for i, n in enumerate(DTYPES)}
NUMPY_DTYPE = {"u8": "<u1", "u16": "<u2", "u32": "<u4", "u64": "<u8",
               "i8": "<i1", "i16": "<i2", "i32": "<i4", "i64": "<i8",
               "f16": "<f2", "f32": "<f4", "f64": "<f8"}
BPE = {"u8": 1, "i8": 1, "u16": 2, "i16": 2, "f16": 2,
       "u32": 4, "i32": 4, "f32": 4, "u64": 8, "i64": 8, "f64": 8}

# enum compression_codec
CODEC_NONE, CODEC_LZ4, CODEC_ZSTD, CODEC_BLOSC_LZ4, CODEC_BLOSC_ZSTD = range(5)
CODEC = {"none": CODEC_NONE, "lz4": CODEC_LZ4, "zstd": CODEC_ZSTD}

# enum lod_reduce_method
REDUCE = {"mean": 0, "min": 1, "max": 2, "median": 3, "max_sup": 4, "min_sup": 5}


class OmeNgffAxis(C.Structure):
    _fields_ = [("unit", C.c_char_p), ("scale", C.c_double), ("type", C.c_int)]


class Dimension(C.Structure):
    _fields_ = [("size", C.c_uint64), ("chunk_size", C.c_uint64),
                ("chunks_per_shard", C.c_uint64), ("name", C.c_char_p),
                ("downsample", C.c_int), ("storage_position", C.c_uint8),
                ("ngff", OmeNgffAxis)]


class CodecConfig(C.Structure):
    _fields_ = [("id", C.c_int), ("level", C.c_uint8), ("shuffle", C.c_int)]


class StreamConfiguration(C.Structure):
    _fields_ = [("buffer_capacity_bytes", C.c_size_t), ("dtype", C.c_int),
                ("rank", C.c_uint8), ("dimensions", C.POINTER(Dimension)),
                ("codec", CodecConfig), ("reduce_method", C.c_int),
                ("append_reduce_method", C.c_int), ("max_nlod", C.c_int),
                ("epochs_per_batch", C.c_uint8),
                ("target_batch_chunks", C.c_uint32),
                ("metadata_update_interval_s", C.c_float),
                ("shard_alignment", C.c_size_t), ("max_threads", C.c_int)]


class StreamMetric(C.Structure):
    _fields_ = [("name", C.c_char_p), ("ms", C.c_float), ("best_ms", C.c_float),
                ("input_bytes", C.c_double), ("output_bytes", C.c_double),
                ("count", C.c_int)]


METRIC_NAMES = ["memcpy", "h2d", "lod_gather", "lod_reduce", "lod_append_fold",
                "lod_morton_chunk", "scatter", "compress", "aggregate", "d2h",
                "sink"]


class StreamMetrics(C.Structure):
    _fields_ = [(n, StreamMetric) for n in METRIC_NAMES]


class StreamStatus(C.Structure):
    _fields_ = [("nlod", C.c_int), ("append_downsample", C.c_int),
                ("epochs_per_batch", C.c_uint32),
                ("max_compressed_size", C.c_size_t), ("dtype", C.c_int),
                ("codec", CodecConfig), ("codec_batch_size", C.c_size_t),
                ("batch_accumulated", C.c_uint32), ("pool_current", C.c_int),
                ("flush_pending", C.c_int)]


class StreamLayout(C.Structure):
    _fields_ = [("lifted_rank", C.c_uint8),
                ("lifted_shape", C.c_uint64 * MAX_RANK),
                ("lifted_strides", C.c_int64 * MAX_RANK),
                ("chunk_elements", C.c_uint64), ("chunk_stride", C.c_uint64),
                ("chunks_per_epoch", C.c_uint64), ("epoch_elements", C.c_uint64),
                ("chunk_pool_bytes", C.c_size_t)]


class MemoryInfo(C.Structure):
    _fields_ = [(n, C.c_size_t) for n in (
        "device_bytes", "host_pinned_bytes", "staging_bytes", "chunk_pool_bytes",
        "compressed_pool_bytes", "aggregate_bytes", "lod_bytes", "codec_bytes",
        "shard_bytes")] + [
        ("chunks_per_epoch", C.c_uint64), ("total_chunks", C.c_uint64),
        ("max_output_size", C.c_size_t), ("nlod", C.c_int),
        ("epochs_per_batch", C.c_uint32)]


class Slice(C.Structure):
    _fields_ = [("beg", C.c_void_p), ("end", C.c_void_p)]


class WriterResult(C.Structure):
    _fields_ = [("error", C.c_int), ("rest", Slice)]


class Writer(C.Structure):
    pass


Writer._fields_ = [
    ("append", C.CFUNCTYPE(WriterResult, C.POINTER(Writer), Slice)),
    ("flush", C.CFUNCTYPE(WriterResult, C.POINTER(Writer)))]


# include/multiarray.gpu.h (src/multiarray.cpu.h:6-26)
MULTIARRAY_OK, MULTIARRAY_FAIL, MULTIARRAY_FINISHED, MULTIARRAY_NOT_FLUSHABLE = range(4)


class MultiarrayWriter(C.Structure):
    pass


MultiarrayWriter._fields_ = [
    ("update", C.CFUNCTYPE(WriterResult, C.POINTER(MultiarrayWriter), C.c_int, Slice)),
    ("flush", C.CFUNCTYPE(WriterResult, C.POINTER(MultiarrayWriter)))]


class IoEvent(C.Structure):
    _fields_ = [("seq", C.c_uint64)]


def make_dims(spec):
    """spec: list of dicts with size, chunk, cps, downsample, name, pos."""
    arr = (Dimension * len(spec))()
    for i, d in enumerate(spec):
        arr[i].size = d.get("size", 0)
        arr[i].chunk_size = d["chunk"]
        arr[i].chunks_per_shard = d.get("cps", 0)
        name = d.get("name")
        arr[i].name = name.encode() if name else None
        arr[i].downsample = 1 if d.get("downsample") else 0
        arr[i].storage_position = d.get("pos", i)
        arr[i].ngff.scale = 1.0
    return arr


def make_config(dims, dtype="u16", codec="none", level=0, reduce="mean",
                append_reduce="mean", max_nlod=0, epochs_per_batch=0,
                target_batch_chunks=0, shard_alignment=0,
                buffer_capacity_bytes=1 << 20, max_threads=0):
    cfg = StreamConfiguration()
    cfg.buffer_capacity_bytes = buffer_capacity_bytes
    cfg.dtype = DTYPE[dtype]
    cfg.rank = len(dims)
    cfg.dimensions = C.cast(dims, C.POINTER(Dimension))
    cfg.codec.id = CODEC[codec] if isinstance(codec, str) else codec
    cfg.codec.level = level
    cfg.reduce_method = REDUCE[reduce]
    cfg.append_reduce_method = REDUCE[append_reduce]
    cfg.max_nlod = max_nlod
    cfg.epochs_per_batch = epochs_per_batch
    cfg.target_batch_chunks = target_batch_chunks
    cfg.metadata_update_interval_s = 1e9
    cfg.shard_alignment = shard_alignment
    cfg.max_threads = max_threads
    return cfg


# include/zarr_fs_sink.h (src/zarr_fs_sink.h:11-80)
class ZarrConfig(C.Structure):
    _fields_ = [("store_path", C.c_char_p), ("array_name", C.c_char_p),
                ("data_type", C.c_int), ("fill_value", C.c_double),
                ("rank", C.c_uint8), ("dimensions", C.POINTER(Dimension)),
                ("unbuffered", C.c_int), ("codec", CodecConfig)]


class ZarrMultiscaleConfig(C.Structure):
    _fields_ = [("store_path", C.c_char_p), ("array_name", C.c_char_p),
                ("data_type", C.c_int), ("fill_value", C.c_double),
                ("rank", C.c_uint8), ("dimensions", C.POINTER(Dimension)),
                ("nlod", C.c_int), ("unbuffered", C.c_int), ("codec", CodecConfig)]


def bind_zarr_fs_sink(lib):
    """Argument types of the fs-sink entry points of `lib` (this library, or
    any other implementation of include/zarr_fs_sink.h)."""
    P = C.c_void_p
    lib.zarr_fs_sink_create.restype = P
    lib.zarr_fs_sink_create.argtypes = [C.POINTER(ZarrConfig)]
    lib.zarr_fs_multiscale_sink_create.restype = P
    lib.zarr_fs_multiscale_sink_create.argtypes = [C.POINTER(ZarrMultiscaleConfig)]
    for pre in ("zarr_fs_sink_", "zarr_fs_multiscale_sink_"):
        getattr(lib, pre + "destroy").argtypes = [P]
        getattr(lib, pre + "flush").argtypes = [P]
        getattr(lib, pre + "pending_bytes").restype = C.c_size_t
        getattr(lib, pre + "pending_bytes").argtypes = [P]
        getattr(lib, pre + "as_shard_sink").restype = P
        getattr(lib, pre + "as_shard_sink").argtypes = [P]
    return lib


# include/chucky_serve.h (served form; no reference counterpart)
class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_streams", C.c_int),
                ("batch_encoders", C.c_int), ("encoder_wave_bytes", C.c_size_t),
                ("encoder_lanes", C.c_int), ("autotune", C.c_int),
                ("batch_deadline_ms", C.c_double)]


class AutotuneEntry(C.Structure):
    """struct chucky_autotune_entry (include/chucky_gb300.h)."""
    _fields_ = [("codec", C.c_int), ("level", C.c_int), ("dtype", C.c_int),
                ("rank", C.c_int), ("chunk_shape", C.c_uint64 * 16),
                ("chunk_bytes", C.c_uint64), ("strength", C.c_int),
                ("min_match", C.c_int), ("encode_gbs", C.c_double),
                ("ratio", C.c_double), ("candidates", C.c_uint32)]


def autotune_entries(lib):
    """The encoder autotuner's table (a list of AutotuneEntry)."""
    lib.chucky_autotune_entries.restype = C.c_size_t
    lib.chucky_autotune_entries.argtypes = [C.c_void_p, C.c_size_t]
    n = lib.chucky_autotune_entries(None, 0)
    arr = (AutotuneEntry * max(1, n))()
    lib.chucky_autotune_entries(arr, n)
    return list(arr)[:n]


class ServerStats(C.Structure):
    _fields_ = [("requests", C.c_uint64), ("input_bytes", C.c_uint64),
                ("epochs", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("max_ms", C.c_double), ("streams_created", C.c_uint64),
                ("streams_reused", C.c_uint64), ("streams_evicted", C.c_uint64),
                ("peak_resident_bytes", C.c_uint64), ("peak_open", C.c_uint64),
                ("engine_rounds", C.c_uint64), ("engine_jobs", C.c_uint64),
                ("engine_launch_sets", C.c_uint64),
                ("engine_max_jobs_per_round", C.c_uint64)]


class ReplayRequest(C.Structure):
    _fields_ = [("config", C.POINTER(StreamConfiguration)), ("sink", C.c_void_p),
                ("data", C.c_void_p), ("bytes", C.c_size_t), ("append_bytes", C.c_size_t),
                ("arrival_s", C.c_double), ("mean_gap_s", C.c_double),
                ("seed", C.c_uint64)]


def bind_server(lib):
    """Argument types of the served-form entry points."""
    P = C.c_void_p
    lib.chucky_server_create.restype = P
    lib.chucky_server_create.argtypes = [C.POINTER(ServerConfig)]
    lib.chucky_server_destroy.argtypes = [P]
    lib.chucky_server_open.restype = P
    lib.chucky_server_open.argtypes = [P, C.POINTER(StreamConfiguration), P, C.c_int]
    lib.chucky_request_writer.restype = C.POINTER(Writer)
    lib.chucky_request_writer.argtypes = [P]
    lib.chucky_request_close.argtypes = [P]
    lib.chucky_server_get_stats.argtypes = [P, C.POINTER(ServerStats)]
    lib.chucky_server_reset_stats.argtypes = [P]
    lib.chucky_server_replay.argtypes = [P, C.POINTER(ReplayRequest), C.c_size_t,
                                         C.POINTER(C.c_double)]
    lib.chucky_server_prewarm.restype = C.c_size_t
    lib.chucky_server_prewarm.argtypes = [P, C.POINTER(C.POINTER(StreamConfiguration)),
                                          C.c_size_t, P]
    return lib
