/* CPU oracle for the streaming ingest path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU backend (src/cpu/*,
 * src/stream/*, src/lod/lod_plan.c, src/zarr/shard_delivery.c,
 * src/zarr/crc32c.c).  Only the tests, the smoke check and the CPU-baseline
 * leg of the benchmark load it; the product library never does.
 *
 * Parity pins: tests/test_oracle_pins.py checks this oracle byte-for-byte
 * against the reference CPU backend compiled from its sources
 * (oracle/_ref/libchucky_ref.so, built by oracle/Makefile where the
 * reference tree is present) and against committed golden fixtures in
 * tests/golden/ that were generated from that same reference build. */
#pragma once

#include "stream.gpu.h"
#include "types.stream.h"
#include "writer.h"

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  struct oracle_stream;

  /* Mirrors tile_stream_cpu_create (src/cpu/stream.c:24-245), f16 allowed
   * (its LOD arithmetic follows src/gpu/lod.cu, the only reference code
   * path that accepts f16). */
  struct oracle_stream* oracle_stream_create(
    const struct tile_stream_configuration* config,
    struct shard_sink* sink);
  void oracle_stream_destroy(struct oracle_stream* s);
  struct writer* oracle_stream_writer(struct oracle_stream* s);
  uint64_t oracle_stream_cursor(const struct oracle_stream* s);
  const struct tile_stream_layout* oracle_stream_layout(
    const struct oracle_stream* s);

  struct oracle_info
  {
    int nlod;
    int append_downsample;
    uint32_t epochs_per_batch;
    uint64_t total_chunks;
    uint64_t chunk_elements;
    uint64_t epoch_elements;
    uint64_t max_output_size;
    uint64_t lod_nelem[LOD_MAX_LEVELS];
    uint64_t level_chunks[LOD_MAX_LEVELS];
    uint64_t shard_inner_count[LOD_MAX_LEVELS];
    uint64_t chunks_per_shard_total[LOD_MAX_LEVELS];
    uint64_t chunks_per_shard_append[LOD_MAX_LEVELS];
    uint64_t fixed_dims_count;
  };
  int oracle_stream_info(const struct oracle_stream* s,
                         struct oracle_info* info);

  /* 1 (default): reproduce the reference exactly, including stale buffer
   * contents it delivers in two corner cases (tail of a partial final epoch
   * in a reused pool slot; the dim-0 drain when K equals a level's period).
   * 0: those regions hold the fill value 0 / the drained data instead. */
  void oracle_set_reference_quirks(int on);

  /* In-memory shard sink: every (level, flat shard index) gets a growable
   * byte buffer; re-opening a shard starts it over. */
  struct oracle_mem_sink;
  struct oracle_mem_sink* oracle_mem_sink_create(void);
  void oracle_mem_sink_destroy(struct oracle_mem_sink* s);
  struct shard_sink* oracle_mem_sink_base(struct oracle_mem_sink* s);
  /* Number of shards held; list them with oracle_mem_sink_at. */
  size_t oracle_mem_sink_count(const struct oracle_mem_sink* s);
  int oracle_mem_sink_at(const struct oracle_mem_sink* s,
                         size_t i,
                         uint8_t* level,
                         uint64_t* shard_index,
                         const uint8_t** data,
                         size_t* size,
                         int* finalized);

  /* Discard sink that only counts bytes (for timing). */
  struct shard_sink* oracle_null_sink_create(void);
  void oracle_null_sink_destroy(struct shard_sink* s);
  uint64_t oracle_null_sink_bytes(const struct shard_sink* s);

  /* A test writer for writer_append_wait: its append consumes nothing for
   * the first `stalls` calls, then `chunk` bytes per call (everything when
   * 0), or fails with writer_error_fail after the stalls when `fail`.  It
   * records the monotonic time (seconds) of each of its first 64 calls. */
  struct oracle_stalling_writer;
  struct oracle_stalling_writer* oracle_stalling_writer_create(int stalls,
                                                               size_t chunk,
                                                               int fail);
  void oracle_stalling_writer_destroy(struct oracle_stalling_writer* w);
  struct writer* oracle_stalling_writer_base(struct oracle_stalling_writer* w);
  int oracle_stalling_writer_calls(const struct oracle_stalling_writer* w);
  double oracle_stalling_writer_time(const struct oracle_stalling_writer* w,
                                     int call);

  /* crc32c (Castagnoli, reflected 0x82F63B78), as src/zarr/crc32c.c:5-28. */
  uint32_t oracle_crc32c(const void* data, size_t len);

  /* Stock-library codecs, loaded at run time from liblz4.so.1 and
   * libzstd.so.1.  Return the decoded size, or (size_t)-1 on error / when
   * the library is missing. */
  size_t oracle_zstd_decompress(void* dst,
                                size_t cap,
                                const void* src,
                                size_t n);
  size_t oracle_lz4_decompress(void* dst,
                               size_t cap,
                               const void* src,
                               size_t n);
  int oracle_codecs_available(void);

  /* Standalone kernels of the restatement, for unit tests. */
  uint64_t oracle_morton_rank(int ndim,
                              const uint64_t* shape,
                              const uint64_t* coords,
                              int depth);
  /* Reduce one window [0, n) of `src` (dtype dt) with `method`; writes one
   * element to dst. */
  int oracle_reduce_window(void* dst,
                           const void* src,
                           uint64_t n,
                           enum dtype dt,
                           enum lod_reduce_method method);
  /* dim-0 fold of n elements at `level` (count = folds so far). */
  int oracle_fold(void* accum,
                  const void* fresh,
                  uint64_t n,
                  uint32_t count,
                  int level,
                  enum dtype dt,
                  enum lod_reduce_method method);
  int oracle_emit(void* dst,
                  const void* accum,
                  uint64_t n,
                  uint32_t count,
                  enum dtype dt,
                  enum lod_reduce_method method);

#ifdef __cplusplus
}
#endif
