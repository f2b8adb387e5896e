/* GPU streaming writer: the drop-in C API of the ingest hot path.
 *
 * Entry points, structs and semantics replace src/stream.gpu.h:1-82 of the
 * reference (create/destroy/append through struct writer, layout, cursor,
 * status, metrics, memory estimate, chunk-size advice).  All arguments are
 * plain C types; a current CUDA device is required, as in the reference. */
#pragma once

#include "types.stream.h"
#include "writer.h"

#ifdef __cplusplus
extern "C"
{
#endif

  /* L0 layout of one epoch in the chunk pool.  Layout matches
   * src/stream/layouts.h:10-21 of the reference. */
  struct tile_stream_layout
  {
    uint8_t lifted_rank;
    uint64_t lifted_shape[MAX_RANK];
    int64_t lifted_strides[MAX_RANK];

    uint64_t chunk_elements;
    uint64_t chunk_stride;
    uint64_t chunks_per_epoch;
    uint64_t epoch_elements;
    size_t chunk_pool_bytes;
  };

  struct tile_stream_layout_gpu
  {
    uint64_t* d_lifted_shape;
    int64_t* d_lifted_strides;
  };

  /* Layout matches src/stream.gpu.h:15-37. */
  struct tile_stream_memory_info
  {
    size_t device_bytes;
    size_t host_pinned_bytes;

    size_t staging_bytes;
    size_t chunk_pool_bytes;
    size_t compressed_pool_bytes;
    size_t aggregate_bytes;
    size_t lod_bytes;
    size_t codec_bytes;

    size_t shard_bytes;

    uint64_t chunks_per_epoch;
    uint64_t total_chunks;
    size_t max_output_size;
    int nlod;
    uint32_t epochs_per_batch;
  };

  struct tile_stream_gpu;

  /* Device/host memory a stream with this config would hold; nothing is
   * allocated.  0 on success.  Replaces src/stream.gpu.h:41-43. */
  int tile_stream_gpu_memory_estimate(
    const struct tile_stream_configuration* config,
    struct tile_stream_memory_info* info);

  /* Largest power-of-two chunk (from target_chunk_bytes down) whose memory
   * estimate fits budget_bytes; edits config->dimensions.  0 on success.
   * Replaces src/stream.gpu.h:45-52. */
  int tile_stream_gpu_advise_chunk_sizes(
    struct tile_stream_configuration* config,
    size_t target_chunk_bytes,
    const uint8_t* ratios,
    size_t budget_bytes);

  /* NULL on an invalid config or a codec the GPU path does not support.
   * config->dimensions must outlive the stream; the sink is borrowed.
   * Replaces src/stream.gpu.h:54-60. */
  struct tile_stream_gpu* tile_stream_gpu_create(
    const struct tile_stream_configuration* config,
    struct shard_sink* sink);

  /* Waits for in-flight work, then frees.  Replaces src/stream.gpu.h:62-63. */
  void tile_stream_gpu_destroy(struct tile_stream_gpu* stream);

  /* Replaces src/stream.gpu.h:65-67. */
  struct stream_metrics tile_stream_gpu_get_metrics(
    const struct tile_stream_gpu* s);

  /* Replaces src/stream.gpu.h:71-72. */
  const struct tile_stream_layout* tile_stream_gpu_layout(
    const struct tile_stream_gpu* s);

  /* Replaces src/stream.gpu.h:74-75. */
  struct writer* tile_stream_gpu_writer(struct tile_stream_gpu* s);

  /* Elements appended so far.  Replaces src/stream.gpu.h:77-78. */
  uint64_t tile_stream_gpu_cursor(const struct tile_stream_gpu* s);

  /* Replaces src/stream.gpu.h:80-81. */
  struct tile_stream_status tile_stream_gpu_status(
    const struct tile_stream_gpu* s);

#ifdef __cplusplus
}
#endif
