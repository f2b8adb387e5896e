/* Extensions of this library beyond the reference's C API.
 *
 * None of these entry points has a counterpart in the reference; they exist
 * for callers that run many arrays through one stream object (serving) and
 * for benchmarking. */
#pragma once

#include "stream.gpu.h"
#include "writer.h"

#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  /* Start a new array on a stream that has been flushed (or never
   * appended to), keeping every device allocation: cursor, shard state and
   * dim-0 accumulators return to their initial state.  `sink` replaces the
   * stream's sink when not NULL.  Returns 0 on success, non-zero when the
   * stream still has unflushed data. */
  int tile_stream_gpu_restart(struct tile_stream_gpu* s,
                              struct shard_sink* sink);

  /* Append-to-delivered latency of every epoch delivered so far, in ms:
   * from the append call that completed the epoch's input to the end of
   * the sink writes of the batch holding it.  Writes up to `cap` values to
   * `out_ms` (may be NULL) and returns the total count. */
  size_t tile_stream_gpu_latencies(const struct tile_stream_gpu* s,
                                   double* out_ms,
                                   size_t cap);
  void tile_stream_gpu_clear_latencies(struct tile_stream_gpu* s);

  /* A shard sink that discards every byte and counts them (the metering
   * sink of a throughput benchmark). */
  struct shard_sink* chucky_discard_sink_create(void);
  void chucky_discard_sink_destroy(struct shard_sink* s);
  uint64_t chucky_discard_sink_bytes(const struct shard_sink* s);

  /* Number of CUDA kernels this library has launched in this process. */
  uint64_t chucky_launch_count(void);

  /* crc32c (Castagnoli) of a buffer, as used by shard indexes. */
  uint32_t chucky_crc32c(const void* data, size_t len);

#ifdef __cplusplus
}
#endif
