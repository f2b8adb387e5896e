/* Several arrays ingested through one writer on one GPU.
 *
 * Mirrors the reference's CPU multi-array stream (src/multiarray.cpu.h:1-47,
 * src/multiarray/stream.c:552-830): a writer whose `update` appends to one
 * array at a time, switching arrays only at that array's epoch boundaries,
 * and whose `flush` finishes every array.  The reference has no GPU
 * multi-array stream (its devlog lists it as open work); this one keeps one
 * resident tile_stream_gpu per array, so switching arrays moves no data and
 * each array's shards are exactly those of the array ingested alone. */
#pragma once

#include "stream.gpu.h"
#include "types.stream.h"
#include "writer.h"

#ifdef __cplusplus
extern "C"
{
#endif

#ifndef CHUCKY_MULTIARRAY_WRITER_TYPES
#define CHUCKY_MULTIARRAY_WRITER_TYPES
  /* src/multiarray.cpu.h:6-26 */
  enum multiarray_writer_error
  {
    multiarray_writer_ok = 0,
    multiarray_writer_fail = 1,
    multiarray_writer_finished = 2,
    multiarray_writer_not_flushable = 3,
  };

  struct multiarray_writer_result
  {
    int error;
    struct slice rest;
  };

  struct multiarray_writer
  {
    struct multiarray_writer_result (*update)(struct multiarray_writer* self,
                                              int array_index,
                                              struct slice data);
    struct multiarray_writer_result (*flush)(struct multiarray_writer* self);
  };
#endif

  struct multiarray_tile_stream_gpu;

  /* Create one GPU stream per array (configs[i] into sinks[i]); NULL when
   * any configuration is invalid or a stream cannot be created.  The
   * configurations' dimension arrays must outlive the stream.  Metrics are
   * always collected; `enable_metrics` is accepted for the reference's
   * signature (src/multiarray.cpu.h:33-37). */
  struct multiarray_tile_stream_gpu* multiarray_tile_stream_gpu_create(
    int n_arrays,
    const struct tile_stream_configuration configs[],
    struct shard_sink* sinks[],
    int enable_metrics);

  void multiarray_tile_stream_gpu_destroy(struct multiarray_tile_stream_gpu* ms);

  /* update(i, data): append to array i.  Switching from the array last
   * appended to is refused with multiarray_writer_not_flushable (data
   * untouched) unless that array stands at an epoch boundary.  An index out
   * of range fails; a bounded array that is full returns
   * multiarray_writer_finished with the unconsumed rest.  flush(): finish
   * every array (partial epochs, dim-0 drains, shard indexes). */
  struct multiarray_writer* multiarray_tile_stream_gpu_writer(
    struct multiarray_tile_stream_gpu* ms);

  /* Sum of the arrays' stage metrics. */
  struct stream_metrics multiarray_tile_stream_gpu_get_metrics(
    const struct multiarray_tile_stream_gpu* ms);

#ifdef __cplusplus
}
#endif
