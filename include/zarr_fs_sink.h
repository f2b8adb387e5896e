/* Zarr v3 filesystem sink (one array, or an OME-NGFF multiscale group).
 * Config structs and entry points replace src/zarr_fs_sink.h:11-80 of the
 * reference. */
#pragma once

#include "dimension.h"
#include "dtype.h"
#include "types.codec.h"
#include "writer.h"

#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  struct zarr_config
  {
    const char* store_path;
    const char* array_name; /* NULL: the array lives at store_path */
    enum dtype data_type;
    double fill_value;
    uint8_t rank;
    const struct dimension* dimensions;
    int unbuffered; /* O_DIRECT shard writes */
    struct codec_config codec;
  };

  struct zarr_fs_sink;

  /* Writes zarr.json for the root, intermediate groups and the array.
   * NULL on error.  Replaces src/zarr_fs_sink.h:26-27. */
  struct zarr_fs_sink* zarr_fs_sink_create(const struct zarr_config* cfg);

  void zarr_fs_sink_destroy(struct zarr_fs_sink* s);

  /* Blocks until every queued write has reached the file. */
  void zarr_fs_sink_flush(struct zarr_fs_sink* s);

  size_t zarr_fs_sink_pending_bytes(struct zarr_fs_sink* s);

  struct shard_sink* zarr_fs_sink_as_shard_sink(struct zarr_fs_sink* s);

  struct zarr_multiscale_config
  {
    const char* store_path;
    const char* array_name; /* group name; NULL: group at store_path */
    enum dtype data_type;
    double fill_value;
    uint8_t rank;
    const struct dimension* dimensions; /* L0 dims */
    int nlod;                           /* 0 = as many as the stream makes */
    int unbuffered;
    struct codec_config codec;
  };

  struct zarr_fs_multiscale_sink;

  /* Arrays "0", "1", ... with the downsampled shapes plus OME-NGFF group
   * metadata.  Replaces src/zarr_fs_sink.h:65-80. */
  struct zarr_fs_multiscale_sink* zarr_fs_multiscale_sink_create(
    const struct zarr_multiscale_config* cfg);

  void zarr_fs_multiscale_sink_destroy(struct zarr_fs_multiscale_sink* s);

  void zarr_fs_multiscale_sink_flush(struct zarr_fs_multiscale_sink* s);

  size_t zarr_fs_multiscale_sink_pending_bytes(
    struct zarr_fs_multiscale_sink* s);

  struct shard_sink* zarr_fs_multiscale_sink_as_shard_sink(
    struct zarr_fs_multiscale_sink* s);

#ifdef __cplusplus
}
#endif
