/* Array dimensions: shape, chunking, sharding, storage order, downsampling.
 * Struct layouts match src/dimension.h:10-39 of the reference; the helper
 * functions replace src/dimension.h:46-119 (same names, same semantics). */
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  enum dimension_axis_type
  {
    dimension_axis_space = 0,
    dimension_axis_time,
    dimension_axis_channel,
    dimension_axis_other,
  };

  /* OME-NGFF v0.5 axis metadata (only read by the zarr metadata writer). */
  struct omengff_axis
  {
    const char* unit; /* NULL means "index" */
    double scale;     /* 0 is treated as 1.0 */
    enum dimension_axis_type type;
  };

  struct dimension
  {
    uint64_t size;             /* 0: unbounded (dim 0 only) */
    uint64_t chunk_size;       /* elements per chunk along this dim */
    uint64_t chunks_per_shard; /* 0: every chunk of the dim in one shard */
    const char* name;          /* optional one-letter label */
    int downsample;            /* 1: dim takes part in the LOD pyramid */
    uint8_t storage_position;  /* 0 = outermost; dims[0] must be 0 */
    struct omengff_axis ngff;
  };

  /* One dim per character of `names`; chunk = size, identity storage order.
   * Returns the rank, 0 on error.  Replaces src/dimension.h:46-47. */
  uint8_t dims_create(struct dimension* dims,
                      const char* names,
                      const uint64_t* sizes);

  /* Storage order from a string of dim names (NULL = identity); append dims
   * must keep their positions.  Replaces src/dimension.h:55-56. */
  int dims_set_storage_order(struct dimension* dims,
                             uint8_t rank,
                             const char* order);

  /* downsample = 1 exactly on the dims named in `names`.
   * Replaces src/dimension.h:60-63. */
  void dims_set_downsample_by_name(struct dimension* dims,
                                   uint8_t rank,
                                   const char* names);

  /* Replaces src/dimension.h:67-70. */
  void dims_set_chunk_sizes(struct dimension* dims,
                            uint8_t rank,
                            const uint64_t* chunk_sizes);

  /* Power-of-two chunk sizes with ~nelem elements, split by `ratios`.
   * Replaces src/dimension.h:78-82. */
  void dims_budget_chunk_size(struct dimension* dims,
                              uint8_t rank,
                              uint64_t nelem,
                              const uint8_t* ratios);

  /* chunks_per_shard from a target shard count per dim (0 = leave).
   * Replaces src/dimension.h:87-90. */
  void dims_set_shard_counts(struct dimension* dims,
                             uint8_t rank,
                             const uint64_t* shard_counts);

  /* Byte-target form of dims_budget_chunk_size.
   * Replaces src/dimension.h:95-100. */
  void dims_budget_chunk_bytes(struct dimension* dims,
                               uint8_t rank,
                               size_t target_chunk_bytes,
                               size_t bytes_per_element,
                               const uint8_t* ratios);

  /* Number of leading append dims (chunk_size == 1 prefix, cut after the
   * first downsampled one); at least 1.  Replaces src/dimension.h:107-108. */
  uint8_t dims_n_append(const struct dimension* dims, uint8_t rank);

  /* 0 if the dims form a valid stream description.
   * Replaces src/dimension.h:114-115. */
  int dims_validate(const struct dimension* dims, uint8_t rank);

  /* Human-readable table on stderr.  Replaces src/dimension.h:118-119. */
  void dims_print(const struct dimension* dims, uint8_t rank);

#ifdef __cplusplus
}
#endif
