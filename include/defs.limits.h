/* Compile-time limits shared by the C API.
 * Values follow src/defs.limits.h:5-10 of the reference so that structs that
 * embed them (tile_stream_layout, lod arrays) keep the same layout. */
#pragma once

#define MAX_RANK 64
#define HALF_MAX_RANK (MAX_RANK / 2)
#define LOD_MAX_NDIM HALF_MAX_RANK
#define LOD_MAX_LEVELS 32
#define MAX_BATCH_EPOCHS 128
#define MAX_ZARR_RANK (HALF_MAX_RANK)
