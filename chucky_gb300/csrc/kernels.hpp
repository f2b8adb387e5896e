// Host-side launchers of the sm_103a kernels (all asynchronous on `st`).
#pragma once

#include "common.cuh"
#include "kernels_codec.hpp"
#include "dtype.h"
#include "types.lod.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace chucky {

// ---- (a) transpose: row-major epoch -> chunk tiles -------------------------

struct TransposeArgs
{
  const uint8_t* src;      // epoch buffer, element 0 = first of the epoch
  uint8_t* dst;            // epoch slot of the chunk pool
  uint64_t n;              // elements present (a partial epoch may be short)
  uint32_t bpe;            // 1, 2, 4 or 8
  FastDiv width;           // innermost lifted extent (count x chunk)
  const uint64_t* row_off; // element offset of (row, 0) in the slot
  const uint64_t* col_off; // element offset of column x within a row
  int vector_ok;           // 16-byte runs stay contiguous and aligned
};
cudaError_t launch_transpose(const TransposeArgs& a, cudaStream_t st);

// ---- (b) LOD pyramid --------------------------------------------------------

// One epoch through the Morton-order path: gather L0 into Morton order,
// reduce every level from the one below, fold/emit the dim-0 accumulators
// and scatter the active levels into the chunk slot.
struct LodMortonArgs
{
  int dtype;
  int reduce_method;
  int append_method;
  int nlod;
  uint64_t fixed_count;
  const uint64_t* lod_nelem;       // host array [nlod]
  const uint64_t* level_beg;       // host array [nlod] (element offsets)
  const uint64_t* accum_beg;       // host array [nlod] (levels >= 1)
  const uint64_t* d_ends;          // device window ends, levels >= 1
  const uint64_t* ends_beg;        // host array [nlod] offset into d_ends
  const uint32_t* d_gather_lut;    // [lod_nelem[0]]
  const uint64_t* d_gather_fixed;  // [fixed_count]
  const uint32_t* const* d_chunk_lut;   // host array of device ptrs [nlod]
  const uint64_t* const* d_chunk_fixed; // host array of device ptrs [nlod]
};

cudaError_t launch_lod_gather(const LodMortonArgs& a,
                              const uint8_t* linear,
                              uint8_t* values,
                              cudaStream_t st);
cudaError_t launch_lod_reduce(const LodMortonArgs& a,
                              uint8_t* values,
                              cudaStream_t st);
cudaError_t launch_lod_fold(const LodMortonArgs& a,
                            int level,
                            uint32_t count,
                            const uint8_t* values,
                            uint8_t* accum,
                            cudaStream_t st);
cudaError_t launch_lod_emit(const LodMortonArgs& a,
                            int level,
                            uint32_t count,
                            const uint8_t* accum,
                            uint8_t* values,
                            cudaStream_t st);
cudaError_t launch_lod_to_chunks(const LodMortonArgs& a,
                                 int level,
                                 const uint8_t* values,
                                 uint8_t* slot,
                                 cudaStream_t st);

// Tiled single-pass pyramid (1..3 LOD dims, nlod - 1 <= lod_tile_levels).
struct LodTileArgs
{
  int dtype, method, append_method, nlod, lod_ndim;
  uint64_t fixed_count;
  const uint8_t* linear; // row-major epoch buffer
  uint8_t* slot;         // epoch slot of the chunk pool
  uint8_t* accum;        // dense dim-0 accumulators, levels >= 1
  uint32_t emit_mask;    // levels stored into the slot this epoch
  uint32_t fold_mask;    // levels folded into the accumulators
  uint32_t count[16];    // folds so far per level (before this epoch)
  uint64_t tiles[3];     // L0 tiles per LOD dim
  int64_t in_stride[3];  // epoch-buffer stride of each LOD dim
  uint32_t cs[3];        // chunk extent of each LOD dim
  const uint64_t* gather_fixed; // [fixed] epoch-buffer offset per slice
  struct Level
  {
    uint64_t shape[3];             // LOD extents at this level
    uint64_t S[3], s[3];           // chunk / within-chunk strides
    const uint64_t* chunk_fixed;   // [fixed] slot offset per slice
    uint64_t accum_off;            // level start in the accumulators
    uint64_t nelem;                // product of shape
    uint32_t off32;                // offsets within a chunk fit 32 bits
  } lv[16];
};
int lod_tile_levels(int lod_ndim);
uint32_t lod_tile_edge(int lod_ndim);
cudaError_t launch_lod_tile(const LodTileArgs& a, cudaStream_t st);
cudaError_t launch_lod_drain(const LodTileArgs& a,
                             int level,
                             uint32_t count,
                             cudaStream_t st);

// ---- (d) aggregation --------------------------------------------------------

// One level of one batch: n entries (active epochs x chunks per epoch).
struct AggLevel
{
  const uint32_t* gather;  // [n] compressed chunk index
  const uint32_t* perm;    // [n] covering position in shard order
  uint64_t n;              // number of mapped chunks
  uint64_t positions;      // n_active * covering
  uint64_t group;          // n_active * cps_inner (page-pad unit)
  uint64_t* offsets;       // [positions + 1] (written)
  uint64_t* real_sizes;    // [positions] pre-padding sizes (written)
  uint8_t* out;            // shard-ordered bytes (written)
};

struct AggBatch
{
  const uint8_t* comp;      // compressed chunk slots
  uint64_t comp_stride;     // bytes between slots
  const uint64_t* sizes;    // [chunks] compressed sizes
  uint64_t alignment;       // shard alignment (0 = none)
  int nlevels;
  AggLevel lv[32];
};

// sizes -> shard order -> page pad -> exclusive scan, then gather bytes.
cudaError_t launch_aggregate(const AggBatch& b,
                             uint64_t* scratch, // >= max positions
                             cudaStream_t st);

// Shard index (src/zarr/shard_delivery.c:36-102), built on the device.
// Per level the index of every shard of the current shard epoch
// (cps_total (offset, nbytes) u64 pairs, all ones for an empty slot) and
// each shard's file cursor stay resident on the device.  A batch's runs of
// consecutive active epochs add their chunks' entries; a run that completes
// the shard epoch then writes every shard's final index blob -- zero
// padding to the alignment, the index, its crc32c -- and resets the state.
struct IndexRun
{
  uint32_t a0;    // first active epoch of the run within the batch
  uint32_t run;   // epochs
  uint32_t eis0;  // epoch in shard of its first epoch
  uint32_t final; // the run completes the shard epoch
};
struct IndexLevel
{
  uint64_t* index;             // [shards][cps_total][2] (device)
  uint64_t* cursor;            // [shards] bytes in each shard file so far
  const uint64_t* offsets;     // the batch's shard-order offsets (or null)
  const uint64_t* real_sizes;  // pre-padding sizes
  const IndexRun* runs;        // [n_runs]
  uint32_t n_runs;
  uint32_t n_active;           // active epochs of the level in the batch
  uint64_t cpi;                // chunks per shard per epoch (inner)
  uint64_t cps_total;          // index entries per shard
  uint64_t shards;             // shards per shard epoch
  uint8_t* blobs;              // [finalisations][shards][blob_bytes] (mapped)
  uint64_t blob_bytes;         // padded index + crc32c
  int flush;                   // finalise every shard now (no runs)
};
struct IndexBatch
{
  uint64_t alignment;
  int nlevels;
  uint64_t max_shards;
  IndexLevel lv[32];
};
cudaError_t launch_index(const IndexBatch& b, cudaStream_t st);

// The rest of a batch's shard-ordered bytes after a copy-engine transfer of
// the expected size: per level, bytes [start, *total) of `src` (device) to
// `dst` (mapped host memory), where *total is the level's byte count the
// aggregation wrote on the device.  `max_bytes` bounds total - start.
struct TailCopy
{
  uint8_t* dst;
  const uint8_t* src; // readable 20 bytes past *total + extra
  const uint64_t* total;
  uint64_t extra;     // bytes copied past *total (the alignment slack)
  uint64_t start;
};
struct TailCopies
{
  int n;
  TailCopy lv[32];
};
cudaError_t launch_tail_copy(const TailCopies& t, uint64_t max_bytes, cudaStream_t st);

cudaError_t launch_fill_u64(uint64_t* p, uint64_t v, uint64_t n, cudaStream_t st);

// n 32-bit words from mapped pinned host memory to the device with SM
// loads.  Small host-built tables (chunk lists, shard-order tables) travel
// this way rather than as copy-engine transfers, which would queue behind
// the large input copies to the device that are in flight at the time.
cudaError_t launch_stage_copy(uint32_t* dst, const uint32_t* src, uint64_t n,
                              cudaStream_t st);

} // namespace chucky
