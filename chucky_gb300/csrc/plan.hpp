// Stream layout planning (host only).
//
// Produces every derived quantity of a stream configuration: the epoch-split
// level shapes of the LOD pyramid, the lifted chunk layout of each level, the
// window ends used by the Morton-order reduction, the per-level shard
// geometry and aggregate (shard-order) layout, and the batch size K.
// The arithmetic restates the reference planner:
//   src/stream/config.c:31-376      (validation, level layouts, K, geometry)
//   src/lod/lod_plan.c:12-370       (Morton ranks, window ends, level shapes)
//   src/stream/types.aggregate.c:28-143 (shard-order permutation)
//   src/util/index.ops.c:97-113     (lifted strides)
#pragma once

#include "stream.gpu.h"

#include <cstdint>
#include <vector>

namespace chucky {

struct LevelPlan
{
  uint64_t shape[HALF_MAX_RANK] = {}; // epoch-split extent of every dim
  uint64_t lod_nelem = 1;             // product of the LOD-dim extents
  tile_stream_layout layout = {};     // lifted chunk layout of one epoch
  uint64_t chunk_offset = 0;          // first chunk of this level in a slot

  // shard geometry / aggregate layout (storage-ordered inner dims)
  uint8_t agg_rank = 0;
  uint64_t agg_shape[MAX_RANK] = {};
  int64_t agg_strides[MAX_RANK] = {};
  uint64_t covering = 0;          // C >= chunks_per_epoch
  uint64_t cps_inner = 1;         // chunks of one shard inside an epoch
  uint64_t cps_append = 1;        // epochs per shard
  uint64_t cps_total = 1;         // index slots per shard
  uint64_t shard_inner_count = 1; // shards per shard-epoch
  uint32_t batch_active = 0;      // epochs active in a full batch
  uint32_t period = 1;            // emits every `period` epochs
};

struct StreamPlan
{
  uint8_t rank = 0, na = 1;
  uint64_t bpe = 0;
  int append_downsample = 0;
  uint32_t lod_mask = 0;
  uint8_t order[HALF_MAX_RANK] = {}; // storage position -> dim
  int multiscale = 0;
  int nlod = 1;
  int lod_ndim = 0;
  int lod_to_dim[LOD_MAX_NDIM] = {};
  int fixed_ndim = 0;
  int fixed_to_dim[LOD_MAX_NDIM] = {};
  uint64_t fixed_shape[LOD_MAX_NDIM] = {};
  uint64_t fixed_count = 1;
  uint64_t lod_end[LOD_MAX_LEVELS] = {}; // cumulative lod_nelem
  std::vector<uint64_t> ends;            // Morton window ends, levels >= 1
  LevelPlan lv[LOD_MAX_LEVELS];
  uint64_t total_chunks = 0;
  uint32_t K = 1;
  uint64_t max_out = 0;     // bound on one compressed chunk
  uint64_t max_cursor = 0;  // 0 = unbounded
  uint64_t chunk_bytes = 0; // chunk_elements * bpe (codec input)
  uint64_t slot_bytes = 0;  // one epoch of every level in the pool
  uint64_t epoch_bytes = 0; // epoch_elements * bpe (input per epoch)
  uint64_t n_ends = 0;      // entries of the Morton window-end table
};

// Alignment of chunk strides in the chunk pool (bytes).  Chunk strides only
// pad the pool; codec input is always chunk_elements * bpe.
constexpr uint64_t kChunkAlign = 256;

// Worst-case compressed size of one chunk for this library's encoders.
uint64_t codec_bound(int codec_id, uint64_t chunk_bytes);

// 0 on success.  Validation follows src/stream/config.c:144-221.
int plan_stream(const tile_stream_configuration* cfg, StreamPlan* out);

// Fill P.ends (P.n_ends entries), the Morton window ends the general LOD
// path reads; plan_stream leaves it empty.
void plan_build_ends(StreamPlan& P);

// The tiled single-pass pyramid kernel covers this plan (it needs neither
// the window-end table nor Morton-ordered level buffers).
bool lod_plan_is_tiled(const StreamPlan& P);

uint64_t morton_rank(int ndim,
                     const uint64_t* shape,
                     const uint64_t* coords,
                     int depth);

uint64_t ravel(int rank,
               const uint64_t* shape,
               const int64_t* strides,
               uint64_t idx);

// Pinned staging slots of a stream.
constexpr uint64_t kStreamStageSlots = 4;

// Bytes of one pinned staging slot of a stream (it keeps four): a quarter
// of the configured buffer capacity, 256 KiB to 32 MiB, in whole 4 KiB pages.
inline uint64_t staging_slot_bytes(uint64_t buffer_capacity_bytes)
{
  uint64_t b = buffer_capacity_bytes / 4;
  b = b < (256ull << 10) ? (256ull << 10) : b;
  b = b > (32ull << 20) ? (32ull << 20) : b;
  return (b + 4095) / 4096 * 4096;
}

} // namespace chucky
