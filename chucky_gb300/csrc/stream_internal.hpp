// Internal state of one GPU stream (not part of the C ABI).
#pragma once

#include "autotune.hpp"
#include "engine.hpp"
#include "kernels.hpp"
#include "plan.hpp"
#include "stream.gpu.h"

#include <cuda_runtime.h>
#include <vector>

namespace chucky {

struct Shard
{
  uint64_t cursor = 0; // bytes written so far
  shard_writer* w = nullptr;
};

struct Shards
{
  uint64_t epoch_in_shard = 0;
  uint64_t shard_epoch = 0;
  std::vector<Shard> sh;
};

// Mapped pinned host memory the aggregation kernel writes into.
struct DeliverySlot
{
  struct Level
  {
    uint64_t* offsets = nullptr;    // [positions + 1]
    uint64_t* real_sizes = nullptr; // [positions]
    uint8_t* data = nullptr;        // host (mapped) shard-ordered bytes
    uint8_t* d_data = nullptr;      // device copy (compressed codecs)
    uint64_t positions_cap = 0, data_cap = 0;
    uint64_t positions = 0;         // of the batch in the slot
    uint64_t copied = 0;            // bytes already copied to the host
    // shard index: the batch's runs of active epochs (host-written, read
    // by the index kernel) and the final index blobs of the shard epochs
    // the batch completes (written by the index kernel)
    IndexRun* runs = nullptr;       // mapped
    uint32_t n_runs = 0, runs_cap = 0;
    uint8_t* blobs = nullptr;       // mapped [finals_cap][shards][blob_bytes]
    uint32_t finals_cap = 0;
  };
  Level lv[LOD_MAX_LEVELS];
  uint32_t active[LOD_MAX_LEVELS] = {};
  int level_of[LOD_MAX_LEVELS] = {};
  int n_levels = 0;
  io_event fence[LOD_MAX_LEVELS] = {};
  std::vector<double> epoch_done_ms; // host time each epoch's input was in
  int busy = 0;
  uint64_t seq = 0;
};

struct Stream
{
  tile_stream_configuration cfg{};
  shard_sink* sink = nullptr;
  StreamPlan P;
  tile_stream_layout layout{};
  int device = 0;
  cudaStream_t s_copy = nullptr, s_comp = nullptr;

  // input
  uint8_t* d_epoch[2] = {};
  cudaEvent_t ev_input_ready[2] = {}, ev_input_free[2] = {};
  int in_buf = 0;
  uint64_t in_fill = 0;

  // Pinned staging ring for appends of pageable memory and small appends of
  // any host memory: `append` copies the caller's bytes into a slot with the
  // CPU and returns; the slot's copy to the epoch buffer runs on the copy
  // stream.  Consecutive appends that land next to each other in the epoch
  // buffer share a slot, whose copy is issued when it is full, when the
  // epoch is complete, or at the flush.  A slot is written again only after
  // its copy has finished (its event).
  static constexpr int kStageSlots = int(kStreamStageSlots);
  uint8_t* h_stage[kStageSlots] = {};
  cudaEvent_t ev_stage[kStageSlots] = {};
  bool stage_used[kStageSlots] = {};
  uint64_t stage_bytes = 0;  // bytes per slot
  int stage_cur = 0;         // slot being filled
  uint64_t stage_fill = 0;   // bytes in it not yet issued
  uint8_t* stage_dst = nullptr; // device destination of its first byte
  // appends of pinned host memory up to this size (256 KiB at most) go
  // through the ring
  uint64_t stage_small = 0;
  // stream-ordered appends of device memory (append_async)
  cudaEvent_t ev_producer = nullptr, ev_consumed = nullptr;

  // chunk pool / compression.  With a codec the pool has two halves, one
  // per delivery slot: the LOD of the next batch fills one half while the
  // encoders of the previous one read the other.  Each slot has its own
  // encoder stream and scratch, so consecutive batches' encoders overlap.
  uint8_t* d_pool = nullptr;
  uint64_t pool_half_bytes = 0; // 0: one pool (no codec)
  bool pool_claimed = false;    // the filling half waited for its last encode
  cudaStream_t s_enc[2] = {}; // encoders, one stream per delivery slot
  cudaEvent_t ev_pool_ready = nullptr;
  uint8_t* d_comp[2] = {}; // compressed slots, one per delivery slot
  cudaStream_t s_agg = nullptr; // aggregation (host-link bound) stream
  cudaEvent_t ev_codec_done[2] = {}, ev_agg_done[2] = {};
  uint64_t* d_sizes[2] = {}; // compressed sizes, one per delivery slot
  uint64_t comp_stride = 0;
  void* codec_state[2] = {}; // encoder scratch, one per delivery slot
  uint64_t wave_chunks = 0; // chunks per encoder launch
  uint32_t* h_chunk_ids[2] = {};   // pinned staging of the encode list
  uint32_t* d_chunk_ids[2] = {};
  // With a shared encoder engine (the served form) the stream has no
  // encoder scratch: each batch's chunks go to the engine as a job, whose
  // encoders signal ev_engine_done of the delivery slot.
  Engine* engine = nullptr;
  EncodeJob job[2];
  cudaEvent_t ev_engine_done[2] = {};
  // encoder parameters: the autotuner's for this stream's key (chosen at
  // the first batch when tuning is on), else the level's defaults
  TuneKey tune_key{};
  TuneParams tune{};
  bool tuned = false;

  // transpose
  uint64_t* d_row_off = nullptr;
  uint64_t* d_col_off = nullptr;
  TransposeArgs tr{};

  // LOD
  uint8_t* d_values = nullptr;
  uint8_t* d_accum = nullptr;
  uint64_t* d_ends = nullptr;
  uint32_t* d_gather_lut = nullptr;
  uint64_t* d_gather_fixed = nullptr;
  uint32_t* d_chunk_lut[LOD_MAX_LEVELS] = {};
  uint64_t* d_chunk_fixed[LOD_MAX_LEVELS] = {};
  uint64_t lod_nelem[LOD_MAX_LEVELS] = {};
  uint64_t level_beg[LOD_MAX_LEVELS] = {};
  uint64_t accum_beg[LOD_MAX_LEVELS] = {};
  uint64_t ends_beg[LOD_MAX_LEVELS] = {};
  uint32_t counts[LOD_MAX_LEVELS] = {};
  LodMortonArgs lod{};
  bool lod_tiled = false; // single-pass tile kernel instead of Morton path
  LodTileArgs tile{};

  // aggregation
  uint32_t* d_gather[LOD_MAX_LEVELS] = {};
  uint32_t* d_perm[LOD_MAX_LEVELS] = {};
  uint32_t* d_gather_tmp[2][LOD_MAX_LEVELS] = {};
  uint32_t* d_perm_tmp[2][LOD_MAX_LEVELS] = {};
  uint32_t* h_lut_stage[2][LOD_MAX_LEVELS] = {}; // per delivery slot
  // active epochs of the tables last uploaded to d_gather_tmp/d_perm_tmp
  // per slot and level (an unchanged pattern needs no new upload)
  std::vector<uint32_t> lut_eps[2][LOD_MAX_LEVELS];
  uint32_t lut_cap[LOD_MAX_LEVELS] = {};
  uint32_t planned_count[LOD_MAX_LEVELS] = {};
  uint64_t* d_agg_scratch = nullptr;
  // bytes per level copied device -> host with the batch (the rest, if
  // any, at delivery): the last batch's size plus a margin
  uint64_t agg_estimate[LOD_MAX_LEVELS] = {};
  uint64_t agg_prev_total[LOD_MAX_LEVELS] = {}; // the batch before the last
  uint64_t agg_scratch_slot = 0; // entries per delivery slot
  DeliverySlot slot[2];
  cudaEvent_t ev_batch[2] = {};
  int next_slot = 0;
  uint64_t batch_seq = 0;

  // shards
  Shards shards[LOD_MAX_LEVELS];
  // the shard index of the current shard epoch of every level, resident on
  // the device, and the padded index + crc32c bytes per shard
  uint64_t* d_index[LOD_MAX_LEVELS] = {};
  uint64_t* d_cursor[LOD_MAX_LEVELS] = {};
  uint64_t blob_bytes[LOD_MAX_LEVELS] = {};
  uint8_t* h_flush_blobs[LOD_MAX_LEVELS] = {}; // mapped [shards][blob_bytes]
  uint32_t kick_eis[LOD_MAX_LEVELS] = {}; // epoch in shard after the last kick
  io_event io_done[LOD_MAX_LEVELS] = {};

  // append-to-delivered latency per epoch (ms)
  std::vector<double> pending_epoch_ms; // epochs of the batch being filled
  // > 0: an append starts the batch being filled as a partial batch once
  // its oldest epoch has waited this long, and delivers finished batches
  double batch_deadline_ms = 0;
  std::vector<double> latencies_ms;

  // progress
  uint64_t cursor = 0, max_cursor = 0;
  uint32_t accumulated = 0;
  uint32_t masks[MAX_BATCH_EPOCHS] = {};
  int flushed = 0;

  // metrics: event pairs resolved lazily
  struct Timer
  {
    cudaEvent_t a = nullptr, b = nullptr;
    stream_metric* metric = nullptr;
    double in = 0, out = 0;
  };
  static constexpr size_t kMaxTimers = 64;
  Timer timers[kMaxTimers];
  size_t timers_used = 0;
  stream_metrics metrics{};

  int init(const tile_stream_configuration* c, shard_sink* s);
  void release();
  int setup_transpose();
  int setup_lod();
  int setup_aggregate();
  void build_luts(int l,
                  uint32_t n_active,
                  const uint32_t* eps,
                  uint32_t* gather,
                  uint32_t* perm) const;
  uint8_t* pool_slot(uint32_t e) const;
  int claim_pool();
  int run_epoch(uint64_t present);
  int kick_batch(uint32_t n_epochs, const uint32_t* epoch_masks);
  int batch_boundary();
  int deliver(int si);
  int drain_all();
  int deliver_ready(); // deliver the batches the GPU has finished, in order
  int finalize_level(int l);
  int write_index_blobs(int l, const uint8_t* blobs);
  cudaStream_t agg_stream() const { return cfg.codec.id != CODEC_NONE ? s_agg : s_comp; }
  int flush_all();
  writer_result append(slice in);
  // Device memory appended in stream order with `producer` (a cudaStream_t
  // of the caller): the copies wait for the producer's work so far, and the
  // producer's later work waits for the copies; the host does not wait.
  writer_result append_async(slice in, cudaStream_t producer);
  writer_result flush();
  int stage_issue();
  int stage_copy(uint8_t* dst, const uint8_t* src, uint64_t bytes);

  int codec_init();
  int codec_compress(const uint8_t* pool,
                     uint64_t nchunks,
                     const uint32_t* d_ids,
                     const ChunkRuns* runs,
                     uint8_t* out,
                     uint64_t* sizes,
                     void* scratch,
                     cudaStream_t st);
  void codec_release();

  int timed_begin(cudaStream_t st, stream_metric* m, double in, double out);
  int timed_end(cudaStream_t st);
  void resolve_timers(bool wait);
};

} // namespace chucky

// The C handle: the writer vtable must come first (the vtable callbacks
// recover the stream from the writer pointer).
struct tile_stream_gpu
{
  writer w;
  chucky::Stream impl;
};
