// Shared encoder engine of the served form: the batches of many streams
// encoded by common launches.
//
// A stream created with an engine does not launch its own encoders.  At a
// batch boundary it hands the engine an EncodeJob (its chunk slots, where
// the compressed chunks and sizes go, the event that says its chunk pool is
// filled) and waits until the engine has enqueued the job's encoders.  The
// engine thread takes every job queued at that moment, groups them by
// (codec, level, parse parameters, chunk bytes) and encodes each group as one batch over a list of
// per-chunk addresses (CodecBatch::refs) -- one launch set for the chunks
// of all streams, in waves of at most `wave_bytes` of input -- on one of
// two engine CUDA streams (consecutive rounds alternate, so they overlap on
// the device).  It then records each job's `done` event, after which the
// stream's aggregation may read the compressed chunks.
//
// Every chunk is encoded exactly as a stream encoding alone would encode it
// (the encoders work per chunk), so a stream's output does not depend on
// which other streams shared its launches.
#pragma once

#include "kernels_codec.hpp"

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace chucky {

struct EncodeJob
{
  int codec = 0;             // CODEC_LZ4_NON_STANDARD or CODEC_ZSTD
  int level = 0;
  int strength = 0, min_match = 0; // parse parameters (CodecBatch)
  uint32_t chunk_bytes = 0;  // codec input per chunk
  const uint8_t* pool = nullptr; // chunk slot s at pool + s * in_stride
  uint64_t in_stride = 0;
  const uint32_t* slots = nullptr; // [n] chunk slots to encode (host)
  uint64_t n = 0;
  uint8_t* out = nullptr;    // compressed slot s at out + s * out_stride
  uint64_t out_stride = 0;
  uint64_t* sizes = nullptr; // compressed size of slot s at sizes[s]
  cudaEvent_t ready = nullptr;    // the pool is filled
  cudaEvent_t out_free = nullptr; // `out` / `sizes` may be overwritten
  cudaEvent_t done = nullptr;     // recorded by the engine after encoding
  // filled in by the engine
  bool enqueued = false;
  int rc = 0;
};

struct EngineStats
{
  uint64_t rounds = 0, jobs = 0, chunks = 0, launch_sets = 0;
  uint64_t input_bytes = 0;
  uint64_t max_jobs_per_round = 0;
};

class Engine
{
public:
  // Scratch and reference lists for waves of up to wave_bytes of input, on
  // the current device, with `lanes` engine CUDA streams (1..kMaxLanes;
  // consecutive rounds go to consecutive lanes and may overlap on the
  // device).  Returns 0 on success.
  int init(uint64_t wave_bytes, int lanes);
  ~Engine();

  // Enqueue the job's encoders with the next round; returns once they are
  // enqueued (job.rc: 0 or an error).
  int run(EncodeJob& job);

  EngineStats stats();

private:
  struct Lane
  {
    cudaStream_t st = nullptr;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    ChunkRef* d_refs = nullptr;
    uint64_t refs_cap = 0;
  };
  static constexpr int kMaxLanes = 8;
  static constexpr int kHostRefSlots = 8;

  void loop();
  int process(std::vector<EncodeJob*>& jobs);
  int encode_group(Lane& L, std::vector<EncodeJob*>& group);
  int reserve_scratch(Lane& L, size_t bytes);

  int device_ = 0;
  uint64_t wave_bytes_ = 0;
  Lane lane_[kMaxLanes];
  int lanes_ = 2;
  int next_lane_ = 0;
  // pinned host staging of reference lists, each reused after its copy to
  // the device has run
  ChunkRef* h_refs_[kHostRefSlots] = {};
  cudaEvent_t h_refs_free_[kHostRefSlots] = {};
  bool h_refs_used_[kHostRefSlots] = {};
  uint64_t h_refs_cap_ = 0;
  int next_host_ = 0;

  std::mutex m_;
  std::condition_variable cv_jobs_, cv_done_;
  std::deque<EncodeJob*> queue_;
  bool stop_ = false;
  std::thread thread_;
  EngineStats stats_{};
};

} // namespace chucky
