// Shared encoder engine (engine.hpp).
#include "engine.hpp"

#include "kernels.hpp"
#include "types.codec.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>

namespace chucky {

namespace {

#define ECK(expr)                                                              \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "chucky_gb300 engine: %s failed: %s (%s:%d)\n",     \
                   #expr, cudaGetErrorString(e_), __FILE__, __LINE__);         \
      return 1;                                                                \
    }                                                                          \
  } while (0)

constexpr uint64_t kRefWords = sizeof(ChunkRef) / 4;
static_assert(sizeof(ChunkRef) % 4 == 0, "references travel as 32-bit words");

} // namespace

int Engine::init(uint64_t wave_bytes, int lanes)
{
  ECK(cudaGetDevice(&device_));
  wave_bytes_ = wave_bytes;
  lanes_ = std::max(1, std::min(lanes, kMaxLanes));
  for (int i = 0; i < lanes_; ++i)
    ECK(cudaStreamCreateWithFlags(&lane_[i].st, cudaStreamNonBlocking));
  h_refs_cap_ = 1 << 14;
  for (int i = 0; i < kHostRefSlots; ++i) {
    ECK(cudaHostAlloc(&h_refs_[i], h_refs_cap_ * sizeof(ChunkRef), cudaHostAllocMapped));
    ECK(cudaEventCreateWithFlags(&h_refs_free_[i], cudaEventDisableTiming));
  }
  thread_ = std::thread([this] { loop(); });
  return 0;
}

Engine::~Engine()
{
  {
    std::lock_guard<std::mutex> lk(m_);
    stop_ = true;
  }
  cv_jobs_.notify_all();
  if (thread_.joinable())
    thread_.join();
  for (Lane& L : lane_) {
    if (L.st) {
      cudaStreamSynchronize(L.st);
      cudaStreamDestroy(L.st);
    }
    cudaFree(L.scratch);
    cudaFree(L.d_refs);
  }
  for (int i = 0; i < kHostRefSlots; ++i) {
    cudaFreeHost(h_refs_[i]);
    if (h_refs_free_[i])
      cudaEventDestroy(h_refs_free_[i]);
  }
}

int Engine::run(EncodeJob& job)
{
  std::unique_lock<std::mutex> lk(m_);
  job.enqueued = false;
  job.rc = 0;
  queue_.push_back(&job);
  cv_jobs_.notify_one();
  cv_done_.wait(lk, [&] { return job.enqueued; });
  return job.rc;
}

EngineStats Engine::stats()
{
  std::lock_guard<std::mutex> lk(m_);
  return stats_;
}

void Engine::loop()
{
  cudaSetDevice(device_);
  std::unique_lock<std::mutex> lk(m_);
  for (;;) {
    cv_jobs_.wait(lk, [&] { return stop_ || !queue_.empty(); });
    if (queue_.empty())
      break; // stopping
    std::vector<EncodeJob*> jobs(queue_.begin(), queue_.end());
    queue_.clear();
    lk.unlock();
    const int rc = process(jobs);
    lk.lock();
    stats_.rounds++;
    stats_.jobs += jobs.size();
    stats_.max_jobs_per_round = std::max<uint64_t>(stats_.max_jobs_per_round, jobs.size());
    for (EncodeJob* j : jobs) {
      stats_.chunks += j->n;
      stats_.input_bytes += j->n * j->chunk_bytes;
      j->rc = rc;
      j->enqueued = true;
    }
    cv_done_.notify_all();
  }
}

int Engine::reserve_scratch(Lane& L, size_t bytes)
{
  if (bytes <= L.scratch_bytes)
    return 0;
  ECK(cudaStreamSynchronize(L.st)); // earlier rounds may still use it
  cudaFree(L.scratch);
  L.scratch = nullptr;
  L.scratch_bytes = 0;
  ECK(cudaMalloc(&L.scratch, bytes));
  L.scratch_bytes = bytes;
  return 0;
}

// One round: every job waits for its inputs on the lane's stream, then each
// (codec, level, parse parameters, chunk bytes) group is encoded as one
// batch, then every
// job's `done` event is recorded.
int Engine::process(std::vector<EncodeJob*>& jobs)
{
  Lane& L = lane_[next_lane_];
  next_lane_ = (next_lane_ + 1) % lanes_;
  for (EncodeJob* j : jobs) {
    ECK(cudaStreamWaitEvent(L.st, j->ready, 0));
    if (j->out_free)
      ECK(cudaStreamWaitEvent(L.st, j->out_free, 0));
  }
  std::map<std::tuple<int, int, int, int, uint32_t>, std::vector<EncodeJob*>> groups;
  for (EncodeJob* j : jobs)
    if (j->n)
      groups[std::make_tuple(j->codec, j->level, j->strength, j->min_match,
                             j->chunk_bytes)].push_back(j);
  for (auto& g : groups)
    if (encode_group(L, g.second))
      return 1;
  for (EncodeJob* j : jobs)
    ECK(cudaEventRecord(j->done, L.st));
  return 0;
}

int Engine::encode_group(Lane& L, std::vector<EncodeJob*>& group)
{
  const EncodeJob& first = *group.front();
  const uint32_t cb = first.chunk_bytes;
  uint64_t total = 0;
  for (EncodeJob* j : group)
    total += j->n;
  const uint64_t wave = std::max<uint64_t>(
    1, std::min<uint64_t>(total, wave_bytes_ / std::max<uint32_t>(1, cb)));
  const size_t need = first.codec == CODEC_ZSTD ? zstd_scratch_bytes(wave, cb, first.level)
                                                : lz4_scratch_bytes(wave, cb, first.level);
  if (reserve_scratch(L, need))
    return 1;
  if (total > L.refs_cap) {
    ECK(cudaStreamSynchronize(L.st));
    cudaFree(L.d_refs);
    L.d_refs = nullptr;
    L.refs_cap = std::max<uint64_t>(total, 2 * L.refs_cap);
    ECK(cudaMalloc(&L.d_refs, L.refs_cap * sizeof(ChunkRef)));
  }
  // the group's chunk references, staged through pinned memory in pieces
  // of at most one host slot
  uint64_t done_refs = 0;
  size_t ji = 0;
  uint64_t within = 0;
  while (done_refs < total) {
    const int h = next_host_;
    next_host_ = (next_host_ + 1) % kHostRefSlots;
    if (h_refs_used_[h])
      ECK(cudaEventSynchronize(h_refs_free_[h]));
    const uint64_t n = std::min<uint64_t>(h_refs_cap_, total - done_refs);
    ChunkRef* r = h_refs_[h];
    for (uint64_t k = 0; k < n; ++k) {
      while (within >= group[ji]->n) {
        ++ji;
        within = 0;
      }
      const EncodeJob& j = *group[ji];
      const uint32_t s = j.slots[within++];
      r[k].in = j.pool + uint64_t(s) * j.in_stride;
      r[k].out = j.out + uint64_t(s) * j.out_stride;
      r[k].size = j.sizes + s;
    }
    ECK(launch_stage_copy(reinterpret_cast<uint32_t*>(L.d_refs + done_refs),
                          reinterpret_cast<const uint32_t*>(r), n * kRefWords, L.st));
    ECK(cudaEventRecord(h_refs_free_[h], L.st));
    h_refs_used_[h] = true;
    done_refs += n;
  }
  for (uint64_t f = 0; f < total; f += wave) {
    CodecBatch b{};
    b.chunk_bytes = cb;
    b.n_chunks = std::min<uint64_t>(wave, total - f);
    b.level = first.level;
    b.strength = first.strength;
    b.min_match = first.min_match;
    b.refs = L.d_refs + f;
    const cudaError_t e = first.codec == CODEC_ZSTD ? launch_zstd(b, L.scratch, L.st)
                                                    : launch_lz4(b, L.scratch, L.st);
    if (e != cudaSuccess) {
      std::fprintf(stderr, "chucky_gb300 engine: encoder launch failed: %s\n",
                   cudaGetErrorString(e));
      return 1;
    }
    std::lock_guard<std::mutex> lk(m_);
    stats_.launch_sets++;
  }
  return 0;
}

} // namespace chucky
