// Encoder autotuner (see autotune.hpp).
#include "autotune.hpp"
#include "plan.hpp"

#include "chucky_gb300.h"
#include "types.codec.h"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace chucky {

bool TuneKey::operator<(const TuneKey& o) const
{
  if (codec != o.codec)
    return codec < o.codec;
  if (level != o.level)
    return level < o.level;
  if (dtype != o.dtype)
    return dtype < o.dtype;
  if (rank != o.rank)
    return rank < o.rank;
  return std::lexicographical_compare(chunk, chunk + 16, o.chunk, o.chunk + 16);
}

namespace {

struct Entry
{
  TuneParams p;
  uint64_t chunk_bytes = 0;
  double encode_gbs = 0, ratio = 0;
  uint32_t candidates = 0; // 0: not tuned (defaults)
};

// Per-device trial resources, kept for the process.
struct DeviceRes
{
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  uint8_t* out = nullptr;
  size_t out_bytes = 0;
  uint64_t* sizes = nullptr;
  ChunkRef* refs = nullptr; // kMaxSample entries
  double d2h_gbs = 0;
};

constexpr uint32_t kMaxSample = 16;
constexpr uint64_t kMaxSampleBytes = 64ull << 20;

std::mutex g_m;
std::map<TuneKey, Entry> g_table;
std::map<int, DeviceRes> g_dev;
std::atomic<int> g_enabled{ -1 }; // -1: the environment not read yet

struct Candidate
{
  int strength, min_match;
};

// The candidates of a (codec, level); the first is the defaults.
std::vector<Candidate> candidates(int codec, int level)
{
  const bool wide = codec == CODEC_ZSTD ? level >= 3 : level >= 2;
  const int strengths_fast[] = { 0, 4, 5, 7, 8 }; // 0: the default (6)
  const int strengths_wide[] = { 0, 5, 7 };
  std::vector<int> mm;
  if (wide)
    mm = { 0 };
  else if (codec == CODEC_ZSTD)
    mm = { 0, 6, 12 }; // 0: the default (8)
  else
    mm = { 0, 5, 6 }; // 0: 4, LZ4's shortest
  std::vector<Candidate> out;
  for (int m : mm) {
    if (wide)
      for (int s : strengths_wide)
        out.push_back({ s, m });
    else
      for (int s : strengths_fast)
        out.push_back({ s, m });
  }
  return out;
}

bool reserve(void** p, size_t* have, size_t need)
{
  if (*have >= need)
    return true;
  cudaFree(*p);
  *p = nullptr;
  *have = 0;
  need = (need + (16u << 20) - 1) / (16u << 20) * (16u << 20);
  if (cudaMalloc(p, need) != cudaSuccess)
    return false;
  *have = need;
  return true;
}

// Device-to-host copy rate, once per device (best of three 32 MiB copies
// into pinned memory).
double measure_d2h(DeviceRes& R)
{
  constexpr size_t kBytes = 32u << 20;
  void* d = nullptr;
  void* h = nullptr;
  double best = 0;
  if (cudaMalloc(&d, kBytes) == cudaSuccess &&
      cudaHostAlloc(&h, kBytes, cudaHostAllocDefault) == cudaSuccess) {
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(R.e0, R.st);
      cudaMemcpyAsync(h, d, kBytes, cudaMemcpyDeviceToHost, R.st);
      cudaEventRecord(R.e1, R.st);
      float ms = 0;
      if (cudaEventSynchronize(R.e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, R.e0, R.e1) != cudaSuccess || ms <= 0)
        break;
      best = std::max(best, kBytes / (ms * 1e-3) / 1e9);
    }
  }
  cudaFree(d);
  cudaFreeHost(h);
  cudaGetLastError();
  return best > 0 ? best : 100.0;
}

// One candidate on the sample: best of two timed runs after a warm-up.
bool trial(DeviceRes& R,
           const TuneKey& key,
           uint32_t cb,
           uint32_t n,
           const Candidate& c,
           double& secs,
           double& bytes)
{
  CodecBatch b{};
  b.chunk_bytes = cb;
  b.n_chunks = n;
  b.level = key.level;
  b.strength = c.strength;
  b.min_match = c.min_match;
  b.refs = R.refs;
  auto launch = [&]() {
    return key.codec == CODEC_ZSTD ? launch_zstd(b, R.scratch, R.st)
                                   : launch_lz4(b, R.scratch, R.st);
  };
  if (launch() != cudaSuccess)
    return false;
  float best = 1e30f;
  for (int r = 0; r < 2; ++r) {
    float ms = 0;
    if (cudaEventRecord(R.e0, R.st) != cudaSuccess || launch() != cudaSuccess ||
        cudaEventRecord(R.e1, R.st) != cudaSuccess ||
        cudaEventSynchronize(R.e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, R.e0, R.e1) != cudaSuccess)
      return false;
    best = std::min(best, ms);
  }
  std::vector<uint64_t> h(n);
  if (cudaMemcpy(h.data(), R.sizes, n * sizeof(uint64_t), cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return false;
  bytes = 0;
  for (uint64_t v : h)
    bytes += double(v);
  secs = best * 1e-3;
  return true;
}

bool tune(const TuneKey& key,
          uint32_t cb,
          const uint8_t* const* sample,
          uint32_t n,
          cudaEvent_t ready,
          Entry& E)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return false;
  DeviceRes& R = g_dev[dev];
  if (!R.st) {
    if (cudaStreamCreateWithFlags(&R.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&R.e0) != cudaSuccess || cudaEventCreate(&R.e1) != cudaSuccess)
      return false;
    R.d2h_gbs = measure_d2h(R);
  }
  const uint64_t stride = (codec_bound(key.codec, cb) + 15) / 16 * 16;
  const size_t scratch = key.codec == CODEC_ZSTD ? zstd_scratch_bytes(n, cb, key.level)
                                                 : lz4_scratch_bytes(n, cb, key.level);
  if (!reserve(&R.scratch, &R.scratch_bytes, scratch) ||
      !reserve(reinterpret_cast<void**>(&R.out), &R.out_bytes, n * stride))
    return false;
  if (!R.refs) { // room for the largest sample
    if (cudaMalloc(&R.refs, kMaxSample * sizeof(ChunkRef)) != cudaSuccess ||
        cudaMalloc(&R.sizes, kMaxSample * sizeof(uint64_t)) != cudaSuccess)
      return false;
  }
  std::vector<ChunkRef> h(n);
  for (uint32_t i = 0; i < n; ++i)
    h[i] = ChunkRef{ sample[i], R.out + i * stride, R.sizes + i };
  if (cudaMemcpy(R.refs, h.data(), n * sizeof(ChunkRef), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return false;
  if (ready && cudaStreamWaitEvent(R.st, ready, 0) != cudaSuccess)
    return false;
  const std::vector<Candidate> cand = candidates(key.codec, key.level);
  std::vector<double> secs(cand.size()), bytes(cand.size());
  for (size_t i = 0; i < cand.size(); ++i)
    if (!trial(R, key, cb, n, cand[i], secs[i], bytes[i]))
      return false;
  const double in_bytes = double(n) * cb;
  const int k = autotune_pick(secs.data(), bytes.data(), int(cand.size()), in_bytes,
                              R.d2h_gbs, 0);
  E.p = TuneParams{ cand[k].strength, cand[k].min_match };
  E.encode_gbs = in_bytes / secs[k] / 1e9;
  E.ratio = in_bytes / std::max(1.0, bytes[k]);
  E.candidates = uint32_t(cand.size());
  return true;
}

} // namespace

bool autotune_enabled()
{
  int e = g_enabled.load();
  if (e < 0) {
    const char* v = std::getenv("CHUCKY_AUTOTUNE");
    e = v && v[0] == '1' ? 1 : 0;
    int expected = -1;
    g_enabled.compare_exchange_strong(expected, e);
    e = g_enabled.load();
  }
  return e == 1;
}

void autotune_set_enabled(bool on)
{
  g_enabled.store(on ? 1 : 0);
}

int autotune_pick(const double* enc_s,
                  const double* out_bytes,
                  int n,
                  double in_bytes,
                  double d2h_gbs,
                  int preferred)
{
  if (n <= 0 || in_bytes <= 0)
    return 0;
  // eligible: no more than 1 % above the preferred candidate's output (the
  // defaults'; without one, the smallest output): the tuner buys speed or
  // ratio, never speed with ratio
  const bool pref = preferred >= 0 && preferred < n;
  double least = pref ? out_bytes[preferred] : out_bytes[0];
  if (!pref)
    for (int i = 1; i < n; ++i)
      least = std::min(least, out_bytes[i]);
  std::vector<double> cost(n);
  int best = -1;
  for (int i = 0; i < n; ++i) {
    const double a = enc_s[i] / in_bytes;                       // encode, s per byte
    const double c = out_bytes[i] / in_bytes / (d2h_gbs * 1e9); // copy-out
    cost[i] = std::max(a, c) + 0.25 * std::min(a, c);
    if (out_bytes[i] <= 1.01 * least && (best < 0 || cost[i] < cost[best]))
      best = i;
  }
  if (pref && cost[preferred] <= 1.01 * cost[best])
    return preferred;
  return best;
}

TuneParams autotune(const TuneKey& key,
                    uint32_t chunk_bytes,
                    const uint8_t* const* sample,
                    uint32_t n,
                    cudaEvent_t ready)
{
  if (!autotune_enabled() || n == 0 || chunk_bytes == 0 ||
      (key.codec != CODEC_LZ4_NON_STANDARD && key.codec != CODEC_ZSTD))
    return TuneParams{};
  std::lock_guard<std::mutex> lk(g_m);
  auto it = g_table.find(key);
  if (it != g_table.end())
    return it->second.p;
  Entry E;
  E.chunk_bytes = chunk_bytes;
  n = std::min<uint32_t>(n, kMaxSample);
  n = std::min<uint32_t>(n, uint32_t(std::max<uint64_t>(1, kMaxSampleBytes / chunk_bytes)));
  if (!tune(key, chunk_bytes, sample, n, ready, E)) {
    cudaGetLastError();
    E = Entry{};
    E.chunk_bytes = chunk_bytes;
  }
  g_table[key] = E;
  return E.p;
}

} // namespace chucky

// ---- C API (include/chucky_gb300.h) -----------------------------------------

extern "C" void
chucky_autotune_set_enabled(int on)
{
  chucky::autotune_set_enabled(on != 0);
}

extern "C" int
chucky_autotune_enabled(void)
{
  return chucky::autotune_enabled() ? 1 : 0;
}

extern "C" size_t
chucky_autotune_entries(struct chucky_autotune_entry* out, size_t cap)
{
  std::lock_guard<std::mutex> lk(chucky::g_m);
  size_t i = 0;
  for (const auto& kv : chucky::g_table) {
    if (out && i < cap) {
      chucky_autotune_entry& e = out[i];
      std::memset(&e, 0, sizeof e);
      e.codec = kv.first.codec;
      e.level = kv.first.level;
      e.dtype = kv.first.dtype;
      e.rank = kv.first.rank;
      for (int k = 0; k < 16 && k < kv.first.rank; ++k)
        e.chunk_shape[k] = kv.first.chunk[k];
      e.chunk_bytes = kv.second.chunk_bytes;
      e.strength = kv.second.p.strength;
      e.min_match = kv.second.p.min_match;
      e.encode_gbs = kv.second.encode_gbs;
      e.ratio = kv.second.ratio;
      e.candidates = kv.second.candidates;
    }
    ++i;
  }
  return i;
}

extern "C" void
chucky_autotune_clear(void)
{
  std::lock_guard<std::mutex> lk(chucky::g_m);
  chucky::g_table.clear();
}

extern "C" int
chucky_autotune_pick(const double* enc_s,
                     const double* out_bytes,
                     int n,
                     double in_bytes,
                     double d2h_gbs,
                     int preferred)
{
  return chucky::autotune_pick(enc_s, out_bytes, n, in_bytes, d2h_gbs, preferred);
}
