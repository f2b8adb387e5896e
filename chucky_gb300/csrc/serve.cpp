// Served form (include/chucky_serve.h): resident GPU streams handed to
// requests under an HBM budget, encoders batched across streams by a shared
// engine, and a request-loop driver.
#include "chucky_serve.h"
#include "chucky_gb300.h"
#include "autotune.hpp"
#include "engine.hpp"
#include "stream_internal.hpp"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace chucky {
tile_stream_gpu* create_stream(const tile_stream_configuration* config,
                               shard_sink* sink,
                               Engine* engine);
int estimate_stream(const tile_stream_configuration* config,
                    tile_stream_memory_info* info,
                    bool shared_encoder);
} // namespace chucky

namespace {

// Everything of a configuration that shapes its stream's allocations and
// output (the dimension values, not the pointer to them).
std::string config_key(const tile_stream_configuration* c)
{
  std::string k;
  auto put = [&](const void* p, size_t n) {
    k.append(static_cast<const char*>(p), n);
  };
  put(&c->buffer_capacity_bytes, sizeof c->buffer_capacity_bytes);
  put(&c->dtype, sizeof c->dtype);
  put(&c->rank, sizeof c->rank);
  put(&c->codec.id, sizeof c->codec.id);
  put(&c->codec.level, sizeof c->codec.level);
  put(&c->codec.shuffle, sizeof c->codec.shuffle);
  put(&c->reduce_method, sizeof c->reduce_method);
  put(&c->append_reduce_method, sizeof c->append_reduce_method);
  put(&c->max_nlod, sizeof c->max_nlod);
  put(&c->epochs_per_batch, sizeof c->epochs_per_batch);
  put(&c->target_batch_chunks, sizeof c->target_batch_chunks);
  put(&c->shard_alignment, sizeof c->shard_alignment);
  for (int d = 0; d < c->rank; ++d) {
    const dimension& D = c->dimensions[d];
    put(&D.size, sizeof D.size);
    put(&D.chunk_size, sizeof D.chunk_size);
    put(&D.chunks_per_shard, sizeof D.chunks_per_shard);
    put(&D.downsample, sizeof D.downsample);
    put(&D.storage_position, sizeof D.storage_position);
    k += D.name ? D.name : "";
    k += '\0';
  }
  return k;
}

double now_s()
{
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Idle
{
  tile_stream_gpu* s;
  uint64_t bytes;
  std::string key;
};

} // namespace

struct chucky_server
{
  chucky_server_config cfg{};
  int device = 0;
  std::unique_ptr<chucky::Engine> engine;
  std::mutex m;
  std::condition_variable cv;
  std::list<Idle> idle; // least recently released first
  std::map<std::string, uint64_t> need; // device estimate per configuration
  uint64_t resident = 0;
  int open = 0;
  // statistics
  std::vector<double> lat_ms;
  uint64_t requests = 0, input_bytes = 0, created = 0, reused = 0, evicted = 0;
  uint64_t peak_resident = 0, peak_open = 0;
};

struct chucky_request
{
  chucky_server* srv = nullptr;
  tile_stream_gpu* s = nullptr;
  uint64_t bytes = 0; // device estimate charged to the budget
  std::string key;
};

extern "C" chucky_server*
chucky_server_create(const chucky_server_config* config)
{
  if (!config || config->max_streams < 1 || !config->hbm_budget_bytes ||
      !(config->batch_deadline_ms >= 0))
    return nullptr;
  auto* s = new (std::nothrow) chucky_server();
  if (!s)
    return nullptr;
  s->cfg = *config;
  if (cudaGetDevice(&s->device) != cudaSuccess) {
    delete s;
    return nullptr;
  }
  if (config->autotune)
    chucky::autotune_set_enabled(true);
  if (config->batch_encoders) {
    s->engine.reset(new (std::nothrow) chucky::Engine());
    const uint64_t wave = config->encoder_wave_bytes ? config->encoder_wave_bytes
                                                     : (256ull << 20);
    const int lanes = config->encoder_lanes > 0 ? config->encoder_lanes : 2;
    if (!s->engine || s->engine->init(wave, lanes)) {
      delete s;
      return nullptr;
    }
  }
  return s;
}

extern "C" void
chucky_server_destroy(chucky_server* s)
{
  if (!s)
    return;
  cudaSetDevice(s->device);
  for (Idle& i : s->idle)
    tile_stream_gpu_destroy(i.s);
  s->idle.clear();
  s->engine.reset();
  delete s;
}

extern "C" chucky_request*
chucky_server_open(chucky_server* s,
                   const tile_stream_configuration* config,
                   shard_sink* sink,
                   int timeout_ms)
{
  if (!s || !config || !sink)
    return nullptr;
  if (cudaSetDevice(s->device) != cudaSuccess)
    return nullptr;
  const std::string key = config_key(config);
  uint64_t need = 0;
  {
    std::lock_guard<std::mutex> lk(s->m);
    auto it = s->need.find(key);
    if (it != s->need.end())
      need = it->second;
  }
  if (!need) { // planning a configuration costs host time: once per key
    tile_stream_memory_info info{};
    if (chucky::estimate_stream(config, &info, s->engine != nullptr))
      return nullptr;
    need = info.device_bytes;
    std::lock_guard<std::mutex> lk(s->m);
    s->need[key] = need;
  }
  if (need > s->cfg.hbm_budget_bytes)
    return nullptr;
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  std::unique_lock<std::mutex> lk(s->m);
  for (;;) {
    if (s->open < s->cfg.max_streams) {
      // an idle stream of this configuration
      auto it = std::find_if(s->idle.begin(), s->idle.end(),
                             [&](const Idle& i) { return i.key == key; });
      if (it != s->idle.end()) {
        Idle got = *it;
        s->idle.erase(it);
        s->open++;
        s->reused++;
        s->peak_open = std::max<uint64_t>(s->peak_open, s->open);
        lk.unlock();
        if (tile_stream_gpu_restart(got.s, sink) == 0) {
          tile_stream_gpu_set_batch_deadline(got.s, s->cfg.batch_deadline_ms);
          auto* r = new chucky_request{ s, got.s, got.bytes, key };
          return r;
        }
        tile_stream_gpu_destroy(got.s);
        lk.lock();
        s->resident -= got.bytes;
        s->open--;
        s->cv.notify_all();
        continue;
      }
      // room for a new one, releasing idle streams of other configurations
      std::vector<Idle> victims;
      uint64_t freed = 0;
      for (auto v = s->idle.begin();
           v != s->idle.end() && s->resident - freed + need > s->cfg.hbm_budget_bytes;) {
        freed += v->bytes;
        victims.push_back(*v);
        v = s->idle.erase(v);
      }
      s->resident -= freed;
      s->evicted += victims.size();
      if (s->resident + need <= s->cfg.hbm_budget_bytes) {
        s->resident += need;
        s->open++;
        s->created++;
        s->peak_open = std::max<uint64_t>(s->peak_open, s->open);
        s->peak_resident = std::max(s->peak_resident, s->resident);
        lk.unlock();
        for (Idle& v : victims)
          tile_stream_gpu_destroy(v.s);
        tile_stream_gpu* st = chucky::create_stream(config, sink, s->engine.get());
        if (!st) {
          lk.lock();
          s->resident -= need;
          s->open--;
          s->cv.notify_all();
          return nullptr;
        }
        tile_stream_gpu_set_batch_deadline(st, s->cfg.batch_deadline_ms);
        return new chucky_request{ s, st, need, key };
      }
      if (!victims.empty()) {
        lk.unlock();
        for (Idle& v : victims)
          tile_stream_gpu_destroy(v.s);
        lk.lock();
        continue;
      }
    }
    if (timeout_ms < 0)
      s->cv.wait(lk);
    else if (s->cv.wait_until(lk, deadline) == std::cv_status::timeout)
      return nullptr;
  }
}

extern "C" size_t
chucky_server_prewarm(chucky_server* s,
                      const tile_stream_configuration* const* configs,
                      size_t n,
                      shard_sink* sink)
{
  if (!s || !sink || (!configs && n))
    return 0;
  cudaSetDevice(s->device);
  size_t made = 0;
  for (size_t i = 0; i < n; ++i) {
    const tile_stream_configuration* c = configs[i];
    if (!c)
      continue;
    const std::string key = config_key(c);
    uint64_t need = 0;
    {
      std::lock_guard<std::mutex> lk(s->m);
      auto it = s->need.find(key);
      if (it != s->need.end())
        need = it->second;
    }
    if (!need) {
      tile_stream_memory_info info{};
      if (chucky::estimate_stream(c, &info, s->engine != nullptr))
        continue;
      need = info.device_bytes;
      std::lock_guard<std::mutex> lk(s->m);
      s->need[key] = need;
    }
    {
      std::lock_guard<std::mutex> lk(s->m);
      if (s->resident + need > s->cfg.hbm_budget_bytes)
        continue;
      s->resident += need;
    }
    tile_stream_gpu* st = chucky::create_stream(c, sink, s->engine.get());
    std::lock_guard<std::mutex> lk(s->m);
    if (!st) {
      s->resident -= need;
      continue;
    }
    s->idle.push_back(Idle{ st, need, key });
    s->peak_resident = std::max(s->peak_resident, s->resident);
    ++made;
  }
  return made;
}

extern "C" writer*
chucky_request_writer(chucky_request* r)
{
  return r ? tile_stream_gpu_writer(r->s) : nullptr;
}

extern "C" int
chucky_request_close(chucky_request* r)
{
  if (!r)
    return 1;
  chucky_server* s = r->srv;
  cudaSetDevice(s->device);
  const bool flushed = r->s->impl.flushed != 0;
  std::vector<double> lat(tile_stream_gpu_latencies(r->s, nullptr, 0));
  tile_stream_gpu_latencies(r->s, lat.data(), lat.size());
  tile_stream_gpu_clear_latencies(r->s);
  const uint64_t in = tile_stream_gpu_cursor(r->s) * r->s->impl.P.bpe;
  if (!flushed) {
    tile_stream_gpu_destroy(r->s);
  }
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->open--;
    s->requests++;
    s->input_bytes += in;
    s->lat_ms.insert(s->lat_ms.end(), lat.begin(), lat.end());
    if (flushed)
      s->idle.push_back(Idle{ r->s, r->bytes, r->key });
    else
      s->resident -= r->bytes;
  }
  s->cv.notify_all();
  delete r;
  return flushed ? 0 : 1;
}

extern "C" void
chucky_server_get_stats(chucky_server* s, chucky_server_stats* out)
{
  if (!s || !out)
    return;
  std::memset(out, 0, sizeof(*out));
  std::vector<double> lat;
  {
    std::lock_guard<std::mutex> lk(s->m);
    lat = s->lat_ms;
    out->requests = s->requests;
    out->input_bytes = s->input_bytes;
    out->streams_created = s->created;
    out->streams_reused = s->reused;
    out->streams_evicted = s->evicted;
    out->peak_resident_bytes = s->peak_resident;
    out->peak_open = s->peak_open;
  }
  out->epochs = lat.size();
  if (!lat.empty()) {
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) {
      const double x = q * double(lat.size() - 1);
      const size_t i = size_t(x);
      const double f = x - double(i);
      return i + 1 < lat.size() ? lat[i] * (1 - f) + lat[i + 1] * f : lat[i];
    };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = lat.back();
  }
  if (s->engine) {
    const chucky::EngineStats e = s->engine->stats();
    out->engine_rounds = e.rounds;
    out->engine_jobs = e.jobs;
    out->engine_launch_sets = e.launch_sets;
    out->engine_max_jobs_per_round = e.max_jobs_per_round;
  }
}

extern "C" void
chucky_server_reset_stats(chucky_server* s)
{
  if (!s)
    return;
  std::lock_guard<std::mutex> lk(s->m);
  s->lat_ms.clear();
  s->requests = s->input_bytes = 0;
  s->created = s->reused = s->evicted = 0;
  s->peak_resident = s->resident;
  s->peak_open = uint64_t(s->open);
}

extern "C" int
chucky_server_replay(chucky_server* s,
                     const chucky_replay_request* reqs,
                     size_t n,
                     double* wall_s)
{
  if (!s || (!reqs && n))
    return 1;
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i)
    order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return reqs[a].arrival_s < reqs[b].arrival_s;
  });
  std::vector<std::thread> workers;
  std::vector<int> rc(n, 0);
  const double t0 = now_s();
  const int device = s->device;
  // admission in arrival order; one worker thread per admitted request
  for (size_t k = 0; k < n; ++k) {
    const size_t i = order[k];
    const chucky_replay_request& q = reqs[i];
    const double wait = q.arrival_s - (now_s() - t0);
    if (wait > 0)
      std::this_thread::sleep_for(std::chrono::duration<double>(wait));
    chucky_request* r = chucky_server_open(s, q.config, q.sink, -1);
    if (!r) {
      rc[i] = 1;
      continue;
    }
    workers.emplace_back([&, i, r, device] {
      cudaSetDevice(device);
      const chucky_replay_request& Q = reqs[i];
      std::mt19937_64 rng(Q.seed);
      std::exponential_distribution<double> gap(Q.mean_gap_s > 0 ? 1.0 / Q.mean_gap_s : 1.0);
      writer* w = chucky_request_writer(r);
      const uint8_t* p = static_cast<const uint8_t*>(Q.data);
      const uint8_t* end = p + Q.bytes;
      const size_t step = Q.append_bytes ? Q.append_bytes : Q.bytes;
      // device-resident input goes in stream order with a stream of this
      // request (tile_stream_gpu_append_device): no host wait per append
      cudaPointerAttributes pa{};
      cudaStream_t producer = nullptr;
      if (cudaPointerGetAttributes(&pa, p) == cudaSuccess &&
          (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged))
        cudaStreamCreateWithFlags(&producer, cudaStreamNonBlocking);
      cudaGetLastError();
      int err = 0;
      while (p < end && !err) {
        if (Q.mean_gap_s > 0)
          std::this_thread::sleep_for(std::chrono::duration<double>(gap(rng)));
        const uint8_t* e = std::min(end, p + step);
        const writer_result res =
          producer ? tile_stream_gpu_append_device(r->s, slice{ p, e }, producer)
                   : writer_append(w, slice{ p, e });
        if (res.error)
          err = 1;
        p = e;
      }
      if (producer) {
        cudaStreamSynchronize(producer);
        cudaStreamDestroy(producer);
      }
      if (!err && writer_flush(w).error)
        err = 1;
      if (chucky_request_close(r))
        err = 1;
      rc[i] = err;
    });
  }
  for (std::thread& t : workers)
    t.join();
  if (wall_s)
    *wall_s = now_s() - t0;
  for (int x : rc)
    if (x)
      return 1;
  return 0;
}
