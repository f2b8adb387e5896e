// Zarr v3 filesystem sink (include/zarr_fs_sink.h).
//
// Shard files live at <array>/c/<i>/<j>/... and are written by one IO worker
// thread per array (pwrite jobs; O_DIRECT when `unbuffered`).  `write`
// copies the bytes into the job, `write_direct` hands the caller's buffer to
// the worker and the caller keeps it alive until the fence it records has
// retired.  Metadata: zarr.json for the root and intermediate groups and the
// array (sharding_indexed with bytes + lz4/zstd inner codecs, bytes + crc32c
// index codecs, index at the end); the multiscale sink adds OME-NGFF 0.5
// "multiscales" group metadata over arrays "0", "1", ...
// Layout, keys and JSON content follow src/zarr/zarr_fs_sink.c:17-830 and
// src/zarr/zarr_metadata.c:11-411 of the reference.
#include "zarr_fs_sink.h"

#include "defs.limits.h"

#include <atomic>
#include <cerrno>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fcntl.h>
#include <functional>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <unistd.h>
#include <vector>

namespace {

uint64_t div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

// ---- IO worker -------------------------------------------------------------

class IoQueue
{
public:
  IoQueue()
    : worker_([this] { run(); })
  {
  }
  ~IoQueue()
  {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    worker_.join();
  }
  void post(std::function<void()> job)
  {
    {
      std::lock_guard<std::mutex> g(m_);
      jobs_.push_back(std::move(job));
      ++posted_;
    }
    cv_.notify_all();
  }
  io_event record()
  {
    std::lock_guard<std::mutex> g(m_);
    return io_event{ posted_ };
  }
  void wait(io_event ev)
  {
    std::unique_lock<std::mutex> g(m_);
    done_cv_.wait(g, [&] { return done_ >= ev.seq; });
  }

private:
  void run()
  {
    for (;;) {
      std::function<void()> job;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return stop_ || !jobs_.empty(); });
        if (jobs_.empty())
          return;
        job = std::move(jobs_.front());
        jobs_.pop_front();
      }
      job();
      {
        std::lock_guard<std::mutex> g(m_);
        ++done_;
      }
      done_cv_.notify_all();
    }
  }
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  std::deque<std::function<void()>> jobs_;
  uint64_t posted_ = 0, done_ = 0;
  bool stop_ = false;
  std::thread worker_;
};

int pwrite_all(int fd, const void* buf, size_t n, uint64_t off)
{
  const char* p = static_cast<const char*>(buf);
  while (n > 0) {
    const ssize_t w = pwrite(fd, p, n, off_t(off));
    if (w < 0) {
      if (errno == EINTR)
        continue;
      return 1;
    }
    p += w;
    n -= size_t(w);
    off += uint64_t(w);
  }
  return 0;
}

int mkdirp(const std::string& path)
{
  std::string cur;
  size_t i = 0;
  while (i <= path.size()) {
    const size_t j = path.find('/', i);
    const size_t end = j == std::string::npos ? path.size() : j;
    cur = path.substr(0, end);
    if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
      return 1;
    if (j == std::string::npos)
      break;
    i = j + 1;
  }
  return 0;
}

int write_file(const std::string& path, const std::string& text)
{
  const int fd = open(path.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0)
    return 1;
  const int rc = pwrite_all(fd, text.data(), text.size(), 0);
  close(fd);
  return rc;
}

// ---- JSON ------------------------------------------------------------------

std::string jstr(const char* s)
{
  std::string o = "\"";
  for (; *s; ++s) {
    const unsigned char c = (unsigned char)*s;
    if (c == '"')
      o += "\\\"";
    else if (c == '\\')
      o += "\\\\";
    else if (c == '\n')
      o += "\\n";
    else if (c == '\r')
      o += "\\r";
    else if (c == '\t')
      o += "\\t";
    else if (c < 0x20) {
      char b[8];
      std::snprintf(b, sizeof b, "\\u%04x", c);
      o += b;
    } else
      o += char(c);
  }
  return o + "\"";
}

std::string jfloat(double v)
{
  char b[64];
  if (v == double((long long)v) && v >= -1e15 && v <= 1e15)
    std::snprintf(b, sizeof b, "%.1f", v);
  else
    std::snprintf(b, sizeof b, "%g", v);
  return b;
}

std::string root_json()
{
  return "{\"zarr_format\":3,\"node_type\":\"group\",\"consolidated_metadata\":"
         "null,\"attributes\":{}}";
}

std::string array_json(uint8_t rank,
                       const dimension* dims,
                       enum dtype dt,
                       double fill,
                       const uint64_t* cps,
                       codec_config codec)
{
  std::string s = "{\"zarr_format\":3,\"node_type\":\"array\",\"shape\":[";
  for (int d = 0; d < rank; ++d)
    s += (d ? "," : "") + std::to_string(dims[d].size);
  s += "],\"data_type\":" + jstr(dtype_zarr_string(dt));
  s += ",\"chunk_grid\":{\"name\":\"regular\",\"configuration\":{"
       "\"chunk_shape\":[";
  for (int d = 0; d < rank; ++d)
    s += (d ? "," : "") + std::to_string(dims[d].chunk_size * cps[d]);
  s += "]}},\"chunk_key_encoding\":{\"name\":\"default\",\"configuration\":{"
       "\"separator\":\"/\"}},\"codecs\":[{\"name\":\"sharding_indexed\","
       "\"configuration\":{\"chunk_shape\":[";
  for (int d = 0; d < rank; ++d)
    s += (d ? "," : "") + std::to_string(dims[d].chunk_size);
  s += "],\"codecs\":[{\"name\":\"bytes\",\"configuration\":{\"endian\":"
       "\"little\"}}";
  if (codec.id == CODEC_LZ4_NON_STANDARD)
    s += ",{\"name\":\"lz4\",\"configuration\":{}}";
  else if (codec.id == CODEC_ZSTD)
    s += ",{\"name\":\"zstd\",\"configuration\":{\"level\":" +
         std::to_string(int(codec.level)) + ",\"checksum\":false}}";
  s += "],\"index_codecs\":[{\"name\":\"bytes\",\"configuration\":{\"endian\":"
       "\"little\"}},{\"name\":\"crc32c\",\"configuration\":{}}],"
       "\"index_location\":\"end\"}}],\"fill_value\":" +
       jfloat(fill);
  bool named = false;
  for (int d = 0; d < rank; ++d)
    named |= dims[d].name != nullptr;
  if (named) {
    s += ",\"dimension_names\":[";
    for (int d = 0; d < rank; ++d)
      s += std::string(d ? "," : "") + (dims[d].name ? jstr(dims[d].name) : "null");
    s += "]";
  }
  return s + "}";
}

// shard coordinates of a flat index, dim 0 outermost and unbounded
std::string shard_key(uint8_t rank, const uint64_t* nshards, uint64_t flat)
{
  uint64_t c[MAX_ZARR_RANK];
  for (int d = rank - 1; d >= 0; --d) {
    if (d == 0)
      c[d] = flat;
    else {
      c[d] = flat % nshards[d];
      flat /= nshards[d];
    }
  }
  std::string k = "c";
  for (int d = 0; d < rank; ++d)
    k += "/" + std::to_string(c[d]);
  return k;
}

uint8_t n_append_dims(const dimension* dims, uint8_t rank)
{
  uint8_t n = 0;
  while (n < rank && dims[n].chunk_size == 1)
    ++n;
  if (n <= 1)
    return 1;
  for (uint8_t d = 0; d < n; ++d)
    if (dims[d].downsample)
      return uint8_t(d + 1);
  return n;
}

} // namespace

// ---- single-array sink -----------------------------------------------------

struct ZarrShardWriter
{
  shard_writer base;
  struct zarr_fs_sink* owner;
  int fd = -1;
};

struct zarr_fs_sink
{
  shard_sink base;
  IoQueue* queue = nullptr;
  int unbuffered = 0;
  uint8_t rank = 0;
  dimension dims[MAX_ZARR_RANK];
  uint64_t nshards[MAX_ZARR_RANK] = {};
  uint64_t cps[MAX_ZARR_RANK] = {};
  uint64_t shard_inner_count = 1;
  std::string array_dir;
  std::vector<ZarrShardWriter> writers;
  enum dtype data_type = dtype_u8;
  double fill_value = 0;
  codec_config codec{};
  std::atomic<uint64_t> retired{ 0 };
  uint64_t queued = 0;
  std::atomic<int> io_error{ 0 };
};

namespace {

constexpr size_t kPage = 4096;

int zs_write(shard_writer* self, uint64_t off, const void* b, const void* e)
{
  ZarrShardWriter* w = reinterpret_cast<ZarrShardWriter*>(self);
  zarr_fs_sink* zs = w->owner;
  const size_t n = size_t(static_cast<const char*>(e) - static_cast<const char*>(b));
  void* copy = nullptr;
  if (posix_memalign(&copy, kPage, n ? n : 1))
    return 1;
  std::memcpy(copy, b, n);
  const int fd = w->fd;
  zs->queued += n;
  zs->queue->post([zs, fd, copy, n, off] {
    if (pwrite_all(fd, copy, n, off))
      zs->io_error = 1;
    std::free(copy);
    zs->retired += n;
  });
  return 0;
}

int zs_write_direct(shard_writer* self, uint64_t off, const void* b, const void* e)
{
  ZarrShardWriter* w = reinterpret_cast<ZarrShardWriter*>(self);
  zarr_fs_sink* zs = w->owner;
  const size_t n = size_t(static_cast<const char*>(e) - static_cast<const char*>(b));
  if (!n)
    return 0;
  const int fd = w->fd;
  zs->queued += n;
  zs->queue->post([zs, fd, b, n, off] {
    if (pwrite_all(fd, b, n, off))
      zs->io_error = 1;
    zs->retired += n;
  });
  return 0;
}

int zs_finalize(shard_writer* self)
{
  ZarrShardWriter* w = reinterpret_cast<ZarrShardWriter*>(self);
  if (w->fd < 0)
    return 0;
  const int fd = w->fd;
  w->fd = -1;
  w->owner->queue->post([fd] { close(fd); });
  return w->owner->io_error.load() ? 1 : 0;
}

shard_writer* zs_open(shard_sink* self, uint8_t level, uint64_t index)
{
  (void)level;
  zarr_fs_sink* zs = reinterpret_cast<zarr_fs_sink*>(self);
  ZarrShardWriter& w = zs->writers[index % zs->shard_inner_count];
  const std::string path =
    zs->array_dir + "/" + shard_key(zs->rank, zs->nshards, index);
  int flags = O_WRONLY | O_CREAT | O_TRUNC;
#ifdef O_DIRECT
  if (zs->unbuffered)
    flags |= O_DIRECT;
#endif
  // files still being written by the worker are closed there; wait so the
  // reused writer slot never races with its previous file
  w.fd = open(path.c_str(), flags, 0644);
  if (w.fd < 0) {
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos && mkdirp(path.substr(0, slash)) == 0)
      w.fd = open(path.c_str(), flags, 0644);
  }
  if (w.fd < 0) {
    std::fprintf(stderr, "zarr_fs_sink: open(%s) failed\n", path.c_str());
    return nullptr;
  }
  return &w.base;
}

int write_array_meta(const zarr_fs_sink* zs)
{
  return write_file(zs->array_dir + "/zarr.json",
                    array_json(zs->rank, zs->dims, zs->data_type, zs->fill_value,
                               zs->cps, zs->codec));
}

int zs_update_append(shard_sink* self,
                     uint8_t level,
                     uint8_t n_append,
                     const uint64_t* sizes)
{
  (void)level;
  zarr_fs_sink* zs = reinterpret_cast<zarr_fs_sink*>(self);
  if (n_append == 0 || n_append > zs->rank)
    return 1;
  bool changed = false;
  for (uint8_t d = 0; d < n_append; ++d)
    changed |= zs->dims[d].size != sizes[d];
  if (!changed)
    return 0;
  for (uint8_t d = 0; d < n_append; ++d)
    zs->dims[d].size = sizes[d];
  return write_array_meta(zs);
}

io_event zs_record(shard_sink* self, uint8_t level)
{
  (void)level;
  return reinterpret_cast<zarr_fs_sink*>(self)->queue->record();
}

void zs_wait(shard_sink* self, uint8_t level, io_event ev)
{
  (void)level;
  reinterpret_cast<zarr_fs_sink*>(self)->queue->wait(ev);
}

// Root + intermediate groups for "a/b/c" (src/zarr/zarr_metadata.c:349-380).
int write_groups(const std::string& store, const char* array_name)
{
  if (mkdirp(store) || write_file(store + "/zarr.json", root_json()))
    return 1;
  if (!array_name)
    return 0;
  const std::string name = array_name;
  if (name.empty() || name.front() == '/' || name.back() == '/' ||
      name.find("//") != std::string::npos)
    return 1;
  for (size_t i = 0; i < name.size(); ++i)
    if (name[i] == '/') {
      const std::string dir = store + "/" + name.substr(0, i);
      if (mkdirp(dir) || write_file(dir + "/zarr.json", root_json()))
        return 1;
    }
  return 0;
}

} // namespace

extern "C" zarr_fs_sink*
zarr_fs_sink_create(const zarr_config* cfg)
{
  if (!cfg || !cfg->store_path || !cfg->dimensions || cfg->rank == 0 ||
      cfg->rank > MAX_ZARR_RANK)
    return nullptr;
  zarr_fs_sink* zs = new zarr_fs_sink();
  zs->base.open = zs_open;
  zs->base.update_append = zs_update_append;
  zs->base.record_fence = zs_record;
  zs->base.wait_fence = zs_wait;
  zs->unbuffered = cfg->unbuffered;
  zs->rank = cfg->rank;
  zs->data_type = cfg->data_type;
  zs->fill_value = cfg->fill_value;
  zs->codec = cfg->codec;
  const uint8_t na = n_append_dims(cfg->dimensions, cfg->rank);
  for (int d = 0; d < cfg->rank; ++d) {
    zs->dims[d] = cfg->dimensions[d];
    const uint64_t s = cfg->dimensions[d].size;
    const uint64_t cc = s ? div_up(s, cfg->dimensions[d].chunk_size) : 1;
    uint64_t c = cfg->dimensions[d].chunks_per_shard;
    if (!c)
      c = cc;
    if (s && cc < c)
      c = cc;
    zs->cps[d] = c;
    zs->nshards[d] = div_up(cc, c);
    if (d >= na)
      zs->shard_inner_count *= zs->nshards[d];
  }
  zs->array_dir = cfg->store_path;
  if (cfg->array_name)
    zs->array_dir += std::string("/") + cfg->array_name;
  bool ok = true;
  if (cfg->array_name)
    ok = write_groups(cfg->store_path, cfg->array_name) == 0;
  ok = ok && mkdirp(zs->array_dir) == 0;
  // pre-create shard directories of the first shard epoch (all of them
  // when dim 0 is bounded)
  uint64_t total = zs->shard_inner_count;
  for (int d = 1; d < na; ++d)
    total *= zs->nshards[d];
  if (cfg->dimensions[0].size > 0)
    total *= zs->nshards[0];
  for (uint64_t f = 0; ok && f < total; ++f) {
    const std::string key = shard_key(zs->rank, zs->nshards, f);
    ok = mkdirp(zs->array_dir + "/" + key.substr(0, key.rfind('/'))) == 0;
  }
  ok = ok && write_array_meta(zs) == 0;
  if (!ok) {
    delete zs;
    return nullptr;
  }
  zs->writers.resize(zs->shard_inner_count);
  for (auto& w : zs->writers) {
    w.base.write = zs_write;
    w.base.write_direct = zs_write_direct;
    w.base.finalize = zs_finalize;
    w.owner = zs;
  }
  zs->queue = new IoQueue();
  return zs;
}

extern "C" void
zarr_fs_sink_flush(zarr_fs_sink* s)
{
  if (s && s->queue)
    s->queue->wait(s->queue->record());
}

extern "C" size_t
zarr_fs_sink_pending_bytes(zarr_fs_sink* s)
{
  return s ? size_t(s->queued - s->retired.load()) : 0;
}

extern "C" void
zarr_fs_sink_destroy(zarr_fs_sink* s)
{
  if (!s)
    return;
  zarr_fs_sink_flush(s);
  delete s->queue;
  for (auto& w : s->writers)
    if (w.fd >= 0)
      close(w.fd);
  delete s;
}

extern "C" shard_sink*
zarr_fs_sink_as_shard_sink(zarr_fs_sink* s)
{
  return &s->base;
}

// ---- multiscale ------------------------------------------------------------

struct zarr_fs_multiscale_sink
{
  shard_sink base;
  std::vector<zarr_fs_sink*> levels;
  std::string group;
  uint8_t rank = 0;
};

namespace {

std::string multiscale_json(const zarr_fs_multiscale_sink* ms)
{
  const dimension* l0 = ms->levels[0]->dims;
  std::string s = "{\"zarr_format\":3,\"node_type\":\"group\","
                  "\"consolidated_metadata\":null,\"attributes\":{\"ome\":{"
                  "\"version\":\"0.5\",\"multiscales\":[{\"axes\":[";
  for (int d = 0; d < ms->rank; ++d) {
    std::string nm = l0[d].name ? l0[d].name : "d" + std::to_string(d);
    const char* type = "space";
    switch (l0[d].ngff.type) {
      case dimension_axis_time:
        type = "time";
        break;
      case dimension_axis_channel:
        type = "channel";
        break;
      case dimension_axis_other:
        type = "custom";
        break;
      default:
        break;
    }
    s += std::string(d ? "," : "") + "{\"name\":" + jstr(nm.c_str()) +
         ",\"type\":" + jstr(type);
    if (l0[d].ngff.unit)
      s += ",\"unit\":" + jstr(l0[d].ngff.unit);
    s += "}";
  }
  s += "],\"datasets\":[";
  for (size_t lv = 0; lv < ms->levels.size(); ++lv) {
    const dimension* ld = ms->levels[lv]->dims;
    std::string sc, tr;
    for (int d = 0; d < ms->rank; ++d) {
      const double phys = l0[d].ngff.scale > 0 ? l0[d].ngff.scale : 1.0;
      double f = 1.0;
      if (l0[d].size > 0 && ld[d].size > 0)
        f = double(l0[d].size) / double(ld[d].size);
      sc += (d ? "," : "") + jfloat(phys * f);
      tr += (d ? "," : "") + jfloat(0.5 * phys * (f - 1.0));
    }
    s += std::string(lv ? "," : "") + "{\"path\":\"" + std::to_string(lv) +
         "\",\"coordinateTransformations\":[{\"type\":\"scale\",\"scale\":[" +
         sc + "]},{\"type\":\"translation\",\"translation\":[" + tr + "]}]}";
  }
  return s + "]}]}}}";
}

shard_writer* ms_open(shard_sink* self, uint8_t level, uint64_t index)
{
  auto* ms = reinterpret_cast<zarr_fs_multiscale_sink*>(self);
  if (level >= ms->levels.size())
    return nullptr;
  return ms->levels[level]->base.open(&ms->levels[level]->base, level, index);
}

int ms_update_append(shard_sink* self,
                     uint8_t level,
                     uint8_t n_append,
                     const uint64_t* sizes)
{
  auto* ms = reinterpret_cast<zarr_fs_multiscale_sink*>(self);
  if (level >= ms->levels.size())
    return 1;
  const uint64_t old = ms->levels[level]->dims[0].size;
  if (zs_update_append(&ms->levels[level]->base, level, n_append, sizes))
    return 1;
  if (old == sizes[0])
    return 0;
  return write_file(ms->group + "/zarr.json", multiscale_json(ms));
}

io_event ms_record(shard_sink* self, uint8_t level)
{
  auto* ms = reinterpret_cast<zarr_fs_multiscale_sink*>(self);
  if (level >= ms->levels.size())
    return io_event{ 0 };
  return ms->levels[level]->queue->record();
}

void ms_wait(shard_sink* self, uint8_t level, io_event ev)
{
  auto* ms = reinterpret_cast<zarr_fs_multiscale_sink*>(self);
  if (level < ms->levels.size())
    ms->levels[level]->queue->wait(ev);
}

} // namespace

extern "C" zarr_fs_multiscale_sink*
zarr_fs_multiscale_sink_create(const zarr_multiscale_config* cfg)
{
  if (!cfg || !cfg->store_path || !cfg->dimensions || cfg->rank == 0 ||
      cfg->rank > MAX_ZARR_RANK)
    return nullptr;
  const uint8_t rank = cfg->rank;
  const dimension* dims = cfg->dimensions;
  const uint8_t na = n_append_dims(dims, rank);
  // level shapes over the whole array: inner downsampled dims halve until
  // each fits one chunk (src/lod/lod_plan.c:151-275, 296-326)
  std::vector<std::vector<uint64_t>> shapes(1, std::vector<uint64_t>(rank));
  for (int d = 0; d < rank; ++d)
    shapes[0][d] = dims[d].size ? dims[d].size : dims[d].chunk_size;
  const int max_lv = cfg->nlod > 0 ? cfg->nlod : LOD_MAX_LEVELS;
  for (;;) {
    const auto& cur = shapes.back();
    bool any = false, fits = true;
    for (int d = na; d < rank; ++d)
      if (dims[d].downsample) {
        any = true;
        fits &= div_up(cur[d], dims[d].chunk_size) <= 1;
      }
    if (!any || fits || int(shapes.size()) >= max_lv)
      break;
    std::vector<uint64_t> nx = cur;
    for (int d = na; d < rank; ++d)
      if (dims[d].downsample)
        nx[d] = (cur[d] + 1) / 2;
    shapes.push_back(nx);
  }
  zarr_fs_multiscale_sink* ms = new zarr_fs_multiscale_sink();
  ms->base.open = ms_open;
  ms->base.update_append = ms_update_append;
  ms->base.record_fence = ms_record;
  ms->base.wait_fence = ms_wait;
  ms->rank = rank;
  ms->group = cfg->store_path;
  if (cfg->array_name)
    ms->group += std::string("/") + cfg->array_name;
  bool ok = cfg->array_name ? write_groups(cfg->store_path, cfg->array_name) == 0
                            : true;
  ok = ok && mkdirp(ms->group) == 0;
  for (size_t lv = 0; ok && lv < shapes.size(); ++lv) {
    dimension ld[MAX_ZARR_RANK];
    for (int d = 0; d < rank; ++d) {
      ld[d] = dims[d];
      ld[d].size = (d == 0 && dims[0].size == 0) ? 0 : shapes[lv][d];
      const uint64_t s = shapes[lv][d];
      const uint64_t cc = s ? div_up(s, dims[d].chunk_size) : 1;
      uint64_t c = dims[d].chunks_per_shard ? dims[d].chunks_per_shard : cc;
      if (s && cc < c)
        c = cc;
      ld[d].chunks_per_shard = c;
    }
    const std::string name = std::to_string(lv);
    zarr_config zc{};
    zc.store_path = ms->group.c_str();
    zc.array_name = name.c_str();
    zc.data_type = cfg->data_type;
    zc.fill_value = cfg->fill_value;
    zc.rank = rank;
    zc.dimensions = ld;
    zc.unbuffered = cfg->unbuffered;
    zc.codec = cfg->codec;
    zarr_fs_sink* z = zarr_fs_sink_create(&zc);
    ok = z != nullptr;
    if (z)
      ms->levels.push_back(z);
  }
  ok = ok && write_file(ms->group + "/zarr.json", multiscale_json(ms)) == 0;
  if (!ok) {
    for (auto* z : ms->levels)
      zarr_fs_sink_destroy(z);
    delete ms;
    return nullptr;
  }
  return ms;
}

extern "C" void
zarr_fs_multiscale_sink_destroy(zarr_fs_multiscale_sink* s)
{
  if (!s)
    return;
  for (auto* z : s->levels)
    zarr_fs_sink_destroy(z);
  delete s;
}

extern "C" void
zarr_fs_multiscale_sink_flush(zarr_fs_multiscale_sink* s)
{
  if (s)
    for (auto* z : s->levels)
      zarr_fs_sink_flush(z);
}

extern "C" size_t
zarr_fs_multiscale_sink_pending_bytes(zarr_fs_multiscale_sink* s)
{
  size_t t = 0;
  if (s)
    for (auto* z : s->levels)
      t += zarr_fs_sink_pending_bytes(z);
  return t;
}

extern "C" shard_sink*
zarr_fs_multiscale_sink_as_shard_sink(zarr_fs_multiscale_sink* s)
{
  return &s->base;
}
