// Host-only parts of the C ABI: dimension helpers, writer helpers, codec
// predicates, crc32c, memory estimate and chunk-size advice.
#include "kernels_codec.hpp"
#include "plan.hpp"
#include "stream.gpu.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <thread>

// ---- dimension helpers (replace src/dimension.c of the reference) ---------

namespace {

const char* one_letter_name(unsigned char c)
{
  // stable storage for single-character names
  static char table[128][2];
  static bool init = false;
  if (!init) {
    for (int i = 0; i < 128; ++i) {
      table[i][0] = char(i);
      table[i][1] = 0;
    }
    init = true;
  }
  const bool ok = (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') ||
                  (c >= '0' && c <= '9');
  return ok ? table[c] : nullptr;
}

inline uint64_t div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

} // namespace

extern "C" uint8_t
dims_create(dimension* dims, const char* names, const uint64_t* sizes)
{
  if (!dims || !names || !sizes)
    return 0;
  const size_t len = std::strlen(names);
  if (len == 0 || len > HALF_MAX_RANK)
    return 0;
  for (size_t i = 0; i < len; ++i) {
    const char* nm = one_letter_name((unsigned char)names[i]);
    if (!nm)
      return 0;
    dims[i] = dimension{};
    dims[i].size = sizes[i];
    dims[i].chunk_size = sizes[i];
    dims[i].name = nm;
    dims[i].storage_position = uint8_t(i);
    dims[i].ngff.scale = 1.0;
    dims[i].ngff.type = dimension_axis_space;
  }
  return uint8_t(len);
}

extern "C" uint8_t
dims_n_append(const dimension* dims, uint8_t rank)
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

extern "C" int
dims_set_storage_order(dimension* dims, uint8_t rank, const char* order)
{
  if (!order) {
    for (uint8_t i = 0; i < rank; ++i)
      dims[i].storage_position = i;
    return 0;
  }
  if (std::strlen(order) != rank)
    return 1;
  const uint8_t na = dims_n_append(dims, rank);
  for (uint8_t d = 0; d < na; ++d)
    if (!dims[d].name || order[d] != dims[d].name[0])
      return 1;
  for (uint8_t i = 0; i < rank; ++i) {
    bool found = false;
    for (uint8_t j = 0; j < rank && !found; ++j)
      if (dims[j].name && dims[j].name[0] == order[i]) {
        dims[j].storage_position = i;
        found = true;
      }
    if (!found)
      return 1;
  }
  return 0;
}

extern "C" void
dims_set_downsample_by_name(dimension* dims, uint8_t rank, const char* names)
{
  for (uint8_t i = 0; i < rank; ++i)
    dims[i].downsample =
      (names && dims[i].name && std::strchr(names, dims[i].name[0])) ? 1 : 0;
}

extern "C" void
dims_set_chunk_sizes(dimension* dims, uint8_t rank, const uint64_t* chunk_sizes)
{
  for (uint8_t i = 0; i < rank; ++i)
    dims[i].chunk_size = chunk_sizes[i];
}

extern "C" void
dims_budget_chunk_size(dimension* dims,
                       uint8_t rank,
                       uint64_t nelem,
                       const uint8_t* ratios)
{
  // floor(log2(nelem)) bits handed out one at a time to the dim with the
  // smallest bits/ratio (ties to the higher index), as
  // src/dimension.c:109-146 of the reference.
  if (nelem == 0)
    return;
  int total_bits = 63 - __builtin_clzll(nelem);
  uint32_t sum = 0;
  for (uint8_t i = 0; i < rank; ++i)
    sum += ratios[i];
  if (sum == 0)
    return;
  int bits[HALF_MAX_RANK] = {};
  for (int b = 0; b < total_bits; ++b) {
    int best = -1;
    for (uint8_t i = 0; i < rank; ++i) {
      if (!ratios[i])
        continue;
      if (best < 0 || bits[i] * ratios[best] <= bits[best] * ratios[i])
        best = i;
    }
    bits[best]++;
  }
  for (uint8_t i = 0; i < rank; ++i)
    dims[i].chunk_size = uint64_t(1) << bits[i];
}

extern "C" void
dims_budget_chunk_bytes(dimension* dims,
                        uint8_t rank,
                        size_t target_chunk_bytes,
                        size_t bytes_per_element,
                        const uint8_t* ratios)
{
  if (bytes_per_element == 0 || target_chunk_bytes < bytes_per_element)
    return;
  dims_budget_chunk_size(dims, rank, target_chunk_bytes / bytes_per_element,
                         ratios);
}

extern "C" void
dims_set_shard_counts(dimension* dims, uint8_t rank, const uint64_t* counts)
{
  for (uint8_t i = 0; i < rank; ++i) {
    if (!counts[i])
      continue;
    const uint64_t n_chunks = div_up(dims[i].size, dims[i].chunk_size);
    dims[i].chunks_per_shard = div_up(n_chunks, counts[i]);
  }
}

extern "C" int
dims_validate(const dimension* dims, uint8_t rank)
{
  if (!dims || rank == 0 || rank > HALF_MAX_RANK)
    return 1;
  for (int d = 0; d < rank; ++d)
    if (dims[d].chunk_size == 0 || (d > 0 && dims[d].size == 0))
      return 1;
  if (dims[0].size == 0 && dims[0].chunks_per_shard == 0)
    return 1;
  const uint8_t na = dims_n_append(dims, rank);
  uint64_t seen = 0;
  for (int d = 0; d < rank; ++d) {
    const uint8_t p = dims[d].storage_position;
    if (p >= rank || (seen >> p & 1) || (d < na && p != d))
      return 1;
    seen |= uint64_t(1) << p;
  }
  return 0;
}

extern "C" void
dims_print(const dimension* dims, uint8_t rank)
{
  std::fprintf(stderr, "dim  name  %10s  %10s  %8s  %6s  %8s  storage  ds\n",
               "size", "chunk", "chunks", "cps", "shards");
  const uint8_t na = dims_n_append(dims, rank);
  uint64_t chunk_elements = 1, chunks_per_epoch = 1;
  for (uint8_t i = 0; i < rank; ++i) {
    const uint64_t tc = div_up(dims[i].size, dims[i].chunk_size);
    const uint64_t cps = dims[i].chunks_per_shard ? dims[i].chunks_per_shard : tc;
    std::fprintf(stderr, "%3d  %-4s  %10llu  %10llu  %8llu  %6llu  %8llu  %7d  %s\n",
                 i, dims[i].name ? dims[i].name : "?",
                 (unsigned long long)dims[i].size,
                 (unsigned long long)dims[i].chunk_size,
                 (unsigned long long)tc, (unsigned long long)cps,
                 (unsigned long long)(cps ? div_up(tc, cps) : 0),
                 int(dims[i].storage_position), dims[i].downsample ? "Y" : ".");
    chunk_elements *= dims[i].chunk_size;
    if (i >= na)
      chunks_per_epoch *= tc;
  }
  std::fprintf(stderr, "chunk_elements: %llu  chunks/epoch: %llu\n",
               (unsigned long long)chunk_elements,
               (unsigned long long)chunks_per_epoch);
}

// ---- writer helpers (replace src/writer.c) --------------------------------

extern "C" writer_result
writer_ok(void)
{
  return writer_result{ 0, { nullptr, nullptr } };
}

extern "C" writer_result
writer_error(void)
{
  return writer_result{ writer_error_fail, { nullptr, nullptr } };
}

extern "C" writer_result
writer_error_at(const void* beg, const void* end)
{
  return writer_result{ writer_error_fail, { beg, end } };
}

extern "C" writer_result
writer_finished_at(const void* beg, const void* end)
{
  return writer_result{ writer_error_finished, { beg, end } };
}

extern "C" writer_result
writer_append(writer* w, slice data)
{
  return w->append(w, data);
}

extern "C" writer_result
writer_flush(writer* w)
{
  return w->flush(w);
}

extern "C" writer_result
writer_append_wait(writer* w, slice data)
{
  int stalls = 0;
  while (data.beg < data.end) {
    const writer_result r = writer_append(w, data);
    if (r.error)
      return r;
    if (r.rest.beg == data.beg) {
      if (++stalls >= 10) {
        std::fprintf(stderr, "writer_append_wait: no progress after %d tries\n",
                     stalls);
        return writer_error_at(data.beg, data.end);
      }
      std::this_thread::sleep_for(
        std::chrono::milliseconds(1 << (stalls < 6 ? stalls : 6)));
    } else {
      stalls = 0;
    }
    data = r.rest;
  }
  return writer_ok();
}

// ---- codecs ----------------------------------------------------------------

extern "C" int
codec_is_blosc(enum compression_codec c)
{
  return c == CODEC_BLOSC_LZ4 || c == CODEC_BLOSC_ZSTD;
}

extern "C" int
codec_is_gpu_supported(enum compression_codec c)
{
  return c == CODEC_NONE || c == CODEC_LZ4_NON_STANDARD || c == CODEC_ZSTD;
}

// ---- crc32c (Castagnoli, reflected polynomial 0x82F63B78) -----------------

namespace chucky {

uint32_t crc32c_host(const void* data, size_t len)
{
  static uint32_t table[8][256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k)
        c = (c >> 1) ^ (0x82F63B78u & (0u - (c & 1)));
      table[0][i] = c;
    }
    for (int t = 1; t < 8; ++t)
      for (uint32_t i = 0; i < 256; ++i)
        table[t][i] = (table[t - 1][i] >> 8) ^ table[0][table[t - 1][i] & 0xFF];
    init = true;
  }
  const uint8_t* p = static_cast<const uint8_t*>(data);
  uint32_t c = 0xFFFFFFFFu;
  while (len >= 8) { // slicing-by-8
    uint32_t lo, hi;
    std::memcpy(&lo, p, 4);
    std::memcpy(&hi, p + 4, 4);
    lo ^= c;
    c = table[7][lo & 0xFF] ^ table[6][(lo >> 8) & 0xFF] ^
        table[5][(lo >> 16) & 0xFF] ^ table[4][lo >> 24] ^
        table[3][hi & 0xFF] ^ table[2][(hi >> 8) & 0xFF] ^
        table[1][(hi >> 16) & 0xFF] ^ table[0][hi >> 24];
    p += 8;
    len -= 8;
  }
  while (len--)
    c = table[0][(c ^ *p++) & 0xFF] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

} // namespace chucky

extern "C" uint32_t
chucky_crc32c(const void* data, size_t len)
{
  return chucky::crc32c_host(data, len);
}

// ---- memory estimate / chunk advice (replace src/gpu/stream.init.c:321-488)

namespace chucky {

// `shared_encoder`: the stream encodes through a server's engine and holds
// no encoder scratch of its own.
int estimate_stream(const tile_stream_configuration* config,
                    tile_stream_memory_info* info,
                    bool shared_encoder)
{
  if (!info)
    return 1;
  std::memset(info, 0, sizeof(*info));
  chucky::StreamPlan P;
  if (chucky::plan_stream(config, &P))
    return 1;
  const uint64_t K = P.K;
  info->staging_bytes = 2 * (P.epoch_bytes + 512);
  // two halves with a codec (LOD fills one while the encoders read the other)
  info->chunk_pool_bytes =
    K * P.slot_bytes * (config->codec.id == CODEC_NONE ? 1 : 2);
  const uint64_t nchunks = K * P.total_chunks;
  info->compressed_pool_bytes =
    config->codec.id == CODEC_NONE ? 0
                                   : 2 * nchunks * ((P.max_out + 15) / 16 * 16);
  uint64_t agg_host = 0, agg_dev = 0, shard = 0;
  for (int l = 0; l < P.nlod; ++l) {
    const chucky::LevelPlan& V = P.lv[l];
    const uint64_t cap = V.batch_active ? V.batch_active : 1;
    const uint64_t M = V.layout.chunks_per_epoch;
    const uint64_t pos = cap * V.covering;
    const uint64_t sa = config->shard_alignment;
    const uint64_t nsh = V.covering / V.cps_inner;
    agg_host += 2 * ((pos + 1) * 8 + pos * 8 + 8 + cap * M * P.max_out +
                     (sa ? (nsh + 1) * sa : 0) + 64);
    agg_dev += 4 * cap * M * 4 + (pos + 1) * 8;
    if (config->codec.id != CODEC_NONE) // device copy of both delivery slots
      agg_dev += 2 * (cap * M * P.max_out + (sa ? (nsh + 1) * sa : 0) + 64);
    shard += V.shard_inner_count * V.cps_total * 16;
  }
  info->aggregate_bytes = agg_dev;
  if (P.multiscale) {
    uint64_t values = 0;
    for (int l = 0; l < P.nlod; ++l)
      values += P.fixed_count * P.lv[l].lod_nelem;
    // dim-0 accumulators (levels >= 1), per-slice offsets; the general path
    // adds Morton-ordered level buffers, window ends and LUTs
    const uint64_t above0 = values - P.fixed_count * P.lv[0].lod_nelem;
    info->lod_bytes = (P.append_downsample ? above0 * P.bpe : 0) +
                      P.fixed_count * 8 * uint64_t(P.nlod + 1);
    if (!chucky::lod_plan_is_tiled(P)) {
      info->lod_bytes += values * P.bpe + P.n_ends * 8 + P.lv[0].lod_nelem * 4;
      for (int l = 0; l < P.nlod; ++l)
        info->lod_bytes += P.lv[l].lod_nelem * 4;
    }
  }
  {
    // encoder scratch of one wave (256 MiB of input per encoder launch)
    const uint64_t wave = std::max<uint64_t>(
      1, std::min<uint64_t>(nchunks, (256ull << 20) / std::max<uint64_t>(1, P.chunk_bytes)));
    uint64_t scratch = 0;
    if (config->codec.id == CODEC_ZSTD)
      scratch = chucky::zstd_scratch_bytes(wave, uint32_t(P.chunk_bytes), config->codec.level);
    else if (config->codec.id == CODEC_LZ4_NON_STANDARD)
      scratch = chucky::lz4_scratch_bytes(wave, uint32_t(P.chunk_bytes), config->codec.level);
    info->codec_bytes =
      2 * nchunks * 8 + (shared_encoder ? 0 : 2 * scratch); // one scratch per slot
  }
  info->shard_bytes = shard;
  info->device_bytes = info->staging_bytes + info->chunk_pool_bytes +
                       info->compressed_pool_bytes + info->aggregate_bytes +
                       info->lod_bytes + info->codec_bytes;
  info->host_pinned_bytes =
    agg_host + chucky::kStreamStageSlots * chucky::staging_slot_bytes(config->buffer_capacity_bytes);
  info->chunks_per_epoch = P.lv[0].layout.chunks_per_epoch;
  info->total_chunks = P.total_chunks;
  info->max_output_size = P.max_out;
  info->nlod = P.nlod;
  info->epochs_per_batch = P.K;
  return 0;
}

} // namespace chucky

extern "C" int
tile_stream_gpu_memory_estimate(const tile_stream_configuration* config,
                                tile_stream_memory_info* info)
{
  return chucky::estimate_stream(config, info, false);
}

extern "C" int
tile_stream_gpu_advise_chunk_sizes(tile_stream_configuration* config,
                                   size_t target_chunk_bytes,
                                   const uint8_t* ratios,
                                   size_t budget_bytes)
{
  const size_t bpe = dtype_bpe(config->dtype);
  if (!bpe || !budget_bytes)
    return 1;
  for (size_t t = target_chunk_bytes; t >= bpe; t >>= 1) {
    dims_budget_chunk_bytes(config->dimensions, config->rank, t, bpe, ratios);
    tile_stream_memory_info mem;
    if (tile_stream_gpu_memory_estimate(config, &mem))
      return 1;
    if (mem.device_bytes <= budget_bytes)
      return 0;
  }
  return 1;
}

// ---- launch counter ---------------------------------------------------------

namespace chucky {
static std::atomic<uint64_t> g_launches{ 0 };
void note_launches(unsigned n)
{
  g_launches += n;
}

// Streaming multiprocessors of the current device (cached per device; grid
// caps are multiples of it).
int device_sm_count()
{
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return 1;
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n > 0)
    return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      n <= 0) {
    cudaGetLastError();
    return 1;
  }
  cache[dev].store(n, std::memory_order_relaxed);
  return n;
}
} // namespace chucky

extern "C" uint64_t
chucky_launch_count(void)
{
  return chucky::g_launches.load();
}
