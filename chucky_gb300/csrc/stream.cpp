// GPU streaming writer: tile_stream_gpu_* (include/stream.gpu.h).
//
// One stream object owns, on the current CUDA device:
//   * two epoch input buffers (row-major, one epoch each) filled by
//     cudaMemcpyAsync on the copy stream straight from the caller's slice
//     (pinned, pageable or device memory alike);
//   * one chunk pool of K epoch slots x all levels, written by the epoch
//     kernel (transpose, or the LOD pyramid) on the compute stream;
//   * the compressed pool and sizes, written by the batch encoders;
//   * per-level shard-order LUTs (planned batch resident on the device).
// Aggregated shard bytes, offsets and sizes are written by the aggregation
// kernel directly into one of two mapped pinned host "delivery slots", so
// nothing is copied back except finished shard data.  The host delivers a
// batch to the shard sink (index + crc32c + finalize) while the GPU works on
// the next one.
//
// Control flow and contract follow the reference's GPU/CPU streams:
//   append: src/gpu/stream.c:66-170, src/cpu/stream.c:528-666
//   flush:  src/gpu/stream.c:173-245, src/cpu/stream.c:668-774
//   batch:  src/cpu/pipeline.c:113-190, src/gpu/flush.compress_agg.c:224-371
//   shards: src/zarr/shard_delivery.c:10-204
#include "plan.hpp"
#include "stream_internal.hpp"

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

namespace chucky {

namespace {

inline uint64_t round_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

#define CK(expr)                                                               \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "chucky_gb300: %s failed: %s (%s:%d)\n", #expr,     \
                   cudaGetErrorString(e_), __FILE__, __LINE__);                \
      return 1;                                                                \
    }                                                                          \
  } while (0)

stream_metric mk_metric(const char* name)
{
  stream_metric m{};
  m.name = name;
  m.best_ms = 1e30f;
  return m;
}

void add_metric(stream_metric& m, float ms, double in, double out)
{
  m.ms += ms;
  if (ms < m.best_ms)
    m.best_ms = ms;
  m.input_bytes += in;
  m.output_bytes += out;
  m.count += 1;
}

double now_ms()
{
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch())
    .count();
}

} // namespace

// ---------------------------------------------------------------------------
// setup / teardown
// ---------------------------------------------------------------------------

int Stream::timed_begin(cudaStream_t st, stream_metric* m, double in, double out)
{
  if (timers_used >= kMaxTimers)
    resolve_timers(true);
  Timer& t = timers[timers_used++];
  t.metric = m;
  t.in = in;
  t.out = out;
  CK(cudaEventRecord(t.a, st));
  return 0;
}

int Stream::timed_end(cudaStream_t st)
{
  CK(cudaEventRecord(timers[timers_used - 1].b, st));
  return 0;
}

void Stream::resolve_timers(bool wait)
{
  size_t keep = 0;
  for (size_t i = 0; i < timers_used; ++i) {
    Timer& t = timers[i];
    if (wait)
      cudaEventSynchronize(t.b);
    float ms = 0;
    if (cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
      add_metric(*t.metric, ms, t.in, t.out);
    } else { // not finished yet: keep it
      std::swap(timers[keep], timers[i]);
      ++keep;
    }
  }
  timers_used = keep;
}

int Stream::init(const tile_stream_configuration* c, shard_sink* sk)
{
  cfg = *c;
  sink = sk;
  if (plan_stream(&cfg, &P))
    return 1;
  layout = P.lv[0].layout;
  CK(cudaGetDevice(&device));
  CK(cudaStreamCreateWithFlags(&s_copy, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&s_comp, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&s_agg, cudaStreamNonBlocking));
  for (int i = 0; i < 2; ++i)
    CK(cudaStreamCreateWithFlags(&s_enc[i], cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ev_pool_ready, cudaEventDisableTiming));
  for (auto& t : timers) {
    CK(cudaEventCreate(&t.a));
    CK(cudaEventCreate(&t.b));
  }
  for (int i = 0; i < 2; ++i) {
    CK(cudaEventCreateWithFlags(&ev_input_ready[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_input_free[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_batch[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_codec_done[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_agg_done[i], cudaEventDisableTiming));
    CK(cudaEventRecord(ev_agg_done[i], s_comp));
    CK(cudaEventRecord(ev_codec_done[i], s_enc[i]));
    CK(cudaMalloc(&d_epoch[i], round_up(P.epoch_bytes, 256) + 256));
    CK(cudaEventRecord(ev_input_free[i], s_comp));
  }
  stage_bytes = staging_slot_bytes(cfg.buffer_capacity_bytes);
  // a CPU copy into the ring costs about what a direct copy's wait does at
  // a few hundred KiB: larger pinned appends are copied directly
  stage_small = std::min<uint64_t>(stage_bytes, 256u << 10);
  for (int i = 0; i < kStageSlots; ++i) {
    CK(cudaHostAlloc(&h_stage[i], stage_bytes, cudaHostAllocDefault));
    CK(cudaEventCreateWithFlags(&ev_stage[i], cudaEventDisableTiming));
  }
  for (cudaEvent_t* e : { &ev_producer, &ev_consumed })
    CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  const uint64_t half = uint64_t(P.K) * P.slot_bytes;
  pool_half_bytes = cfg.codec.id == CODEC_NONE ? 0 : half;
  const uint64_t pool_bytes = half + pool_half_bytes;
  CK(cudaMalloc(&d_pool, pool_bytes + 256)); // encoders read 8 B past a chunk
  CK(cudaMemsetAsync(d_pool, 0, pool_bytes, s_comp));
  const uint64_t nchunks = uint64_t(P.K) * P.total_chunks;
  if (cfg.codec.id == CODEC_NONE) {
    comp_stride = layout.chunk_stride * P.bpe;
    CK(cudaMalloc(&d_sizes[0], nchunks * sizeof(uint64_t)));
    d_sizes[1] = d_sizes[0]; // constant: every chunk is chunk_bytes
    CK(launch_fill_u64(d_sizes[0], P.chunk_bytes, nchunks, s_comp));
  } else {
    for (int i = 0; i < 2; ++i)
      CK(cudaMalloc(&d_sizes[i], nchunks * sizeof(uint64_t)));
    comp_stride = round_up(P.max_out, 16);
    for (int i = 0; i < 2; ++i)
      CK(cudaMalloc(&d_comp[i], nchunks * comp_stride + 64));
    if (codec_init())
      return 1;
  }
  if (setup_transpose() || setup_lod() || setup_aggregate())
    return 1;

  metrics.memcpy = mk_metric("memcpy");
  metrics.h2d = mk_metric("h2d");
  metrics.scatter = mk_metric("scatter");
  metrics.compress = mk_metric("compress");
  metrics.aggregate = mk_metric("aggregate");
  metrics.d2h = mk_metric("d2h");
  metrics.sink = mk_metric("sink");
  if (P.multiscale) {
    metrics.lod_gather = mk_metric("lod_gather");
    metrics.lod_reduce = mk_metric("lod_reduce");
    metrics.lod_append_fold = mk_metric("lod_append_fold");
    metrics.lod_morton_chunk = mk_metric("lod_morton");
  }
  max_cursor = P.max_cursor;
  CK(cudaStreamSynchronize(s_comp));
  return 0;
}

int Stream::setup_transpose()
{
  if (P.multiscale)
    return 0;
  const tile_stream_layout& L = layout;
  const int r = L.lifted_rank;
  const uint64_t cs = L.lifted_shape[r - 1];
  const uint64_t width = L.lifted_shape[r - 2] * cs;
  const uint64_t rows = L.epoch_elements / width;
  std::vector<uint64_t> row(rows), col(width);
  for (uint64_t x = 0; x < width; ++x)
    col[x] = (x / cs) * uint64_t(L.lifted_strides[r - 2]) +
             (x % cs) * uint64_t(L.lifted_strides[r - 1]);
  for (uint64_t y = 0; y < rows; ++y)
    row[y] = ravel(r - 2, L.lifted_shape, L.lifted_strides, y);
  CK(cudaMalloc(&d_row_off, rows * sizeof(uint64_t)));
  CK(cudaMalloc(&d_col_off, width * sizeof(uint64_t)));
  CK(cudaMemcpy(d_row_off, row.data(), rows * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_col_off, col.data(), width * 8, cudaMemcpyHostToDevice));
  tr.width = FastDiv(width);
  tr.row_off = d_row_off;
  tr.col_off = d_col_off;
  tr.bpe = uint32_t(P.bpe);
  tr.vector_ok = L.lifted_strides[r - 1] == 1 && (cs * P.bpe) % 16 == 0 &&
                 16 % P.bpe == 0;
  return 0;
}

// Whether the tiled single-pass kernel produces every level of this plan
// from one read of L0 (1..3 LOD dims, the pyramid inside one tile).
bool lod_plan_is_tiled(const StreamPlan& P)
{
  return P.multiscale && P.lod_ndim >= 1 && P.lod_ndim <= 3 && P.nlod <= 16 &&
         P.nlod - 1 <= lod_tile_levels(P.lod_ndim);
}

int Stream::setup_lod()
{
  if (!P.multiscale)
    return 0;
  const int nlod = P.nlod;
  lod_tiled = lod_plan_is_tiled(P);
  uint64_t total_values = 0, total_accum = 0;
  for (int l = 0; l < nlod; ++l) {
    lod_nelem[l] = P.lv[l].lod_nelem;
    level_beg[l] = total_values;
    total_values += P.fixed_count * P.lv[l].lod_nelem;
    if (l >= 1) {
      accum_beg[l] = total_accum;
      total_accum += P.fixed_count * P.lv[l].lod_nelem;
    }
    ends_beg[l] = l >= 1 ? P.lod_end[l - 1] - P.lod_end[0] : 0;
  }
  if (P.append_downsample && total_accum)
    CK(cudaMalloc(&d_accum, total_accum * P.bpe + 16));

  // row-major strides of the epoch buffer
  uint64_t stride[HALF_MAX_RANK];
  stride[P.rank - 1] = 1;
  for (int d = P.rank - 2; d >= 0; --d)
    stride[d] = stride[d + 1] * P.lv[0].shape[d + 1];
  // per slice of the fixed dims: its offset in the epoch buffer and in
  // each level's chunk slot (both paths)
  {
    std::vector<uint64_t> fixed(P.fixed_count);
    for (uint64_t b = 0; b < P.fixed_count; ++b) {
      uint64_t r = b, off = 0;
      for (int k = P.fixed_ndim - 1; k >= 0; --k) {
        off += (r % P.fixed_shape[k]) * stride[P.fixed_to_dim[k]];
        r /= P.fixed_shape[k];
      }
      fixed[b] = off;
    }
    CK(cudaMalloc(&d_gather_fixed, P.fixed_count * 8));
    CK(cudaMemcpy(d_gather_fixed, fixed.data(), P.fixed_count * 8,
                  cudaMemcpyHostToDevice));
  }
  for (int l = 0; l < nlod; ++l) {
    const tile_stream_layout& L = P.lv[l].layout;
    std::vector<uint64_t> fixed(P.fixed_count);
    for (uint64_t b = 0; b < P.fixed_count; ++b) {
      uint64_t r = b;
      int64_t off = 0;
      for (int k = P.fixed_ndim - 1; k >= 0; --k) {
        const uint64_t coord = r % P.fixed_shape[k];
        r /= P.fixed_shape[k];
        const int d = P.fixed_to_dim[k];
        const uint64_t cs = L.lifted_shape[2 * d + 1];
        off += int64_t(coord / cs) * L.lifted_strides[2 * d] +
               int64_t(coord % cs) * L.lifted_strides[2 * d + 1];
      }
      fixed[b] = uint64_t(off) + P.lv[l].chunk_offset * L.chunk_stride;
    }
    CK(cudaMalloc(&d_chunk_fixed[l], P.fixed_count * 8));
    CK(cudaMemcpy(d_chunk_fixed[l], fixed.data(), P.fixed_count * 8,
                  cudaMemcpyHostToDevice));
  }

  if (!lod_tiled) {
    // The general path: Morton-ordered level buffers, window ends and the
    // L0 gather / per-level scatter LUTs (host work and memory in
    // proportion to the pyramid's element count).
    CK(cudaMalloc(&d_values, total_values * P.bpe + 16));
    plan_build_ends(P);
    if (!P.ends.empty()) {
      CK(cudaMalloc(&d_ends, P.ends.size() * 8));
      CK(cudaMemcpy(d_ends, P.ends.data(), P.ends.size() * 8,
                    cudaMemcpyHostToDevice));
    }
    // L0 gather LUT over the row-major epoch (src/cpu/lod.cpp:181-239).
    {
      const uint64_t n0 = P.lv[0].lod_nelem;
      std::vector<uint32_t> lut(n0);
      uint64_t shp[LOD_MAX_NDIM];
      for (int k = 0; k < P.lod_ndim; ++k)
        shp[k] = P.lv[0].shape[P.lod_to_dim[k]];
      for (uint64_t g = 0; g < n0; ++g) {
        uint64_t c[LOD_MAX_NDIM], r = g, off = 0;
        for (int k = P.lod_ndim - 1; k >= 0; --k) {
          c[k] = r % shp[k];
          r /= shp[k];
          off += c[k] * stride[P.lod_to_dim[k]];
        }
        lut[morton_rank(P.lod_ndim, shp, c, 0)] = uint32_t(off);
      }
      CK(cudaMalloc(&d_gather_lut, n0 * 4));
      CK(cudaMemcpy(d_gather_lut, lut.data(), n0 * 4, cudaMemcpyHostToDevice));
    }
    // Morton -> chunk LUTs per level (src/cpu/lod.cpp:318-352,
    // src/cpu/pipeline.c:373-398).
    for (int l = 0; l < nlod; ++l) {
      const tile_stream_layout& L = P.lv[l].layout;
      const uint64_t n = P.lv[l].lod_nelem;
      std::vector<uint32_t> lut(n);
      uint64_t shp[LOD_MAX_NDIM];
      for (int k = 0; k < P.lod_ndim; ++k)
        shp[k] = P.lv[l].shape[P.lod_to_dim[k]];
      for (uint64_t g = 0; g < n; ++g) {
        uint64_t c[LOD_MAX_NDIM], r = g;
        int64_t off = 0;
        for (int k = P.lod_ndim - 1; k >= 0; --k) {
          c[k] = r % shp[k];
          r /= shp[k];
          const int d = P.lod_to_dim[k];
          const uint64_t cs = L.lifted_shape[2 * d + 1];
          off += int64_t(c[k] / cs) * L.lifted_strides[2 * d] +
                 int64_t(c[k] % cs) * L.lifted_strides[2 * d + 1];
        }
        lut[morton_rank(P.lod_ndim, shp, c, 0)] = uint32_t(off);
      }
      CK(cudaMalloc(&d_chunk_lut[l], n * 4));
      CK(cudaMemcpy(d_chunk_lut[l], lut.data(), n * 4, cudaMemcpyHostToDevice));
    }
  } else {
    LodTileArgs& t = tile;
    t.dtype = cfg.dtype;
    t.method = cfg.reduce_method;
    t.append_method = cfg.append_reduce_method;
    t.nlod = P.nlod;
    t.lod_ndim = P.lod_ndim;
    t.fixed_count = P.fixed_count;
    t.gather_fixed = d_gather_fixed;
    const uint32_t edge = lod_tile_edge(P.lod_ndim);
    for (int k = 0; k < P.lod_ndim; ++k) {
      const int d = P.lod_to_dim[k];
      t.tiles[k] = (P.lv[0].shape[d] + edge - 1) / edge;
      t.in_stride[k] = int64_t(stride[d]);
      t.cs[k] = uint32_t(cfg.dimensions[d].chunk_size);
    }
    for (int l = 0; l < nlod; ++l) {
      const tile_stream_layout& L = P.lv[l].layout;
      LodTileArgs::Level& V = t.lv[l];
      V.nelem = P.lv[l].lod_nelem;
      V.accum_off = accum_beg[l];
      V.chunk_fixed = d_chunk_fixed[l];
      V.off32 = uint64_t(L.chunk_stride) <= 0xFFFFFFFFull ? 1u : 0u;
      for (int k = 0; k < P.lod_ndim; ++k) {
        const int d = P.lod_to_dim[k];
        V.shape[k] = P.lv[l].shape[d];
        V.S[k] = uint64_t(L.lifted_strides[2 * d]);
        V.s[k] = uint64_t(L.lifted_strides[2 * d + 1]);
      }
    }
  }
  lod.dtype = cfg.dtype;
  lod.reduce_method = cfg.reduce_method;
  lod.append_method = cfg.append_reduce_method;
  lod.nlod = nlod;
  lod.fixed_count = P.fixed_count;
  lod.lod_nelem = lod_nelem;
  lod.level_beg = level_beg;
  lod.accum_beg = accum_beg;
  lod.d_ends = d_ends;
  lod.ends_beg = ends_beg;
  lod.d_gather_lut = d_gather_lut;
  lod.d_gather_fixed = d_gather_fixed;
  lod.d_chunk_lut = d_chunk_lut;
  lod.d_chunk_fixed = d_chunk_fixed;
  return 0;
}

// Shard-order LUTs of `n_active` epochs of level l read from pool epochs
// `eps` (src/stream/types.aggregate.c:28-62).
void Stream::build_luts(int l,
                        uint32_t n_active,
                        const uint32_t* eps,
                        uint32_t* gather,
                        uint32_t* perm) const
{
  const LevelPlan& V = P.lv[l];
  const uint64_t M = V.layout.chunks_per_epoch, cpi = V.cps_inner;
  const uint64_t nsh = V.covering / cpi;
  for (uint32_t a = 0; a < n_active; ++a)
    for (uint64_t j = 0; j < M; ++j) {
      const uint64_t i = uint64_t(a) * M + j;
      gather[i] = uint32_t(eps[a] * P.total_chunks + V.chunk_offset + j);
      const uint64_t pos = ravel(V.agg_rank, V.agg_shape, V.agg_strides, j);
      perm[i] = uint32_t(((pos / cpi) % nsh) * n_active * cpi + pos % cpi +
                         a * cpi);
    }
}

int Stream::setup_aggregate()
{
  uint64_t max_positions = 0;
  for (int l = 0; l < P.nlod; ++l) {
    const LevelPlan& V = P.lv[l];
    const uint32_t slots = std::max<uint32_t>(V.batch_active, 1);
    // the drain batch of a level may exceed its planned count only when
    // planned is 0, so max(planned, 1) epochs bound every batch
    const uint32_t cap_epochs = std::max<uint32_t>(slots, 1);
    const uint64_t M = V.layout.chunks_per_epoch;
    const uint64_t lut_n = uint64_t(cap_epochs) * M;
    lut_cap[l] = cap_epochs;
    CK(cudaMalloc(&d_gather[l], lut_n * 4));
    CK(cudaMalloc(&d_perm[l], lut_n * 4));
    for (int si = 0; si < 2; ++si) {
      CK(cudaHostAlloc(&h_lut_stage[si][l], 2 * lut_n * 4, cudaHostAllocMapped));
      CK(cudaMalloc(&d_gather_tmp[si][l], lut_n * 4));
      CK(cudaMalloc(&d_perm_tmp[si][l], lut_n * 4));
    }
    planned_count[l] = V.batch_active;
    if (V.batch_active) {
      std::vector<uint32_t> eps(V.batch_active), g(lut_n), pm(lut_n);
      for (uint32_t a = 0; a < V.batch_active; ++a)
        eps[a] = (a + 1) * V.period - 1;
      build_luts(l, V.batch_active, eps.data(), g.data(), pm.data());
      CK(cudaMemcpy(d_gather[l], g.data(), lut_n * 4, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(d_perm[l], pm.data(), lut_n * 4, cudaMemcpyHostToDevice));
    }
    const uint64_t positions = uint64_t(cap_epochs) * V.covering;
    max_positions = std::max(max_positions, positions);
    const uint64_t nshards = V.covering / V.cps_inner;
    const uint64_t sa = cfg.shard_alignment;
    const uint64_t data = uint64_t(cap_epochs) * M * P.max_out +
                          (sa ? (nshards + 1) * sa : 0) + 64;
    for (int s = 0; s < 2; ++s) {
      DeliverySlot::Level& D = slot[s].lv[l];
      D.positions_cap = positions;
      D.data_cap = data;
      CK(cudaHostAlloc(&D.offsets, (positions + 1) * 8, cudaHostAllocMapped));
      CK(cudaHostAlloc(&D.real_sizes, positions * 8 + 8, cudaHostAllocMapped));
      CK(cudaHostAlloc(&D.data, data, cudaHostAllocMapped));
      // compressed batches are gathered in device memory and copied to the
      // host by the copy engine (faster than SM stores over the link)
      if (cfg.codec.id != CODEC_NONE)
        CK(cudaMalloc(&D.d_data, data));
    }
    // shard state (src/zarr/shard_delivery.c:10-34); the index lives on
    // the device
    Shards& S = shards[l];
    S.sh.resize(V.shard_inner_count);
    const uint64_t nidx = V.cps_total * 16, itotal = nidx + 4;
    blob_bytes[l] = sa ? round_up(itotal, sa) : itotal;
    CK(cudaMalloc(&d_index[l], V.shard_inner_count * nidx));
    CK(cudaMemset(d_index[l], 0xFF, V.shard_inner_count * nidx));
    CK(cudaMalloc(&d_cursor[l], V.shard_inner_count * 8));
    CK(cudaMemset(d_cursor[l], 0, V.shard_inner_count * 8));
    CK(cudaHostAlloc(&h_flush_blobs[l], V.shard_inner_count * blob_bytes[l],
                     cudaHostAllocMapped));
    const uint32_t finals = cap_epochs / uint32_t(std::max<uint64_t>(1, V.cps_append)) + 2;
    for (int si = 0; si < 2; ++si) {
      DeliverySlot::Level& D = slot[si].lv[l];
      D.runs_cap = cap_epochs + 2;
      D.finals_cap = finals;
      CK(cudaHostAlloc(&D.runs, D.runs_cap * sizeof(IndexRun), cudaHostAllocMapped));
      CK(cudaHostAlloc(&D.blobs, finals * V.shard_inner_count * blob_bytes[l],
                       cudaHostAllocMapped));
    }
  }
  agg_scratch_slot = (max_positions + 1) * size_t(P.nlod);
  CK(cudaMalloc(&d_agg_scratch, 2 * agg_scratch_slot * 8));
  return 0;
}

void Stream::release()
{
  if (s_comp)
    cudaStreamSynchronize(s_comp);
  for (cudaStream_t e : s_enc)
    if (e)
      cudaStreamSynchronize(e);
  if (s_agg)
    cudaStreamSynchronize(s_agg);
  if (s_copy)
    cudaStreamSynchronize(s_copy);
  codec_release();
  for (int i = 0; i < kStageSlots; ++i) {
    cudaFreeHost(h_stage[i]);
    h_stage[i] = nullptr;
    if (ev_stage[i])
      cudaEventDestroy(ev_stage[i]);
    ev_stage[i] = nullptr;
  }
  for (cudaEvent_t* e : { &ev_producer, &ev_consumed })
    if (*e) {
      cudaEventDestroy(*e);
      *e = nullptr;
    }
  for (int i = 0; i < 2; ++i) {
    cudaFree(d_epoch[i]);
    if (ev_input_ready[i])
      cudaEventDestroy(ev_input_ready[i]);
    if (ev_input_free[i])
      cudaEventDestroy(ev_input_free[i]);
    if (ev_batch[i])
      cudaEventDestroy(ev_batch[i]);
    for (int l = 0; l < LOD_MAX_LEVELS; ++l) {
      cudaFreeHost(slot[i].lv[l].runs);
      cudaFreeHost(slot[i].lv[l].blobs);
      cudaFreeHost(slot[i].lv[l].offsets);
      cudaFreeHost(slot[i].lv[l].real_sizes);
      cudaFreeHost(slot[i].lv[l].data);
      cudaFree(slot[i].lv[l].d_data);
    }
  }
  for (auto& t : timers) {
    if (t.a)
      cudaEventDestroy(t.a);
    if (t.b)
      cudaEventDestroy(t.b);
  }
  cudaFree(d_pool);
  for (int i = 0; i < 2; ++i) {
    cudaFree(d_comp[i]);
    if (ev_codec_done[i])
      cudaEventDestroy(ev_codec_done[i]);
    if (ev_agg_done[i])
      cudaEventDestroy(ev_agg_done[i]);
  }
  if (s_agg)
    cudaStreamDestroy(s_agg);
  for (cudaStream_t e : s_enc)
    if (e)
      cudaStreamDestroy(e);
  if (ev_pool_ready)
    cudaEventDestroy(ev_pool_ready);
  if (d_sizes[1] != d_sizes[0])
    cudaFree(d_sizes[1]);
  cudaFree(d_sizes[0]);
  cudaFree(d_row_off);
  cudaFree(d_col_off);
  cudaFree(d_values);
  cudaFree(d_accum);
  cudaFree(d_ends);
  cudaFree(d_gather_lut);
  cudaFree(d_gather_fixed);
  cudaFree(d_agg_scratch);
  for (int l = 0; l < LOD_MAX_LEVELS; ++l) {
    cudaFree(d_index[l]);
    cudaFree(d_cursor[l]);
    cudaFreeHost(h_flush_blobs[l]);
    d_index[l] = d_cursor[l] = nullptr;
    h_flush_blobs[l] = nullptr;
    cudaFree(d_chunk_lut[l]);
    cudaFree(d_chunk_fixed[l]);
    cudaFree(d_gather[l]);
    cudaFree(d_perm[l]);
    for (int si = 0; si < 2; ++si) {
      cudaFree(d_gather_tmp[si][l]);
      cudaFree(d_perm_tmp[si][l]);
      cudaFreeHost(h_lut_stage[si][l]);
      d_gather_tmp[si][l] = d_perm_tmp[si][l] = nullptr;
      h_lut_stage[si][l] = nullptr;
      lut_eps[si][l].clear();
    }
  }
  if (s_copy)
    cudaStreamDestroy(s_copy);
  if (s_comp)
    cudaStreamDestroy(s_comp);
}

// ---------------------------------------------------------------------------
// epochs
// ---------------------------------------------------------------------------

uint8_t* Stream::pool_slot(uint32_t e) const
{
  return d_pool + next_slot * pool_half_bytes + uint64_t(e) * P.slot_bytes;
}

// Before the first write of a batch into its pool half: the encoders of the
// batch that last used that half must be done reading it.
int Stream::claim_pool()
{
  if (pool_half_bytes && !pool_claimed) {
    CK(cudaStreamWaitEvent(s_comp, ev_codec_done[next_slot], 0));
    pool_claimed = true;
  }
  return 0;
}

int Stream::run_epoch(uint64_t present)
{
  const int b = in_buf;
  if (stage_issue())
    return 1;
  CK(cudaEventRecord(ev_input_ready[b], s_copy));
  CK(cudaStreamWaitEvent(s_comp, ev_input_ready[b], 0));
  if (present < layout.epoch_elements) // partial final epoch: fill value 0
    CK(cudaMemsetAsync(d_epoch[b] + present * P.bpe, 0,
                       (layout.epoch_elements - present) * P.bpe, s_comp));
  if (claim_pool())
    return 1;
  uint8_t* slot_ptr = pool_slot(accumulated);
  uint32_t mask = 1;
  if (!P.multiscale) {
    TransposeArgs a = tr;
    a.src = d_epoch[b];
    a.dst = slot_ptr;
    a.n = layout.epoch_elements;
    if (timed_begin(s_comp, &metrics.scatter, double(P.epoch_bytes),
                    double(P.epoch_bytes)))
      return 1;
    CK(launch_transpose(a, s_comp));
    if (timed_end(s_comp))
      return 1;
  } else if (lod_tiled) {
    const bool folding = P.append_downsample && d_accum;
    LodTileArgs t = tile;
    t.linear = d_epoch[b];
    t.slot = slot_ptr;
    t.accum = d_accum;
    t.fold_mask = 0;
    t.emit_mask = uint32_t((1ull << P.nlod) - 1);
    mask = t.emit_mask;
    if (folding) {
      t.emit_mask = 1;
      for (int l = 1; l < P.nlod; ++l) {
        t.fold_mask |= 1u << l;
        t.count[l] = counts[l];
        if (counts[l] + 1 >= (1u << l))
          t.emit_mask |= 1u << l;
      }
      mask = t.emit_mask;
    }
    if (timed_begin(s_comp, &metrics.lod_reduce, double(P.epoch_bytes),
                    double(P.slot_bytes)))
      return 1;
    CK(launch_lod_tile(t, s_comp));
    if (timed_end(s_comp))
      return 1;
    if (folding)
      for (int l = 1; l < P.nlod; ++l)
        counts[l] = (mask >> l & 1) ? 0 : counts[l] + 1;
  } else {
    const double vb = double(P.fixed_count * P.lv[0].lod_nelem * P.bpe);
    if (timed_begin(s_comp, &metrics.lod_gather, vb, vb))
      return 1;
    CK(launch_lod_gather(lod, d_epoch[b], d_values, s_comp));
    if (timed_end(s_comp))
      return 1;
    if (timed_begin(s_comp, &metrics.lod_reduce, vb, 0))
      return 1;
    CK(launch_lod_reduce(lod, d_values, s_comp));
    if (timed_end(s_comp))
      return 1;
    mask = (P.append_downsample && d_accum) ? 1u
                                             : uint32_t((1ull << P.nlod) - 1);
    if (P.append_downsample && d_accum) {
      if (timed_begin(s_comp, &metrics.lod_append_fold, 0, 0))
        return 1;
      for (int l = 1; l < P.nlod; ++l)
        CK(launch_lod_fold(lod, l, counts[l], d_values, d_accum, s_comp));
      for (int l = 1; l < P.nlod; ++l) {
        counts[l]++;
        if (counts[l] >= (1u << l)) {
          CK(launch_lod_emit(lod, l, counts[l], d_accum, d_values, s_comp));
          counts[l] = 0;
          mask |= 1u << l;
        }
      }
      if (timed_end(s_comp))
        return 1;
    }
    if (timed_begin(s_comp, &metrics.lod_morton_chunk, 0, double(P.slot_bytes)))
      return 1;
    for (int l = 0; l < P.nlod; ++l)
      if (mask >> l & 1)
        CK(launch_lod_to_chunks(lod, l, d_values, slot_ptr, s_comp));
    if (timed_end(s_comp))
      return 1;
  }
  CK(cudaEventRecord(ev_input_free[b], s_comp));
  pending_epoch_ms.push_back(now_ms());
  in_buf ^= 1;
  in_fill = 0;
  if (accumulated >= MAX_BATCH_EPOCHS)
    return 1;
  masks[accumulated++] = mask;
  return 0;
}

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------

int Stream::kick_batch(uint32_t n_epochs, const uint32_t* epoch_masks)
{
  const int si = next_slot;
  DeliverySlot& S = slot[si];
  if (S.busy && deliver(si)) // cannot happen with drain-before-kick
    return 1;
  const uint64_t nchunks = uint64_t(n_epochs) * P.total_chunks;
  const uint8_t* comp = d_pool + si * pool_half_bytes;
  const bool coded = cfg.codec.id != CODEC_NONE;
  // the aggregation's LUT uploads ride on the stream that precedes it
  const cudaStream_t se = s_enc[si];
  const cudaStream_t su = coded ? se : s_comp;
  if (coded) {
    // the encoders start once this batch's pool half is filled
    CK(cudaEventRecord(ev_pool_ready, s_comp));
    CK(cudaStreamWaitEvent(se, ev_pool_ready, 0));
    // encode only the chunks of active (epoch, level) pairs: runs of
    // consecutive slots, passed to the encoders by value; a list on the
    // device only for batches with more runs than that holds
    uint32_t* ids = h_chunk_ids[si];
    ChunkRuns runs{};
    bool fits = true;
    uint64_t n = 0;
    for (uint32_t e = 0; e < n_epochs; ++e)
      for (int l = 0; l < P.nlod; ++l)
        if (epoch_masks[e] >> l & 1) {
          const uint64_t base = uint64_t(e) * P.total_chunks + P.lv[l].chunk_offset;
          const uint64_t cnt = P.lv[l].layout.chunks_per_epoch;
          if (runs.n > 0 && runs.slot[runs.n - 1] + (n - runs.first[runs.n - 1]) == base) {
            // continues the previous run
          } else if (runs.n < uint32_t(CodecBatch::kMaxRuns)) {
            runs.first[runs.n] = uint32_t(n);
            runs.slot[runs.n] = uint32_t(base);
            ++runs.n;
          } else {
            fits = false;
          }
          for (uint64_t j = 0; j < cnt; ++j)
            ids[n++] = uint32_t(base + j);
        }
    runs.first[runs.n] = uint32_t(n);
    if (!tuned) {
      // the autotuner (when on) picks this key's encoder parameters on up
      // to 16 chunks spread over the first batch
      if (autotune_enabled() && n) {
        const uint8_t* sample[16];
        const uint32_t k = uint32_t(std::min<uint64_t>(16, n));
        const uint64_t slot_bytes = layout.chunk_stride * P.bpe;
        for (uint32_t i = 0; i < k; ++i)
          sample[i] = comp + uint64_t(ids[uint64_t(i) * n / k]) * slot_bytes;
        tune = autotune(tune_key, uint32_t(P.chunk_bytes), sample, k, ev_pool_ready);
      }
      tuned = true;
    }
    const uint32_t* d_ids = nullptr;
    const ChunkRuns* rp = nullptr;
    if (n != nchunks) {
      if (fits) {
        rp = &runs;
      } else {
        CK(launch_stage_copy(d_chunk_ids[si], ids, n, se));
        d_ids = d_chunk_ids[si];
      }
    }
    // the aggregation that read this compressed slot two batches ago must
    // be done before the encoders overwrite it
    CK(cudaStreamWaitEvent(se, ev_agg_done[si], 0));
    if (engine) {
      // the shared engine encodes this batch with other streams' batches.
      // The job goes to the engine once its chunks are in the pool, so the
      // engine's launches never wait on the device for one stream's epoch
      // kernels while other streams' chunks are ready.
      CK(cudaEventSynchronize(ev_pool_ready));
      EncodeJob& J = job[si];
      J = EncodeJob{};
      J.codec = cfg.codec.id;
      J.level = cfg.codec.level;
      J.strength = tune.strength;
      J.min_match = tune.min_match;
      J.chunk_bytes = uint32_t(P.chunk_bytes);
      J.pool = comp;
      J.in_stride = layout.chunk_stride * P.bpe;
      J.slots = ids;
      J.n = n;
      J.out = d_comp[si];
      J.out_stride = comp_stride;
      J.sizes = d_sizes[si];
      J.ready = ev_pool_ready;
      J.out_free = ev_agg_done[si];
      J.done = ev_engine_done[si];
      if (engine->run(J))
        return 1;
      CK(cudaStreamWaitEvent(se, ev_engine_done[si], 0));
    } else {
      if (timed_begin(se, &metrics.compress, double(n * P.chunk_bytes), 0))
        return 1;
      if (codec_compress(comp, n, d_ids, rp, d_comp[si], d_sizes[si], codec_state[si], se))
        return 1;
      if (timed_end(se))
        return 1;
    }
    comp = d_comp[si];
  }
  AggBatch ab{};
  ab.comp = comp;
  ab.comp_stride = comp_stride;
  ab.sizes = d_sizes[si];
  ab.alignment = cfg.shard_alignment;
  S.n_levels = 0;
  for (int l = 0; l < P.nlod; ++l) {
    uint32_t eps[MAX_BATCH_EPOCHS], na = 0;
    for (uint32_t e = 0; e < n_epochs; ++e)
      if (epoch_masks[e] >> l & 1)
        eps[na++] = e;
    S.active[l] = na;
    if (!na)
      continue;
    const LevelPlan& V = P.lv[l];
    if (na > lut_cap[l])
      return 1;
    bool planned = na == planned_count[l];
    for (uint32_t a = 0; planned && a < na; ++a)
      planned = eps[a] == (a + 1) * V.period - 1;
    const uint32_t* g = d_gather[l];
    const uint32_t* pm = d_perm[l];
    const uint64_t n = uint64_t(na) * V.layout.chunks_per_epoch;
    if (!planned) {
      // staging of this delivery slot: its previous batch has been
      // delivered, so its uploads are complete.  The tables depend only on
      // the plan and the active epochs: the same pattern as this slot's
      // last upload reuses them.
      std::vector<uint32_t>& last = lut_eps[si][l];
      if (last.size() != na || !std::equal(last.begin(), last.end(), eps)) {
        uint32_t* hg = h_lut_stage[si][l];
        uint32_t* hp = h_lut_stage[si][l] + n;
        build_luts(l, na, eps, hg, hp);
        CK(launch_stage_copy(d_gather_tmp[si][l], hg, n, su));
        CK(launch_stage_copy(d_perm_tmp[si][l], hp, n, su));
        last.assign(eps, eps + na);
      }
      g = d_gather_tmp[si][l];
      pm = d_perm_tmp[si][l];
    }
    AggLevel& A = ab.lv[ab.nlevels++];
    A.gather = g;
    A.perm = pm;
    A.n = n;
    A.positions = uint64_t(na) * V.covering;
    A.group = uint64_t(na) * V.cps_inner;
    DeliverySlot::Level& D = S.lv[l];
    A.offsets = D.offsets;
    A.real_sizes = D.real_sizes;
    A.out = D.d_data ? D.d_data : D.data;
    D.positions = A.positions;
    D.copied = 0;
    // the batch's runs of epochs per shard epoch, as delivery splits them
    // (src/zarr/shard_delivery.c:105-204)
    D.n_runs = 0;
    for (uint32_t a = 0; a < na;) {
      const uint32_t left = uint32_t(V.cps_append - kick_eis[l]);
      const uint32_t run = std::min(left, na - a);
      if (D.n_runs >= D.runs_cap)
        return 1;
      IndexRun& R = D.runs[D.n_runs++];
      R.a0 = a;
      R.run = run;
      R.eis0 = kick_eis[l];
      kick_eis[l] += run;
      R.final = kick_eis[l] >= V.cps_append ? 1u : 0u;
      if (R.final)
        kick_eis[l] = 0;
      a += run;
    }
    S.level_of[S.n_levels++] = l;
  }
  // zero-copy writes handed to the sink from this slot must have retired
  // before the slot is overwritten (src/writer.h:44-49)
  if (sink->wait_fence)
    for (int k = 0; k < S.n_levels; ++k)
      sink->wait_fence(sink, uint8_t(S.level_of[k]), S.fence[S.level_of[k]]);
  // Compressed input: aggregate on its own stream (bound by the host link)
  // so the next batch's LOD and encoders overlap with it.  Uncompressed
  // input reads the chunk pool itself and stays in order on the compute
  // stream.
  cudaStream_t sa = s_comp;
  if (coded) {
    CK(cudaEventRecord(ev_codec_done[si], se));
    CK(cudaStreamWaitEvent(s_agg, ev_codec_done[si], 0));
    sa = s_agg;
  }
  if (timed_begin(sa, &metrics.aggregate, 0, 0))
    return 1;
  CK(launch_aggregate(ab, d_agg_scratch + si * agg_scratch_slot, sa));
  // the shard index entries of the batch and the index blobs (with their
  // crc32c) of every shard epoch it completes
  {
    IndexBatch ib{};
    ib.alignment = cfg.shard_alignment;
    for (int k = 0; k < S.n_levels; ++k) {
      const int l = S.level_of[k];
      const LevelPlan& V = P.lv[l];
      DeliverySlot::Level& D = S.lv[l];
      IndexLevel& X = ib.lv[ib.nlevels++];
      X.index = d_index[l];
      X.cursor = d_cursor[l];
      X.offsets = D.offsets;
      X.real_sizes = D.real_sizes;
      X.runs = D.runs;
      X.n_runs = D.n_runs;
      X.n_active = S.active[l];
      X.cpi = V.cps_inner;
      X.cps_total = V.cps_total;
      X.shards = V.shard_inner_count;
      X.blobs = D.blobs;
      X.blob_bytes = blob_bytes[l];
      ib.max_shards = std::max<uint64_t>(ib.max_shards, V.shard_inner_count);
    }
    CK(launch_index(ib, sa));
  }
  // to the host: the expected bytes by the copy engine, the rest (if the
  // batch is larger: the first batch, or a less compressible one) by a
  // kernel that reads the total on the device -- no host wait either way
  TailCopies tails{};
  uint64_t tail_max = 0;
  for (int k = 0; k < S.n_levels; ++k) {
    DeliverySlot::Level& D = S.lv[S.level_of[k]];
    if (!D.d_data)
      continue;
    D.copied = std::min(agg_estimate[S.level_of[k]], D.data_cap);
    if (D.copied)
      CK(cudaMemcpyAsync(D.data, D.d_data, D.copied, cudaMemcpyDeviceToHost, sa));
    if (D.copied < D.data_cap) {
      TailCopy& t = tails.lv[tails.n++];
      t.dst = D.data;
      t.src = D.d_data;
      t.total = D.offsets + D.positions; // mapped: written by the aggregation
      t.extra = cfg.shard_alignment;     // the zeroed slack after the batch
      t.start = D.copied;
      tail_max = std::max(tail_max, D.data_cap - D.copied);
    }
  }
  CK(launch_tail_copy(tails, tail_max, sa));
  if (timed_end(sa))
    return 1;
  CK(cudaEventRecord(ev_agg_done[si], sa));
  CK(cudaEventRecord(ev_batch[si], sa));
  S.busy = 1;
  S.seq = ++batch_seq;
  S.epoch_done_ms.swap(pending_epoch_ms);
  pending_epoch_ms.clear();
  next_slot ^= 1;
  pool_claimed = false;
  return 0;
}

// Write one delivered batch to the shard sink
// (src/zarr/shard_delivery.c:105-204).
int Stream::deliver(int si)
{
  DeliverySlot& S = slot[si];
  if (!S.busy)
    return 0;
  CK(cudaEventSynchronize(ev_batch[si]));
  S.busy = 0;
  resolve_timers(false);
  for (int k = 0; k < S.n_levels; ++k) {
    const int l = S.level_of[k];
    DeliverySlot::Level& D = S.lv[l];
    if (!D.d_data)
      continue;
    const uint64_t total = D.offsets[D.positions];
    // (bytes beyond the expected size arrived by the tail kernel).  The
    // larger of the last two batches: a partial batch (a request's last)
    // does not shrink the copy of the full one after it (the next request
    // on this stream)
    const uint64_t base = std::max(total, agg_prev_total[l]);
    agg_prev_total[l] = total;
    agg_estimate[l] = base + base / 32 + (16u << 10);
  }
  const double t0 = now_ms();
  uint64_t bytes_out = 0;
  const uint64_t sa = cfg.shard_alignment;
  for (int k = 0; k < S.n_levels; ++k) {
    const int l = S.level_of[k];
    const uint32_t n_active = S.active[l];
    const LevelPlan& V = P.lv[l];
    const DeliverySlot::Level& D = S.lv[l];
    const uint64_t cpi = V.cps_inner;
    Shards& SS = shards[l];
    uint32_t a = 0, finals = 0;
    while (a < n_active) {
      const uint32_t left = uint32_t(V.cps_append - SS.epoch_in_shard);
      const uint32_t run = std::min(left, n_active - a);
      for (uint64_t s = 0; s < V.shard_inner_count; ++s) {
        Shard& sh = SS.sh[s];
        if (!sh.w) {
          sh.w = sink->open(sink, uint8_t(l),
                            SS.shard_epoch * V.shard_inner_count + s);
          if (!sh.w)
            return 1;
        }
        const uint64_t j0 = s * n_active * cpi + uint64_t(a) * cpi;
        const uint64_t j1 = j0 + uint64_t(run) * cpi;
        const uint64_t nbytes = D.offsets[j1] - D.offsets[j0];
        const uint64_t wbytes = sa ? round_up(nbytes, sa) : nbytes;
        if (nbytes > 0) {
          const uint8_t* src = D.data + D.offsets[j0];
          const bool aligned = sa == 0 || uintptr_t(src) % sa == 0;
          int rc;
          if (aligned && sh.w->write_direct)
            rc = sh.w->write_direct(sh.w, sh.cursor, src, src + wbytes);
          else
            rc = sh.w->write(sh.w, sh.cursor, src, src + wbytes);
          if (rc)
            return 1;
          bytes_out += wbytes;
        }
        sh.cursor += wbytes;
      }
      SS.epoch_in_shard += run;
      a += run;
      if (SS.epoch_in_shard >= V.cps_append) {
        // the index blobs the device built for this shard epoch
        const uint8_t* blobs =
          D.blobs + uint64_t(finals) * V.shard_inner_count * blob_bytes[l];
        ++finals;
        if (write_index_blobs(l, blobs))
          return 1;
      }
    }
    if (sink->record_fence) {
      io_done[l] = sink->record_fence(sink, uint8_t(l));
      S.fence[l] = io_done[l];
    }
  }
  const double t1 = now_ms();
  add_metric(metrics.sink, float(t1 - t0), 0, double(bytes_out));
  for (double e : S.epoch_done_ms)
    latencies_ms.push_back(t1 - e);
  S.epoch_done_ms.clear();
  return 0;
}

// Write each open shard's index blob -- zero padding to the alignment, the
// index of (offset, nbytes) u64 pairs (all ones for an empty slot), its
// crc32c, as the device built them -- and finalize the shards of the level
// (src/zarr/shard_delivery.c:36-102).
int Stream::write_index_blobs(int l, const uint8_t* blobs)
{
  Shards& SS = shards[l];
  int err = 0;
  for (size_t s = 0; s < SS.sh.size(); ++s) {
    Shard& sh = SS.sh[s];
    if (!sh.w)
      continue;
    const uint8_t* b = blobs + s * blob_bytes[l];
    if (sh.w->write(sh.w, sh.cursor, b, b + blob_bytes[l]))
      err = 1;
    if (sh.w->finalize(sh.w))
      err = 1;
    sh.w = nullptr;
    sh.cursor = 0;
  }
  SS.epoch_in_shard = 0;
  SS.shard_epoch++;
  return err;
}

// Finalize a level's partly filled shard epoch at the flush: the device
// writes the index blobs of its current state (and resets it).
int Stream::finalize_level(int l)
{
  const LevelPlan& V = P.lv[l];
  IndexBatch ib{};
  ib.alignment = cfg.shard_alignment;
  ib.nlevels = 1;
  ib.max_shards = V.shard_inner_count;
  IndexLevel& X = ib.lv[0];
  X.index = d_index[l];
  X.cursor = d_cursor[l];
  X.cpi = V.cps_inner;
  X.cps_total = V.cps_total;
  X.shards = V.shard_inner_count;
  X.blobs = h_flush_blobs[l];
  X.blob_bytes = blob_bytes[l];
  X.flush = 1;
  const cudaStream_t st = agg_stream();
  CK(launch_index(ib, st));
  CK(cudaStreamSynchronize(st));
  kick_eis[l] = 0;
  return write_index_blobs(l, h_flush_blobs[l]);
}

int Stream::drain_all()
{
  for (int k = 0; k < 2; ++k) {
    // deliver in submission order
    int first = -1;
    for (int i = 0; i < 2; ++i)
      if (slot[i].busy && (first < 0 || slot[i].seq < slot[first].seq))
        first = i;
    if (first < 0)
      break;
    if (deliver(first))
      return 1;
  }
  return 0;
}

int Stream::deliver_ready()
{
  for (int k = 0; k < 2; ++k) {
    int first = -1;
    for (int i = 0; i < 2; ++i)
      if (slot[i].busy && (first < 0 || slot[i].seq < slot[first].seq))
        first = i;
    if (first < 0)
      return 0;
    const cudaError_t q = cudaEventQuery(ev_batch[first]);
    if (q == cudaErrorNotReady)
      return 0;
    if (q != cudaSuccess) {
      std::fprintf(stderr, "chucky_gb300: batch failed: %s\n", cudaGetErrorString(q));
      return 1;
    }
    if (deliver(first))
      return 1;
  }
  return 0;
}

int Stream::batch_boundary()
{
  // The previous batch is delivered while this one runs on the GPU: now if
  // the GPU is already done with it, otherwise when its slot is needed
  // again (the next kick, which delivers a busy slot first) or at the
  // flush.  Not waiting here lets the caller enqueue the next batch's
  // input copies and LOD while two batches are in flight.
  const int prev = next_slot ^ 1;
  if (kick_batch(accumulated, masks))
    return 1;
  accumulated = 0;
  if (slot[prev].busy && slot[prev].seq < batch_seq &&
      cudaEventQuery(ev_batch[prev]) == cudaSuccess)
    return deliver(prev);
  return 0;
}

// ---------------------------------------------------------------------------
// writer vtable
// ---------------------------------------------------------------------------

// Issue the copy of the staging slot being filled (if it holds anything).
int Stream::stage_issue()
{
  if (!stage_fill)
    return 0;
  CK(cudaMemcpyAsync(stage_dst, h_stage[stage_cur], stage_fill,
                     cudaMemcpyHostToDevice, s_copy));
  CK(cudaEventRecord(ev_stage[stage_cur], s_copy));
  stage_used[stage_cur] = true;
  stage_cur = (stage_cur + 1) % kStageSlots;
  stage_fill = 0;
  return 0;
}

// Copy host bytes through the staging ring to `dst` in an epoch buffer.
int Stream::stage_copy(uint8_t* dst, const uint8_t* src, uint64_t bytes)
{
  while (bytes) {
    if (stage_fill && dst != stage_dst + stage_fill && stage_issue())
      return 1;
    if (!stage_fill) {
      if (stage_used[stage_cur]) // its previous copy must have read it
        CK(cudaEventSynchronize(ev_stage[stage_cur]));
      stage_dst = dst;
    }
    const uint64_t n = std::min(bytes, stage_bytes - stage_fill);
    std::memcpy(h_stage[stage_cur] + stage_fill, src, n);
    stage_fill += n;
    dst += n;
    src += n;
    bytes -= n;
    if (stage_fill == stage_bytes && stage_issue())
      return 1;
  }
  return 0;
}

namespace {

enum class Source
{
  staged, // pageable, or small pinned: through the staging ring
  direct, // large pinned host memory: copied from the caller, waited for
  device, // device memory: copied on the device, waited for
};

Source classify(const void* p, uint64_t bytes, uint64_t small)
{
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return Source::staged;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
    return Source::device;
  if (a.type == cudaMemoryTypeHost && bytes > small)
    return Source::direct;
  return Source::staged;
}

} // namespace

writer_result Stream::append(slice in)
{
  return append_async(in, nullptr);
}

writer_result Stream::append_async(slice in, cudaStream_t producer)
{
  if (flushed)
    return writer_finished_at(in.beg, in.end);
  const uint8_t* src = static_cast<const uint8_t*>(in.beg);
  const uint8_t* end = static_cast<const uint8_t*>(in.end);
  if (src >= end)
    return writer_result{ 0, { src, end } };
  const uint64_t ee = layout.epoch_elements;
  const double t0 = now_ms();
  const Source kind = classify(src, uint64_t(end - src), stage_small);
  if (producer) {
    // stream-ordered hand-off of device memory only
    if (kind != Source::device)
      return writer_error_at(src, end);
    if (cudaEventRecord(ev_producer, producer) != cudaSuccess ||
        cudaStreamWaitEvent(s_copy, ev_producer, 0) != cudaSuccess)
      return writer_error_at(src, end);
  }
  uint64_t copied = 0;
  double memcpy_ms = 0;
  while (src < end) {
    if (max_cursor > 0 && cursor >= max_cursor) {
      // every copy out of the caller's buffer has finished after this
      cudaStreamSynchronize(s_copy);
      if (flush_all())
        return writer_error_at(src, end);
      return writer_finished_at(src, end);
    }
    uint64_t n = std::min<uint64_t>(ee - cursor % ee,
                                    uint64_t(end - src) / P.bpe);
    if (max_cursor > 0)
      n = std::min<uint64_t>(n, max_cursor - cursor);
    if (n == 0)
      break;
    if (in_fill == 0 &&
        cudaStreamWaitEvent(s_copy, ev_input_free[in_buf], 0) != cudaSuccess)
      return writer_error_at(src, end);
    uint8_t* dst = d_epoch[in_buf] + in_fill * P.bpe;
    if (kind == Source::staged) {
      const double m0 = now_ms();
      if (stage_copy(dst, src, n * P.bpe))
        return writer_error_at(src, end);
      memcpy_ms += now_ms() - m0;
    } else if (cudaMemcpyAsync(dst, src, n * P.bpe, cudaMemcpyDefault, s_copy) !=
               cudaSuccess) {
      return writer_error_at(src, end);
    }
    copied += n * P.bpe;
    in_fill += n;
    cursor += n;
    src += n * P.bpe;
    if (cursor % ee == 0) {
      if (run_epoch(ee))
        return writer_error_at(src, end);
      if (accumulated == P.K && batch_boundary())
        return writer_error_at(src, end);
    }
  }
  if (batch_deadline_ms > 0) {
    // latency bound: the batch being filled goes as a partial batch once
    // its oldest epoch has waited the deadline, and finished batches are
    // delivered now rather than at the next kick
    if (accumulated > 0 && !pending_epoch_ms.empty() &&
        now_ms() - pending_epoch_ms.front() >= batch_deadline_ms && batch_boundary())
      return writer_error_at(src, end);
    if (deliver_ready())
      return writer_error_at(src, end);
  }
  if (producer) {
    // the producer's later work (e.g. overwriting its buffer) waits for
    // the copies out of it
    if (cudaEventRecord(ev_consumed, s_copy) != cudaSuccess ||
        cudaStreamWaitEvent(producer, ev_consumed, 0) != cudaSuccess)
      return writer_error_at(src, end);
  } else if (kind != Source::staged) {
    // the caller's buffer is only borrowed for the duration of the call
    if (cudaStreamSynchronize(s_copy) != cudaSuccess)
      return writer_error_at(src, end);
  }
  if (copied) {
    add_metric(metrics.h2d, float(now_ms() - t0), double(copied), double(copied));
    if (memcpy_ms > 0)
      add_metric(metrics.memcpy, float(memcpy_ms), double(copied), double(copied));
  }
  return writer_result{ 0, { src, end } };
}

int Stream::flush_all()
{
  const uint64_t ee = layout.epoch_elements;
  if (cursor % ee != 0 && run_epoch(cursor % ee))
    return 1;
  if (accumulated > 0 && batch_boundary())
    return 1;
  if (drain_all())
    return 1;
  if (P.append_downsample && d_accum) {
    uint32_t drain = 0;
    for (int l = 1; l < P.nlod; ++l)
      if (counts[l] > 0) {
        if (claim_pool())
          return 1;
        if (lod_tiled) {
          LodTileArgs t = tile;
          t.slot = pool_slot(0);
          t.accum = d_accum;
          CK(launch_lod_drain(t, l, counts[l], s_comp));
        } else {
          CK(launch_lod_emit(lod, l, counts[l], d_accum, d_values, s_comp));
          CK(launch_lod_to_chunks(lod, l, d_values, pool_slot(0), s_comp));
        }
        counts[l] = 0;
        drain |= 1u << l;
      }
    if (drain) {
      uint32_t m[1] = { drain };
      if (kick_batch(1, m) || drain_all())
        return 1;
    }
  }
  for (int l = 0; l < P.nlod; ++l) {
    if (sink->wait_fence)
      sink->wait_fence(sink, uint8_t(l), io_done[l]);
    if (shards[l].epoch_in_shard > 0 && finalize_level(l))
      return 1;
  }
  if (sink->update_append) {
    const dimension* dims = cfg.dimensions;
    for (int l = 0; l < P.nlod; ++l) {
      uint64_t sizes[HALF_MAX_RANK] = {};
      uint64_t inner = 1;
      for (int d = 1; d < P.rank; ++d)
        inner *= dims[d].size;
      for (int d = 1; d < P.na; ++d)
        sizes[d] = dims[d].size;
      uint64_t d0 = inner ? cursor / inner : 0;
      if (l > 0 && P.append_downsample)
        d0 = (d0 + ((uint64_t(1) << l) - 1)) >> l;
      sizes[0] = d0;
      if (sink->update_append(sink, uint8_t(l), P.na, sizes))
        return 1;
    }
  }
  resolve_timers(true);
  return 0;
}

writer_result Stream::flush()
{
  if (flushed)
    return writer_finished_at(nullptr, nullptr);
  const int rc = flush_all();
  flushed = 1;
  return rc ? writer_error() : writer_ok();
}

} // namespace chucky

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

using chucky::Stream;

static writer_result
vt_append(writer* w, slice s)
{
  return reinterpret_cast<tile_stream_gpu*>(w)->impl.append(s);
}

static writer_result
vt_flush(writer* w)
{
  return reinterpret_cast<tile_stream_gpu*>(w)->impl.flush();
}

namespace chucky {

tile_stream_gpu* create_stream(const tile_stream_configuration* config,
                               shard_sink* sink,
                               Engine* engine)
{
  if (!config || !sink || !sink->open)
    return nullptr;
  tile_stream_gpu* s = new (std::nothrow) tile_stream_gpu();
  if (!s)
    return nullptr;
  s->w.append = vt_append;
  s->w.flush = vt_flush;
  s->impl.engine = engine;
  if (s->impl.init(config, sink)) {
    s->impl.release();
    delete s;
    return nullptr;
  }
  return s;
}

} // namespace chucky

extern "C" tile_stream_gpu*
tile_stream_gpu_create(const tile_stream_configuration* config,
                       shard_sink* sink)
{
  return chucky::create_stream(config, sink, nullptr);
}

extern "C" writer_result
tile_stream_gpu_append_device(tile_stream_gpu* s, slice data, void* cuda_stream)
{
  if (!s || !cuda_stream)
    return writer_error_at(data.beg, data.end);
  return s->impl.append_async(data, static_cast<cudaStream_t>(cuda_stream));
}

extern "C" void
tile_stream_gpu_destroy(tile_stream_gpu* s)
{
  if (!s)
    return;
  s->impl.release();
  delete s;
}

extern "C" stream_metrics
tile_stream_gpu_get_metrics(const tile_stream_gpu* s)
{
  const_cast<tile_stream_gpu*>(s)->impl.resolve_timers(false);
  return s->impl.metrics;
}

extern "C" const tile_stream_layout*
tile_stream_gpu_layout(const tile_stream_gpu* s)
{
  return &s->impl.layout;
}

extern "C" writer*
tile_stream_gpu_writer(tile_stream_gpu* s)
{
  return &s->w;
}

extern "C" uint64_t
tile_stream_gpu_cursor(const tile_stream_gpu* s)
{
  return s->impl.cursor;
}

extern "C" tile_stream_status
tile_stream_gpu_status(const tile_stream_gpu* s)
{
  const Stream& I = s->impl;
  tile_stream_status st{};
  st.nlod = I.P.nlod;
  st.append_downsample = I.P.append_downsample;
  st.epochs_per_batch = I.P.K;
  st.max_compressed_size = I.P.max_out;
  st.dtype = I.cfg.dtype;
  st.codec = I.cfg.codec;
  st.codec_batch_size = size_t(I.P.K) * I.P.total_chunks;
  st.batch_accumulated = I.accumulated;
  st.pool_current = 0;
  st.flush_pending = (I.slot[0].busy || I.slot[1].busy) ? 1 : 0;
  return st;
}

extern "C" int
tile_stream_gpu_restart(tile_stream_gpu* s, shard_sink* sink)
{
  if (!s)
    return 1;
  Stream& I = s->impl;
  if (I.cursor != 0 && !I.flushed)
    return 1;
  if (cudaStreamSynchronize(I.s_comp) != cudaSuccess ||
      cudaStreamSynchronize(I.s_enc[0]) != cudaSuccess ||
      cudaStreamSynchronize(I.s_enc[1]) != cudaSuccess ||
      cudaStreamSynchronize(I.s_agg) != cudaSuccess ||
      cudaStreamSynchronize(I.s_copy) != cudaSuccess)
    return 1;
  if (sink)
    I.sink = sink;
  I.cursor = 0;
  I.flushed = 0;
  I.stage_fill = 0;
  for (bool& u : I.stage_used)
    u = false;
  I.pending_epoch_ms.clear();
  I.accumulated = 0;
  I.in_buf = 0;
  I.in_fill = 0;
  for (auto& c : I.counts)
    c = 0;
  for (int l = 0; l < I.P.nlod; ++l) {
    chucky::Shards& S = I.shards[l];
    S.epoch_in_shard = 0;
    S.shard_epoch = 0;
    for (auto& sh : S.sh) {
      sh.cursor = 0;
      sh.w = nullptr;
    }
    const uint64_t ns = I.P.lv[l].shard_inner_count;
    if (cudaMemsetAsync(I.d_index[l], 0xFF, ns * I.P.lv[l].cps_total * 16, I.s_comp) !=
          cudaSuccess ||
        cudaMemsetAsync(I.d_cursor[l], 0, ns * 8, I.s_comp) != cudaSuccess)
      return 1;
    I.kick_eis[l] = 0;
    I.io_done[l] = io_event{};
  }
  if (cudaStreamSynchronize(I.s_comp) != cudaSuccess)
    return 1;
  for (auto& sl : I.slot) {
    sl.busy = 0;
    for (auto& f : sl.fence)
      f = io_event{};
  }
  return 0;
}

namespace {

struct DiscardSink
{
  shard_sink base;
  shard_writer w;
  std::atomic<uint64_t> bytes; // one sink may serve streams on several threads
};

int discard_write(shard_writer* self, uint64_t, const void* b, const void* e)
{
  DiscardSink* d = reinterpret_cast<DiscardSink*>(
    reinterpret_cast<char*>(self) - offsetof(DiscardSink, w));
  d->bytes.fetch_add(uint64_t(static_cast<const char*>(e) - static_cast<const char*>(b)),
                     std::memory_order_relaxed);
  return 0;
}

int discard_finalize(shard_writer*)
{
  return 0;
}

shard_writer* discard_open(shard_sink* self, uint8_t, uint64_t)
{
  return &reinterpret_cast<DiscardSink*>(self)->w;
}

} // namespace

extern "C" shard_sink*
chucky_discard_sink_create(void)
{
  DiscardSink* d = new (std::nothrow) DiscardSink{};
  if (!d)
    return nullptr;
  d->base.open = discard_open;
  d->w.write = discard_write;
  d->w.finalize = discard_finalize;
  return &d->base;
}

extern "C" void
chucky_discard_sink_destroy(shard_sink* s)
{
  delete reinterpret_cast<DiscardSink*>(s);
}

extern "C" uint64_t
chucky_discard_sink_bytes(const shard_sink* s)
{
  return reinterpret_cast<const DiscardSink*>(s)->bytes.load();
}

extern "C" size_t
tile_stream_gpu_latencies(const tile_stream_gpu* s, double* out_ms, size_t cap)
{
  const auto& v = s->impl.latencies_ms;
  if (out_ms)
    for (size_t i = 0; i < v.size() && i < cap; ++i)
      out_ms[i] = v[i];
  return v.size();
}

extern "C" void
tile_stream_gpu_clear_latencies(tile_stream_gpu* s)
{
  s->impl.latencies_ms.clear();
}

extern "C" int
tile_stream_gpu_set_batch_deadline(tile_stream_gpu* s, double ms)
{
  if (!s || !(ms >= 0))
    return 1;
  s->impl.batch_deadline_ms = ms;
  return 0;
}
