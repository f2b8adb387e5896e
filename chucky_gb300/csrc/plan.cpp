// Stream layout planning; see plan.hpp for the reference files it restates.
#include "plan.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace chucky {

namespace {

inline uint64_t div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
inline uint64_t round_up(uint64_t x, uint64_t a) { return div_up(x, a) * a; }

inline int bits_for(uint64_t v) // smallest p with 2^p >= v
{
  int p = 0;
  while ((uint64_t(1) << p) < v)
    ++p;
  return p;
}

// Leading append dims: the chunk_size == 1 prefix, cut after the first
// downsampled dim (src/dimension.c:178-196).
uint8_t count_append_dims(const dimension* d, uint8_t rank)
{
  uint8_t n = 0;
  while (n < rank && d[n].chunk_size == 1)
    ++n;
  if (n <= 1)
    return 1;
  for (uint8_t i = 0; i < n; ++i)
    if (d[i].downsample)
      return uint8_t(i + 1);
  return n;
}

bool dims_are_valid(const dimension* d, uint8_t rank)
{
  if (!d || rank == 0 || rank > HALF_MAX_RANK)
    return false;
  for (int i = 0; i < rank; ++i)
    if (d[i].chunk_size == 0 || (i > 0 && d[i].size == 0))
      return false;
  if (d[0].size == 0 && d[0].chunks_per_shard == 0)
    return false;
  const uint8_t na = count_append_dims(d, rank);
  uint64_t seen = 0;
  for (int i = 0; i < rank; ++i) {
    const uint8_t p = d[i].storage_position;
    if (p >= rank || (seen >> p & 1) || (i < na && p != i))
      return false;
    seen |= uint64_t(1) << p;
  }
  return true;
}

// Extent of half `b` of a node at (prefix, scale), clipped to `size`.
inline uint64_t half_len(uint64_t size, uint64_t lo, uint64_t scale)
{
  return lo >= size ? 0 : std::min(size - lo, scale);
}

void morton_successor(int ndim, int p, uint64_t* c)
{
  for (int bit = 0; bit < p; ++bit)
    for (int d = 0; d < ndim; ++d) {
      c[d] ^= uint64_t(1) << bit;
      if (c[d] >> bit & 1)
        return;
    }
  std::fill(c, c + ndim, 0);
  c[0] = uint64_t(1) << p;
}

// Lifted layout of one level (src/stream/config.c:84-138).
void level_layout(tile_stream_layout& L,
                  const StreamPlan& P,
                  const dimension* dims,
                  const uint64_t* shape)
{
  std::memset(&L, 0, sizeof(L));
  uint64_t count[HALF_MAX_RANK];
  L.lifted_rank = uint8_t(2 * P.rank);
  L.chunk_elements = 1;
  for (int i = 0; i < P.rank; ++i) {
    count[i] = shape[i] ? div_up(shape[i], dims[i].chunk_size) : 1;
    L.lifted_shape[2 * i] = count[i];
    L.lifted_shape[2 * i + 1] = dims[i].chunk_size;
    L.chunk_elements *= dims[i].chunk_size;
  }
  L.chunk_stride = round_up(L.chunk_elements * P.bpe, kChunkAlign) / P.bpe;
  int64_t within = 1, across = int64_t(L.chunk_stride);
  for (int j = P.rank - 1; j >= 0; --j) { // storage order, innermost last
    const int i = P.order[j];
    L.lifted_strides[2 * i + 1] = within;
    within *= int64_t(dims[i].chunk_size);
    L.lifted_strides[2 * i] = across;
    across *= int64_t(count[i]);
  }
  L.chunks_per_epoch = 1;
  for (int d = P.na; d < P.rank; ++d)
    L.chunks_per_epoch *= count[d];
  L.epoch_elements = L.chunks_per_epoch * L.chunk_elements;
  for (int d = 0; d < P.na; ++d) // every epoch reuses the same slots
    L.lifted_strides[2 * d] = 0;
  L.chunk_pool_bytes = L.chunks_per_epoch * L.chunk_stride * P.bpe;
}

} // namespace

uint64_t codec_bound(int codec_id, uint64_t n)
{
  switch (codec_id) {
    case CODEC_NONE:
      return n;
    case CODEC_LZ4_NON_STANDARD:
      return n + n / 255 + 16;
    case CODEC_ZSTD: {
      const uint64_t lim = 128u << 10;
      return n + (n >> 8) + (n < lim ? (lim - n) >> 11 : 0);
    }
    default:
      return 0;
  }
}

uint64_t morton_rank(int ndim,
                     const uint64_t* shape,
                     const uint64_t* coords,
                     int depth)
{
  // Number of in-shape points that precede `coords` in Z order, where the
  // digit of a tree level packs one bit per dim (dim 0 least significant).
  uint64_t mx = 0;
  for (int d = 0; d < ndim; ++d)
    mx = std::max(mx, shape[d]);
  int p = bits_for(mx);
  for (int d = 0; d < ndim; ++d)
    if (coords[d] > 0)
      p = std::max(p, bits_for(coords[d] + 1));
  const int depth_total = p + depth;
  uint64_t rank = 0;
  uint64_t node[LOD_MAX_NDIM] = {};
  for (int t = 0; t < depth_total; ++t) {
    const uint64_t scale = uint64_t(1) << (depth_total - 1 - t);
    unsigned digit = 0;
    if (t < p)
      for (int d = 0; d < ndim; ++d)
        digit |= unsigned(coords[d] >> (p - 1 - t) & 1) << d;
    uint64_t lo[LOD_MAX_NDIM], hi[LOD_MAX_NDIM];
    for (int d = 0; d < ndim; ++d) {
      lo[d] = half_len(shape[d], (2 * node[d]) * scale, scale);
      hi[d] = half_len(shape[d], (2 * node[d] + 1) * scale, scale);
    }
    // Points in sibling cells ordered before the chosen one: for every
    // set digit bit d, the cells that agree above d, take the low half at
    // d, and are free below d.
    uint64_t free_below[LOD_MAX_NDIM + 1];
    free_below[0] = 1;
    for (int d = 0; d < ndim; ++d)
      free_below[d + 1] = free_below[d] * (lo[d] + hi[d]);
    uint64_t fixed_above = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      const bool set = digit >> d & 1;
      if (set)
        rank += fixed_above * lo[d] * free_below[d];
      fixed_above *= set ? hi[d] : lo[d];
    }
    for (int d = 0; d < ndim; ++d)
      node[d] = 2 * node[d] + (digit >> d & 1);
  }
  return rank;
}

uint64_t ravel(int rank,
               const uint64_t* shape,
               const int64_t* strides,
               uint64_t idx)
{
  uint64_t o = 0;
  for (int d = rank - 1; d >= 0; --d) {
    o += (idx % shape[d]) * uint64_t(strides[d]);
    idx /= shape[d];
  }
  return o;
}

int plan_stream(const tile_stream_configuration* cfg, StreamPlan* out)
{
  if (!cfg || !out)
    return 1;
  StreamPlan& P = *out;
  P = StreamPlan();
  const dimension* dims = cfg->dimensions;
  const uint8_t rank = cfg->rank;
  P.bpe = dtype_bpe(cfg->dtype);
  if (!P.bpe || !cfg->buffer_capacity_bytes || cfg->max_threads < 0 ||
      !dims_are_valid(dims, rank))
    return 1;
  if (cfg->codec.id == CODEC_LZ4_NON_STANDARD && cfg->codec.level == 0)
    return 1; // LZ4 requires level >= 1 (src/stream/config.c:171-174)
  if (!codec_is_gpu_supported(cfg->codec.id))
    return 1;
  if (cfg->max_nlod < 0 || cfg->max_nlod > LOD_MAX_LEVELS)
    return 1;

  P.rank = rank;
  P.na = count_append_dims(dims, rank);
  for (int d = 0; d < rank; ++d)
    P.order[dims[d].storage_position] = uint8_t(d);
  for (int d = P.na; d < rank; ++d)
    if (dims[d].downsample)
      P.lod_mask |= 1u << d;
  P.append_downsample = dims[P.na - 1].downsample ? 1 : 0;
  if (P.append_downsample) {
    const int m = cfg->append_reduce_method;
    if (m != lod_reduce_mean && m != lod_reduce_min && m != lod_reduce_max)
      return 1;
    if (!P.lod_mask)
      return 1;
  }

  // Epoch-split shape: unbounded dims use their chunk size, append dims
  // hold one chunk per epoch (src/lod/lod_plan.c:277-345).
  uint64_t shape0[HALF_MAX_RANK] = {};
  for (int d = 0; d < rank; ++d)
    shape0[d] = d < P.na ? dims[d].chunk_size
                         : (dims[d].size ? dims[d].size : dims[d].chunk_size);
  for (int d = 0; d < rank; ++d) {
    if (P.lod_mask >> d & 1)
      P.lod_to_dim[P.lod_ndim++] = d;
    else {
      P.fixed_to_dim[P.fixed_ndim] = d;
      P.fixed_shape[P.fixed_ndim++] = shape0[d];
      P.fixed_count *= shape0[d];
    }
  }

  // Levels: halve the LOD dims until each fits in one chunk
  // (src/lod/lod_plan.c:213-275).
  const int max_levels = cfg->max_nlod ? cfg->max_nlod : LOD_MAX_LEVELS;
  std::memcpy(P.lv[0].shape, shape0, sizeof(shape0));
  int nlod = 1;
  for (;;) {
    bool fits = true;
    for (int k = 0; k < P.lod_ndim; ++k) {
      const int d = P.lod_to_dim[k];
      fits &= div_up(P.lv[nlod - 1].shape[d], dims[d].chunk_size) <= 1;
    }
    if (nlod >= max_levels || fits)
      break;
    std::memcpy(P.lv[nlod].shape, P.lv[nlod - 1].shape, sizeof(shape0));
    for (int k = 0; k < P.lod_ndim; ++k) {
      const int d = P.lod_to_dim[k];
      P.lv[nlod].shape[d] = (P.lv[nlod - 1].shape[d] + 1) / 2;
    }
    ++nlod;
  }
  P.multiscale = P.lod_mask != 0;
  P.nlod = P.multiscale ? nlod : 1;
  for (int l = 0; l < nlod; ++l) {
    P.lv[l].lod_nelem = 1;
    for (int k = 0; k < P.lod_ndim; ++k)
      P.lv[l].lod_nelem *= P.lv[l].shape[P.lod_to_dim[k]];
    P.lod_end[l] = (l ? P.lod_end[l - 1] : 0) + P.lv[l].lod_nelem;
  }
  P.n_ends = (P.multiscale && P.nlod > 1) ? P.lod_end[P.nlod - 1] - P.lod_end[0] : 0;

  for (int l = 0; l < P.nlod; ++l) {
    level_layout(P.lv[l].layout, P, dims, P.lv[l].shape);
    P.lv[l].chunk_offset = P.total_chunks;
    P.total_chunks += P.lv[l].layout.chunks_per_epoch;
  }
  const tile_stream_layout& L0 = P.lv[0].layout;
  if (L0.chunks_per_epoch == 0 ||
      L0.chunk_elements > UINT64_MAX / L0.chunks_per_epoch)
    return 1;

  // Epochs per batch (src/stream/config.c:31-45).
  uint32_t K = cfg->epochs_per_batch;
  if (K == 0) {
    const uint64_t target =
      cfg->target_batch_chunks ? cfg->target_batch_chunks : 1024;
    const uint64_t need = div_up(target, P.total_chunks);
    K = 1;
    while (K < need && K < MAX_BATCH_EPOCHS)
      K <<= 1;
  }
  P.K = std::min<uint32_t>(K, MAX_BATCH_EPOCHS);

  P.chunk_bytes = L0.chunk_elements * P.bpe;
  P.slot_bytes = P.total_chunks * L0.chunk_stride * P.bpe;
  P.epoch_bytes = L0.epoch_elements * P.bpe;
  P.max_out = codec_bound(cfg->codec.id, P.chunk_bytes);

  // Shard geometry and shard-order layout of each level
  // (src/stream/config.c:298-373, src/stream/types.aggregate.c:65-143).
  for (int l = 0; l < P.nlod; ++l) {
    LevelPlan& V = P.lv[l];
    uint64_t cnt[HALF_MAX_RANK], cps[HALF_MAX_RANK], nsh[HALF_MAX_RANK];
    for (int d = 0; d < rank; ++d) {
      const uint64_t s = l == 0 ? dims[d].size : V.shape[d];
      cnt[d] = s ? div_up(s, dims[d].chunk_size) : 1;
      uint64_t c = dims[d].chunks_per_shard ? dims[d].chunks_per_shard : cnt[d];
      if (s && cnt[d] < c)
        c = cnt[d];
      cps[d] = c;
      nsh[d] = div_up(cnt[d], c);
    }
    V.period = (P.append_downsample && l > 0) ? (1u << l) : 1u;
    V.batch_active = P.K >= V.period ? P.K / V.period : 0;
    V.shard_inner_count = 1;
    for (int d = P.na; d < rank; ++d)
      V.shard_inner_count *= nsh[d];

    V.agg_rank = uint8_t(2 * (rank - P.na));
    V.covering = 1;
    V.cps_inner = 1;
    for (int j = P.na; j < rank; ++j) {
      const int d = P.order[j], k = j - P.na;
      V.agg_shape[2 * k] = nsh[d];
      V.agg_shape[2 * k + 1] = cps[d];
      V.covering *= nsh[d] * cps[d];
      V.cps_inner *= cps[d];
    }
    if (V.covering > UINT32_MAX)
      return 1;
    uint64_t shard_acc = 1, within_acc = 1;
    for (int j = rank - 1; j >= P.na; --j) {
      const int d = P.order[j], k = j - P.na;
      V.agg_strides[2 * k] = int64_t(shard_acc * V.cps_inner);
      shard_acc *= nsh[d];
      V.agg_strides[2 * k + 1] = int64_t(within_acc);
      within_acc *= cps[d];
    }
    uint64_t ca = 1;
    for (int d = 0; d < P.na; ++d)
      ca *= cps[d];
    if (V.period > 1)
      ca = ca > V.period ? ca / V.period : 1;
    V.cps_append = ca;
    V.cps_total = ca * V.cps_inner;
  }

  if (dims[0].size > 0) {
    P.max_cursor = L0.epoch_elements;
    for (int d = 0; d < P.na; ++d)
      P.max_cursor *= div_up(dims[d].size, dims[d].chunk_size);
  }
  return 0;
}

// Morton window ends of every level above 0:
// ends[rank(parent)] = child rank one past the parent's last child
// (src/lod/lod_plan.c:105-125, 151-210).  Host work proportional to the
// pyramid's element count; only the general (Morton-buffer) LOD path reads
// the table.
void plan_build_ends(StreamPlan& P)
{
  P.ends.clear();
  if (!P.n_ends)
    return;
  {
    P.ends.assign(P.n_ends, 0);
    for (int l = 0; l + 1 < P.nlod; ++l) {
      uint64_t child[LOD_MAX_NDIM], parent[LOD_MAX_NDIM];
      uint64_t mx = 0;
      for (int k = 0; k < P.lod_ndim; ++k) {
        child[k] = P.lv[l].shape[P.lod_to_dim[k]];
        parent[k] = P.lv[l + 1].shape[P.lod_to_dim[k]];
        mx = std::max(mx, parent[k]);
      }
      const int p = bits_for(mx);
      uint64_t* seg = P.ends.data() + (P.lod_end[l] - P.lod_end[0]);
      for (uint64_t j = 0; j < P.lv[l + 1].lod_nelem; ++j) {
        uint64_t c[LOD_MAX_NDIM], nx[LOD_MAX_NDIM], r = j;
        for (int k = 0; k < P.lod_ndim; ++k) { // first dim fastest
          c[k] = r % parent[k];
          r /= parent[k];
        }
        std::memcpy(nx, c, sizeof(uint64_t) * size_t(P.lod_ndim));
        morton_successor(P.lod_ndim, p, nx);
        seg[morton_rank(P.lod_ndim, parent, c, 0)] =
          morton_rank(P.lod_ndim, child, nx, 1);
      }
    }
  }
}

} // namespace chucky
