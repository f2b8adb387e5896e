/* CPU oracle for the streaming ingest path -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates the reference CPU backend in plain C.  Each function names the
 * reference file:line whose algorithm it follows.  Loaded only by tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py. */
#define _GNU_SOURCE
#include "oracle.h"

#include <dlfcn.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef _Float16 f16;

/* 1: reproduce the reference byte for byte, including what it leaves in
 * buffers it does not clear (stale tail of a partial final epoch, the dim-0
 * drain LUT above).  0: the tail of a partial epoch is the fill value 0 and
 * drained levels are read from where they were written. */
static int g_quirks = 1;

void
oracle_set_reference_quirks(int on)
{
  g_quirks = on ? 1 : 0;
}

/* ------------------------------------------------------------------ */
/* small helpers (src/util/prelude.h, src/util/ceildiv.h)              */
/* ------------------------------------------------------------------ */

static inline uint64_t
cdiv(uint64_t a, uint64_t b)
{
  return (a + b - 1) / b;
}

static inline uint64_t
aup(uint64_t x, uint64_t a)
{
  return (x + a - 1) / a * a;
}

static inline int
clog2(uint64_t v)
{
  int p = 0;
  while ((1ull << p) < v)
    ++p;
  return p;
}

static uint64_t
shape_max(int n, const uint64_t* s)
{
  uint64_t m = 0;
  for (int i = 0; i < n; ++i)
    if (s[i] > m)
      m = s[i];
  return m;
}

/* ------------------------------------------------------------------ */
/* dims (src/dimension.c:178-196, 198-247)                             */
/* ------------------------------------------------------------------ */

static uint8_t
o_n_append(const struct dimension* dims, uint8_t rank)
{
  uint8_t max_n = 0;
  for (uint8_t d = 0; d < rank; ++d) {
    if (dims[d].chunk_size != 1)
      break;
    max_n = (uint8_t)(d + 1);
  }
  if (max_n <= 1)
    return 1;
  for (uint8_t d = 0; d < max_n; ++d)
    if (dims[d].downsample)
      return (uint8_t)(d + 1);
  return max_n;
}

static int
o_dims_ok(const struct dimension* dims, uint8_t rank)
{
  if (!dims || rank == 0 || rank > HALF_MAX_RANK)
    return 0;
  for (int d = 0; d < rank; ++d)
    if (dims[d].chunk_size == 0)
      return 0;
  for (int d = 1; d < rank; ++d)
    if (dims[d].size == 0)
      return 0;
  if (dims[0].size == 0 && dims[0].chunks_per_shard == 0)
    return 0;
  uint8_t na = o_n_append(dims, rank);
  for (int d = 0; d < na; ++d)
    if (dims[d].storage_position != d)
      return 0;
  uint64_t seen = 0;
  for (int d = 0; d < rank; ++d) {
    uint8_t j = dims[d].storage_position;
    if (j >= rank || (seen & (1ull << j)))
      return 0;
    seen |= 1ull << j;
  }
  return 1;
}

/* ------------------------------------------------------------------ */
/* Morton ranks and LOD windows (src/lod/lod_plan.c:12-125)            */
/* ------------------------------------------------------------------ */

static uint64_t
half_extent(uint64_t size, uint64_t lo, uint64_t scale)
{
  if (lo >= size)
    return 0;
  uint64_t e = size - lo;
  return e < scale ? e : scale;
}

/* Rank of `coords` among the in-shape points of a (possibly non power of
 * two) box enumerated in Z order, dim 0 being the least significant digit
 * bit.  depth>0 treats coords as a node `depth` levels above the leaves and
 * returns the rank of its first leaf.  Follows src/lod/lod_plan.c:21-72. */
uint64_t
oracle_morton_rank(int ndim,
                   const uint64_t* shape,
                   const uint64_t* coords,
                   int depth)
{
  int p = clog2(shape_max(ndim, shape));
  for (int d = 0; d < ndim; ++d) {
    int pc = coords[d] > 0 ? clog2(coords[d] + 1) : 0;
    if (pc > p)
      p = pc;
  }
  const int levels = p + depth;
  uint64_t rank = 0;
  uint64_t prefix[LOD_MAX_NDIM] = { 0 };
  for (int lv = 0; lv < levels; ++lv) {
    const uint64_t scale = 1ull << (levels - 1 - lv);
    int digit = 0;
    if (lv < p)
      for (int d = 0; d < ndim; ++d)
        digit |= (int)((coords[d] >> (p - 1 - lv)) & 1) << d;
    uint64_t ext0[LOD_MAX_NDIM], ext1[LOD_MAX_NDIM];
    for (int d = 0; d < ndim; ++d) {
      ext0[d] = half_extent(shape[d], (prefix[d] * 2) * scale, scale);
      ext1[d] = half_extent(shape[d], (prefix[d] * 2 + 1) * scale, scale);
    }
    /* below[d] = number of points in the node restricted to dims < d */
    uint64_t below[LOD_MAX_NDIM + 1];
    below[0] = 1;
    for (int d = 0; d < ndim; ++d)
      below[d + 1] = below[d] * (ext0[d] + ext1[d]);
    uint64_t above = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      const int bit = (digit >> d) & 1;
      if (bit)
        rank += above * ext0[d] * below[d];
      above *= bit ? ext1[d] : ext0[d];
    }
    for (int d = 0; d < ndim; ++d)
      prefix[d] = prefix[d] * 2 + (uint64_t)((digit >> d) & 1);
  }
  return rank;
}

/* Z-order successor of coords on a 2^p grid (src/lod/lod_plan.c:74-87). */
static void
morton_successor(int ndim, int p, uint64_t* c)
{
  for (int bit = 0; bit < p; ++bit)
    for (int d = 0; d < ndim; ++d) {
      const uint64_t m = 1ull << bit;
      c[d] ^= m;
      if (c[d] & m)
        return;
    }
  memset(c, 0, (size_t)ndim * sizeof(uint64_t));
  c[0] = 1ull << p;
}

/* ends[rank(parent)] = rank (in child Z order) one past the parent's last
 * child (src/lod/lod_plan.c:105-125). */
static void
fill_window_ends(int ndim,
                 const uint64_t* child,
                 const uint64_t* parent,
                 uint64_t n_parents,
                 uint64_t* ends)
{
  const int p = clog2(shape_max(ndim, parent));
  for (uint64_t j = 0; j < n_parents; ++j) {
    uint64_t c[LOD_MAX_NDIM], nx[LOD_MAX_NDIM];
    uint64_t r = j;
    for (int d = 0; d < ndim; ++d) { /* dim 0 fastest, as unravel() */
      c[d] = r % parent[d];
      r /= parent[d];
    }
    const uint64_t pos = oracle_morton_rank(ndim, parent, c, 0);
    memcpy(nx, c, (size_t)ndim * sizeof(uint64_t));
    morton_successor(ndim, p, nx);
    ends[pos] = oracle_morton_rank(ndim, child, nx, 1);
  }
}

/* ------------------------------------------------------------------ */
/* Plan (src/stream/config.c:84-376, src/lod/lod_plan.c:151-345,        */
/*       src/stream/types.aggregate.c:65-143)                          */
/* ------------------------------------------------------------------ */

struct o_level
{
  uint64_t shape[HALF_MAX_RANK]; /* epoch-split shape at this level */
  uint64_t lod_nelem;
  struct tile_stream_layout lay;
  uint64_t chunk_offset;
  /* aggregate layout */
  uint8_t agg_rank;
  uint64_t agg_shape[MAX_RANK];
  int64_t agg_strides[MAX_RANK];
  uint64_t covering;
  uint64_t cps_inner;
  uint64_t cps_append;
  uint64_t cps_total;
  uint64_t shard_inner_count;
  uint32_t batch_active;
};

struct o_plan
{
  uint8_t rank, na;
  int append_downsample;
  uint32_t lod_mask;
  uint8_t order[HALF_MAX_RANK]; /* storage position -> dim */
  int nlod;
  int multiscale;
  int lod_ndim;
  int lod_to_dim[LOD_MAX_NDIM];
  int fixed_ndim;
  int fixed_to_dim[LOD_MAX_NDIM];
  uint64_t fixed_shape[LOD_MAX_NDIM];
  uint64_t fixed_count;
  uint64_t lod_end[LOD_MAX_LEVELS];   /* cumulative lod_nelem */
  uint64_t level_end[LOD_MAX_LEVELS]; /* fixed_count * lod_end */
  uint64_t* ends;                     /* window ends for levels >= 1 */
  struct o_level lv[LOD_MAX_LEVELS];
  uint64_t total_chunks;
  uint32_t K;
  uint64_t max_out;
};

static uint64_t
o_lz4_bound(uint64_t n)
{
  return n + n / 255 + 16;
}

static uint64_t
o_zstd_bound(uint64_t n)
{
  const uint64_t lim = 128u << 10;
  return n + (n >> 8) + (n < lim ? (lim - n) >> 11 : 0);
}

/* Lifted shape/strides of one level (src/stream/config.c:84-138 with
 * src/util/index.ops.c:97-113). */
static void
o_level_layout(struct tile_stream_layout* L,
               const struct o_plan* P,
               const struct dimension* dims,
               const uint64_t* shape,
               uint64_t bpe)
{
  const int rank = P->rank;
  uint64_t cc[HALF_MAX_RANK];
  memset(L, 0, sizeof(*L));
  L->lifted_rank = (uint8_t)(2 * rank);
  L->chunk_elements = 1;
  for (int i = 0; i < rank; ++i) {
    cc[i] = shape[i] == 0 ? 1 : cdiv(shape[i], dims[i].chunk_size);
    L->lifted_shape[2 * i] = cc[i];
    L->lifted_shape[2 * i + 1] = dims[i].chunk_size;
    L->chunk_elements *= dims[i].chunk_size;
  }
  L->chunk_stride = aup(L->chunk_elements * bpe, 1) / bpe;
  int64_t inner = 1, outer = (int64_t)L->chunk_stride;
  for (int j = rank - 1; j >= 0; --j) {
    const int i = P->order[j];
    L->lifted_strides[2 * i + 1] = inner;
    inner *= (int64_t)dims[i].chunk_size;
    L->lifted_strides[2 * i] = outer;
    outer *= (int64_t)cc[i];
  }
  L->chunks_per_epoch = 1;
  for (int d = P->na; d < rank; ++d)
    L->chunks_per_epoch *= cc[d];
  L->epoch_elements = L->chunks_per_epoch * L->chunk_elements;
  for (int d = 0; d < P->na; ++d)
    L->lifted_strides[2 * d] = 0;
  L->chunk_pool_bytes = L->chunks_per_epoch * L->chunk_stride * bpe;
}

static int
o_plan_init(struct o_plan* P, const struct tile_stream_configuration* cfg)
{
  memset(P, 0, sizeof(*P));
  const struct dimension* dims = cfg->dimensions;
  const uint8_t rank = cfg->rank;
  const uint64_t bpe = dtype_bpe(cfg->dtype);
  if (!bpe || !cfg->buffer_capacity_bytes || rank == 0 ||
      rank > HALF_MAX_RANK || !dims || cfg->max_threads < 0)
    return 1;
  if (!o_dims_ok(dims, rank))
    return 1;
  if (cfg->codec.id == CODEC_LZ4_NON_STANDARD && cfg->codec.level == 0)
    return 1;
  if ((cfg->codec.id == CODEC_BLOSC_LZ4 || cfg->codec.id == CODEC_BLOSC_ZSTD))
    return 1; /* blosc is not part of this path */
  if (cfg->max_nlod < 0 || cfg->max_nlod > LOD_MAX_LEVELS)
    return 1;
  P->rank = rank;
  P->na = o_n_append(dims, rank);
  for (int d = 0; d < rank; ++d)
    P->order[dims[d].storage_position] = (uint8_t)d;
  for (int d = P->na; d < rank; ++d)
    if (dims[d].downsample)
      P->lod_mask |= 1u << d;
  P->append_downsample = dims[P->na - 1].downsample ? 1 : 0;
  if (P->append_downsample) {
    const enum lod_reduce_method m = cfg->append_reduce_method;
    if (m != lod_reduce_mean && m != lod_reduce_min && m != lod_reduce_max)
      return 1;
    if (!P->lod_mask)
      return 1;
  }

  /* LOD plan on the epoch-split shape (src/lod/lod_plan.c:151-275,
   * 296-345). */
  uint64_t shape0[HALF_MAX_RANK];
  for (int d = 0; d < rank; ++d)
    shape0[d] = dims[d].size == 0 ? dims[d].chunk_size : dims[d].size;
  for (int d = 0; d < P->na; ++d)
    shape0[d] = dims[d].chunk_size;
  P->fixed_count = 1;
  for (int d = 0; d < rank; ++d) {
    if (P->lod_mask & (1u << d))
      P->lod_to_dim[P->lod_ndim++] = d;
    else {
      P->fixed_to_dim[P->fixed_ndim] = d;
      P->fixed_shape[P->fixed_ndim++] = shape0[d];
      P->fixed_count *= shape0[d];
    }
  }
  const int max_levels = cfg->max_nlod == 0 ? LOD_MAX_LEVELS : cfg->max_nlod;
  memcpy(P->lv[0].shape, shape0, sizeof(shape0));
  int nlod = 1;
  for (;;) {
    int all_one = 1;
    for (int k = 0; k < P->lod_ndim; ++k) {
      const int d = P->lod_to_dim[k];
      if (cdiv(P->lv[nlod - 1].shape[d], dims[d].chunk_size) > 1)
        all_one = 0;
    }
    if (nlod >= max_levels || all_one)
      break;
    memcpy(P->lv[nlod].shape, P->lv[nlod - 1].shape, sizeof(shape0));
    for (int k = 0; k < P->lod_ndim; ++k) {
      const int d = P->lod_to_dim[k];
      P->lv[nlod].shape[d] = (P->lv[nlod - 1].shape[d] + 1) / 2;
    }
    ++nlod;
  }
  P->multiscale = P->lod_mask != 0;
  P->nlod = P->multiscale ? nlod : 1;
  for (int l = 0; l < nlod; ++l) {
    P->lv[l].lod_nelem = 1;
    for (int k = 0; k < P->lod_ndim; ++k)
      P->lv[l].lod_nelem *= P->lv[l].shape[P->lod_to_dim[k]];
    P->lod_end[l] = (l ? P->lod_end[l - 1] : 0) + P->lv[l].lod_nelem;
    P->level_end[l] = P->fixed_count * P->lod_end[l];
  }
  if (P->multiscale && nlod > 1) {
    const uint64_t n = P->lod_end[nlod - 1] - P->lod_end[0];
    P->ends = (uint64_t*)malloc(n * sizeof(uint64_t));
    if (!P->ends)
      return 1;
    for (int l = 0; l + 1 < nlod; ++l) {
      uint64_t child[LOD_MAX_NDIM], parent[LOD_MAX_NDIM];
      for (int k = 0; k < P->lod_ndim; ++k) {
        child[k] = P->lv[l].shape[P->lod_to_dim[k]];
        parent[k] = P->lv[l + 1].shape[P->lod_to_dim[k]];
      }
      fill_window_ends(P->lod_ndim,
                       child,
                       parent,
                       P->lv[l + 1].lod_nelem,
                       P->ends + (P->lod_end[l] - P->lod_end[0]));
    }
  }

  /* Level layouts and geometry. */
  for (int l = 0; l < P->nlod; ++l) {
    o_level_layout(&P->lv[l].lay, P, dims, P->lv[l].shape, bpe);
    P->lv[l].chunk_offset = P->total_chunks;
    P->total_chunks += P->lv[l].lay.chunks_per_epoch;
  }
  if (P->lv[0].lay.chunks_per_epoch == 0 ||
      P->lv[0].lay.chunk_elements > UINT64_MAX / P->lv[0].lay.chunks_per_epoch)
    return 1;

  /* K (src/stream/config.c:31-45). */
  uint32_t K = cfg->epochs_per_batch;
  if (K == 0) {
    uint32_t target = cfg->target_batch_chunks ? cfg->target_batch_chunks : 1024;
    uint64_t k = cdiv(target, P->total_chunks);
    uint32_t p2 = 1;
    while (p2 < k)
      p2 <<= 1;
    K = p2;
  }
  if (K > MAX_BATCH_EPOCHS)
    K = MAX_BATCH_EPOCHS;
  P->K = K;

  const uint64_t chunk_bytes = P->lv[0].lay.chunk_stride * bpe;
  switch (cfg->codec.id) {
    case CODEC_NONE:
      P->max_out = chunk_bytes;
      break;
    case CODEC_LZ4_NON_STANDARD:
      P->max_out = o_lz4_bound(chunk_bytes);
      break;
    case CODEC_ZSTD:
      P->max_out = o_zstd_bound(chunk_bytes);
      break;
    default:
      return 1;
  }

  /* Per-level shard geometry (src/stream/config.c:298-373,
   * src/lod/lod_plan.c:347-370, src/stream/types.aggregate.c:65-143). */
  for (int l = 0; l < P->nlod; ++l) {
    struct o_level* L = &P->lv[l];
    uint64_t cc[HALF_MAX_RANK], cps[HALF_MAX_RANK], sc[HALF_MAX_RANK];
    for (int d = 0; d < rank; ++d) {
      const uint64_t s = l == 0 ? dims[d].size : L->shape[d];
      cc[d] = s == 0 ? 1 : cdiv(s, dims[d].chunk_size);
      uint64_t c = dims[d].chunks_per_shard;
      if (c == 0)
        c = cc[d];
      if (s > 0 && cc[d] < c)
        c = cc[d];
      cps[d] = c;
      sc[d] = cdiv(cc[d], c);
    }
    L->shard_inner_count = 1;
    for (int d = P->na; d < rank; ++d)
      L->shard_inner_count *= sc[d];
    L->batch_active = K;
    if (P->append_downsample && l > 0)
      L->batch_active = K >= (1u << l) ? K >> l : 0;

    /* aggregate layout over storage-ordered inner dims */
    L->agg_rank = (uint8_t)(2 * (rank - P->na));
    L->covering = 1;
    L->cps_inner = 1;
    uint64_t so_sc[HALF_MAX_RANK], so_cps[HALF_MAX_RANK];
    for (int j = P->na; j < rank; ++j) {
      const int d = P->order[j];
      so_cps[j] = cps[d];
      so_sc[j] = cdiv(cc[d], cps[d]);
      const int k = j - P->na;
      L->agg_shape[2 * k] = so_sc[j];
      L->agg_shape[2 * k + 1] = so_cps[j];
      L->covering *= so_sc[j] * so_cps[j];
      L->cps_inner *= so_cps[j];
    }
    if (L->covering > UINT32_MAX)
      return 1;
    uint64_t acc = 1;
    for (int j = rank - 1; j >= P->na; --j) {
      const int k = j - P->na;
      L->agg_strides[2 * k] = (int64_t)(acc * L->cps_inner);
      acc *= so_sc[j];
    }
    acc = 1;
    for (int j = rank - 1; j >= P->na; --j) {
      const int k = j - P->na;
      L->agg_strides[2 * k + 1] = (int64_t)acc;
      acc *= so_cps[j];
    }
    uint64_t ca = 1;
    for (int d = 0; d < P->na; ++d)
      ca *= cps[d];
    if (P->append_downsample && l > 0) {
      const uint64_t div = 1ull << l;
      ca = ca > div ? ca / div : 1;
    }
    L->cps_append = ca;
    L->cps_total = ca * L->cps_inner;
  }
  return 0;
}

/* Row-major ravel of idx over `shape` through `strides`
 * (src/util/index.ops.c:33-44). */
static uint64_t
o_ravel(int rank, const uint64_t* shape, const int64_t* strides, uint64_t idx)
{
  uint64_t o = 0;
  for (int d = rank - 1; d >= 0; --d) {
    o += (idx % shape[d]) * (uint64_t)strides[d];
    idx /= shape[d];
  }
  return o;
}

/* ------------------------------------------------------------------ */
/* LOD arithmetic (src/cpu/lod.cpp:55-127, 366-438; f16 follows        */
/* src/gpu/lod.cu:414-528, 828-941)                                    */
/* ------------------------------------------------------------------ */

#define O_FOR_TYPES(X)                                                         \
  X(dtype_u8, uint8_t, uint32_t, 1)                                            \
  X(dtype_u16, uint16_t, uint32_t, 1)                                          \
  X(dtype_u32, uint32_t, uint64_t, 1)                                          \
  X(dtype_u64, uint64_t, uint64_t, 2)                                          \
  X(dtype_i8, int8_t, int32_t, 1)                                              \
  X(dtype_i16, int16_t, int32_t, 1)                                            \
  X(dtype_i32, int32_t, int64_t, 1)                                            \
  X(dtype_i64, int64_t, int64_t, 2)                                            \
  X(dtype_f16, f16, float, 0)                                                  \
  X(dtype_f32, float, float, 0)                                                \
  X(dtype_f64, double, double, 0)

/* kind: 0 = float, 1 = narrow int (shifted mean fold), 2 = 64-bit int */
#define O_REDUCE(D, T, A, KIND)                                                \
  static T reduce_##D(const T* s, uint64_t a, uint64_t b, int m)               \
  {                                                                            \
    const uint64_t len = b - a;                                                \
    switch (m) {                                                               \
      case lod_reduce_mean: {                                                  \
        A sum = 0;                                                             \
        for (uint64_t j = a; j < b; ++j)                                       \
          sum += (A)s[j];                                                      \
        return (T)(sum / (A)len);                                              \
      }                                                                        \
      case lod_reduce_min: {                                                   \
        T v = s[a];                                                            \
        for (uint64_t j = a + 1; j < b; ++j)                                   \
          if (s[j] < v)                                                        \
            v = s[j];                                                          \
        return v;                                                              \
      }                                                                        \
      case lod_reduce_max: {                                                   \
        T v = s[a];                                                            \
        for (uint64_t j = a + 1; j < b; ++j)                                   \
          if (s[j] > v)                                                        \
            v = s[j];                                                          \
        return v;                                                              \
      }                                                                        \
      case lod_reduce_median: {                                                \
        T buf[16];                                                             \
        const uint64_t n = len <= 16 ? len : 16;                               \
        for (uint64_t j = 0; j < n; ++j)                                       \
          buf[j] = s[a + j];                                                   \
        for (uint64_t i = 1; i < n; ++i) {                                     \
          T key = buf[i];                                                      \
          uint64_t k = i;                                                      \
          while (k > 0 && buf[k - 1] > key) {                                  \
            buf[k] = buf[k - 1];                                               \
            --k;                                                               \
          }                                                                    \
          buf[k] = key;                                                        \
        }                                                                      \
        return buf[n / 2];                                                     \
      }                                                                        \
      case lod_reduce_max_suppressed: {                                        \
        T t1 = s[a], t2 = s[a];                                                \
        for (uint64_t j = a + 1; j < b; ++j) {                                 \
          const T v = s[j];                                                    \
          if (v >= t1) {                                                       \
            t2 = t1;                                                           \
            t1 = v;                                                            \
          } else if (v > t2)                                                   \
            t2 = v;                                                            \
        }                                                                      \
        return t2;                                                             \
      }                                                                        \
      case lod_reduce_min_suppressed: {                                        \
        T t1 = s[a], t2 = s[a];                                                \
        for (uint64_t j = a + 1; j < b; ++j) {                                 \
          const T v = s[j];                                                    \
          if (v <= t1) {                                                       \
            t2 = t1;                                                           \
            t1 = v;                                                            \
          } else if (v < t2)                                                   \
            t2 = v;                                                            \
        }                                                                      \
        return t2;                                                             \
      }                                                                        \
    }                                                                          \
    return (T)0;                                                               \
  }                                                                            \
  static void fold_##D(T* acc, const T* x, uint64_t n, uint32_t count,         \
                       int level, int m)                                       \
  {                                                                            \
    if (count == 0) {                                                          \
      memcpy(acc, x, n * sizeof(T));                                           \
      return;                                                                  \
    }                                                                          \
    for (uint64_t i = 0; i < n; ++i) {                                         \
      if (m == lod_reduce_mean) {                                              \
        acc[i] = addsh_##D(acc[i], x[i], level);                               \
      } else if (m == lod_reduce_min) {                                        \
        if (x[i] < acc[i])                                                     \
          acc[i] = x[i];                                                       \
      } else if (m == lod_reduce_max) {                                        \
        if (x[i] > acc[i])                                                     \
          acc[i] = x[i];                                                       \
      }                                                                        \
    }                                                                          \
  }                                                                            \
  static void emit_##D(T* dst, const T* acc, uint64_t n, uint32_t count,       \
                       int m)                                                  \
  {                                                                            \
    if (KIND == 0 && m == lod_reduce_mean) {                                   \
      for (uint64_t i = 0; i < n; ++i)                                         \
        dst[i] = (T)((A)acc[i] / (A)count);                                    \
      return;                                                                  \
    }                                                                          \
    memcpy(dst, acc, n * sizeof(T));                                           \
  }

/* Overflow-safe (a + b) >> s for 8..32-bit integers, plain a + b for floats
 * and 64-bit integers (src/cpu/lod.cpp:366-378).  Narrow operands promote
 * to int exactly as in the C++ reference. */
#define O_ADDSH_INT(D, T)                                                      \
  static inline T addsh_##D(T a, T b, int s)                                   \
  {                                                                            \
    const T mask = (T)((1u << s) - 1);                                         \
    return (T)((a >> s) + (b >> s) + (((a & mask) + (b & mask)) >> s));        \
  }
#define O_ADDSH_SUM(D, T)                                                      \
  static inline T addsh_##D(T a, T b, int s)                                   \
  {                                                                            \
    (void)s;                                                                   \
    return (T)(a + b);                                                         \
  }
O_ADDSH_INT(dtype_u8, uint8_t)
O_ADDSH_INT(dtype_u16, uint16_t)
O_ADDSH_INT(dtype_u32, uint32_t)
O_ADDSH_INT(dtype_i8, int8_t)
O_ADDSH_INT(dtype_i16, int16_t)
O_ADDSH_INT(dtype_i32, int32_t)
O_ADDSH_SUM(dtype_u64, uint64_t)
O_ADDSH_SUM(dtype_i64, int64_t)
O_ADDSH_SUM(dtype_f16, f16)
O_ADDSH_SUM(dtype_f32, float)
O_ADDSH_SUM(dtype_f64, double)

#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wshift-count-overflow"
#pragma GCC diagnostic ignored "-Wint-in-bool-context"
O_FOR_TYPES(O_REDUCE)
#pragma GCC diagnostic pop

/* ------------------------------------------------------------------ */
/* Stream (src/cpu/stream.c, src/cpu/pipeline.c, src/cpu/aggregate.c,   */
/*         src/zarr/shard_delivery.c)                                  */
/* ------------------------------------------------------------------ */

struct o_shard
{
  uint64_t cursor;
  uint64_t* index;
  struct shard_writer* w;
};

struct o_shards
{
  uint64_t epoch_in_shard, shard_epoch;
  struct o_shard* sh;
};

struct oracle_stream
{
  struct writer writer;
  struct tile_stream_configuration cfg;
  struct shard_sink* sink;
  struct o_plan P;
  uint64_t bpe;
  uint8_t* pool;    /* [K][total_chunks][chunk_stride] */
  uint8_t* comp;    /* [K][total_chunks][max_out] */
  uint64_t* csize;  /* [K*total_chunks] */
  uint8_t* linear;  /* one epoch, row-major */
  uint8_t* values;  /* all levels in Morton order */
  uint8_t* accum;   /* dim-0 accumulators for levels >= 1 */
  uint32_t counts[LOD_MAX_LEVELS];
  uint32_t* scatter_lut;
  uint64_t* scatter_fixed;
  uint32_t* chunk_lut[LOD_MAX_LEVELS];
  uint64_t* chunk_fixed[LOD_MAX_LEVELS];
  struct o_shards shards[LOD_MAX_LEVELS];
  struct io_event io_done[LOD_MAX_LEVELS];
  uint64_t cursor, max_cursor;
  uint32_t accumulated;
  uint32_t masks[MAX_BATCH_EPOCHS];
  int flushed;
  int nthreads;
};

static void*
o_stream_free(struct oracle_stream* s)
{
  if (!s)
    return NULL;
  for (int l = 0; l < LOD_MAX_LEVELS; ++l) {
    free(s->chunk_lut[l]);
    free(s->chunk_fixed[l]);
    if (s->shards[l].sh) {
      for (uint64_t i = 0; i < s->P.lv[l].shard_inner_count; ++i)
        free(s->shards[l].sh[i].index);
      free(s->shards[l].sh);
    }
  }
  free(s->pool);
  free(s->comp);
  free(s->csize);
  free(s->linear);
  free(s->values);
  free(s->accum);
  free(s->scatter_lut);
  free(s->scatter_fixed);
  free(s->P.ends);
  free(s);
  return NULL;
}

static struct writer_result o_append(struct writer* self, struct slice in);
static struct writer_result o_flush_final(struct writer* self);

#define O_SELF(w) ((struct oracle_stream*)(w))

struct oracle_stream*
oracle_stream_create(const struct tile_stream_configuration* cfg,
                     struct shard_sink* sink)
{
  if (!cfg || !sink)
    return NULL;
  struct oracle_stream* s =
    (struct oracle_stream*)calloc(1, sizeof(struct oracle_stream));
  if (!s)
    return NULL;
  s->cfg = *cfg;
  s->sink = sink;
  s->bpe = dtype_bpe(cfg->dtype);
#ifdef _OPENMP
  s->nthreads = cfg->max_threads > 0 ? cfg->max_threads : omp_get_max_threads();
#else
  s->nthreads = 1;
#endif
  if (o_plan_init(&s->P, cfg))
    return o_stream_free(s);
  struct o_plan* P = &s->P;
  const uint64_t stride_b = P->lv[0].lay.chunk_stride * s->bpe;
  const uint64_t slots = (uint64_t)P->K * P->total_chunks;
  s->pool = (uint8_t*)calloc(slots, stride_b);
  s->comp = (uint8_t*)malloc(slots * P->max_out);
  s->csize = (uint64_t*)calloc(slots, sizeof(uint64_t));
  if (!s->pool || !s->comp || !s->csize)
    return o_stream_free(s);
  for (int l = 0; l < P->nlod; ++l) {
    const uint64_t n = P->lv[l].shard_inner_count;
    const uint64_t ni = P->lv[l].cps_total * 2;
    s->shards[l].sh = (struct o_shard*)calloc(n, sizeof(struct o_shard));
    if (!s->shards[l].sh)
      return o_stream_free(s);
    for (uint64_t i = 0; i < n; ++i) {
      s->shards[l].sh[i].index = (uint64_t*)malloc(ni * sizeof(uint64_t));
      if (!s->shards[l].sh[i].index)
        return o_stream_free(s);
      memset(s->shards[l].sh[i].index, 0xFF, ni * sizeof(uint64_t));
    }
  }
  if (P->multiscale) {
    const uint64_t bpe = s->bpe;
    s->linear = (uint8_t*)calloc(P->lv[0].lay.epoch_elements, bpe);
    s->values = (uint8_t*)calloc(P->level_end[P->nlod - 1], bpe);
    if (!s->linear || !s->values)
      return o_stream_free(s);
    if (P->append_downsample) {
      uint64_t n = 0;
      for (int l = 1; l < P->nlod; ++l)
        n += P->fixed_count * P->lv[l].lod_nelem;
      if (n) {
        s->accum = (uint8_t*)calloc(n, bpe);
        if (!s->accum)
          return o_stream_free(s);
      }
    }
    /* L0 gather LUT (src/cpu/lod.cpp:181-239). */
    const uint64_t n0 = P->lv[0].lod_nelem;
    s->scatter_lut = (uint32_t*)malloc(n0 * sizeof(uint32_t));
    s->scatter_fixed = (uint64_t*)calloc(P->fixed_count, sizeof(uint64_t));
    if (!s->scatter_lut || !s->scatter_fixed)
      return o_stream_free(s);
    uint64_t full_stride[HALF_MAX_RANK];
    full_stride[P->rank - 1] = 1;
    for (int d = P->rank - 2; d >= 0; --d)
      full_stride[d] = full_stride[d + 1] * P->lv[0].shape[d + 1];
    uint64_t lshape[LOD_MAX_NDIM];
    for (int k = 0; k < P->lod_ndim; ++k)
      lshape[k] = P->lv[0].shape[P->lod_to_dim[k]];
    for (uint64_t g = 0; g < n0; ++g) {
      uint64_t c[LOD_MAX_NDIM], r = g, off = 0;
      for (int k = P->lod_ndim - 1; k >= 0; --k) {
        c[k] = r % lshape[k];
        r /= lshape[k];
        off += c[k] * full_stride[P->lod_to_dim[k]];
      }
      s->scatter_lut[oracle_morton_rank(P->lod_ndim, lshape, c, 0)] =
        (uint32_t)off;
    }
    for (uint64_t b = 0; b < P->fixed_count; ++b) {
      uint64_t r = b, off = 0;
      for (int k = P->fixed_ndim - 1; k >= 0; --k) {
        off += (r % P->fixed_shape[k]) * full_stride[P->fixed_to_dim[k]];
        r /= P->fixed_shape[k];
      }
      s->scatter_fixed[b] = off;
    }
    /* Morton -> chunk LUTs per level (src/cpu/lod.cpp:318-352,
     * src/cpu/pipeline.c:373-398). */
    for (int l = 0; l < P->nlod; ++l) {
      const struct tile_stream_layout* L = &P->lv[l].lay;
      const uint64_t n = P->lv[l].lod_nelem;
      s->chunk_lut[l] = (uint32_t*)malloc(n * sizeof(uint32_t));
      s->chunk_fixed[l] = (uint64_t*)calloc(P->fixed_count, sizeof(uint64_t));
      if (!s->chunk_lut[l] || !s->chunk_fixed[l])
        return o_stream_free(s);
      uint64_t ls[LOD_MAX_NDIM];
      for (int k = 0; k < P->lod_ndim; ++k)
        ls[k] = P->lv[l].shape[P->lod_to_dim[k]];
      for (uint64_t g = 0; g < n; ++g) {
        uint64_t c[LOD_MAX_NDIM], r = g;
        int64_t off = 0;
        for (int k = P->lod_ndim - 1; k >= 0; --k) {
          c[k] = r % ls[k];
          r /= ls[k];
          const int d = P->lod_to_dim[k];
          const uint64_t cs = L->lifted_shape[2 * d + 1];
          off += (int64_t)(c[k] / cs) * L->lifted_strides[2 * d];
          off += (int64_t)(c[k] % cs) * L->lifted_strides[2 * d + 1];
        }
        s->chunk_lut[l][oracle_morton_rank(P->lod_ndim, ls, c, 0)] =
          (uint32_t)off;
      }
      for (uint64_t b = 0; b < P->fixed_count; ++b) {
        uint64_t r = b;
        int64_t off = 0;
        for (int k = P->fixed_ndim - 1; k >= 0; --k) {
          const uint64_t coord = r % P->fixed_shape[k];
          r /= P->fixed_shape[k];
          const int d = P->fixed_to_dim[k];
          const uint64_t cs = L->lifted_shape[2 * d + 1];
          off += (int64_t)(coord / cs) * L->lifted_strides[2 * d];
          off += (int64_t)(coord % cs) * L->lifted_strides[2 * d + 1];
        }
        s->chunk_fixed[l][b] =
          (uint64_t)off + P->lv[l].chunk_offset * L->chunk_stride;
      }
    }
  }
  {
    const struct dimension* dims = cfg->dimensions;
    if (dims[0].size > 0) {
      s->max_cursor = P->lv[0].lay.epoch_elements;
      for (int d = 0; d < P->na; ++d)
        s->max_cursor *= cdiv(dims[d].size, dims[d].chunk_size);
    }
  }
  s->writer.append = o_append;
  s->writer.flush = o_flush_final;
  return s;
}

void
oracle_stream_destroy(struct oracle_stream* s)
{
  o_stream_free(s);
}

struct writer*
oracle_stream_writer(struct oracle_stream* s)
{
  return &s->writer;
}

uint64_t
oracle_stream_cursor(const struct oracle_stream* s)
{
  return s->cursor;
}

const struct tile_stream_layout*
oracle_stream_layout(const struct oracle_stream* s)
{
  return &s->P.lv[0].lay;
}

int
oracle_stream_info(const struct oracle_stream* s, struct oracle_info* info)
{
  memset(info, 0, sizeof(*info));
  info->nlod = s->P.nlod;
  info->append_downsample = s->P.append_downsample;
  info->epochs_per_batch = s->P.K;
  info->total_chunks = s->P.total_chunks;
  info->chunk_elements = s->P.lv[0].lay.chunk_elements;
  info->epoch_elements = s->P.lv[0].lay.epoch_elements;
  info->max_output_size = s->P.max_out;
  info->fixed_dims_count = s->P.fixed_count;
  for (int l = 0; l < s->P.nlod; ++l) {
    info->lod_nelem[l] = s->P.lv[l].lod_nelem;
    info->level_chunks[l] = s->P.lv[l].lay.chunks_per_epoch;
    info->shard_inner_count[l] = s->P.lv[l].shard_inner_count;
    info->chunks_per_shard_total[l] = s->P.lv[l].cps_total;
    info->chunks_per_shard_append[l] = s->P.lv[l].cps_append;
  }
  return 0;
}

/* Scatter `n` stream elements starting at global index i0 into an epoch
 * slot of the chunk pool (src/cpu/transpose.cpp:10-105). */
static void
o_transpose(uint8_t* dst,
            const uint8_t* src,
            uint64_t n,
            uint64_t bpe,
            uint64_t i0,
            const struct tile_stream_layout* L)
{
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t o =
      o_ravel(L->lifted_rank, L->lifted_shape, L->lifted_strides, i0 + i);
    memcpy(dst + o * bpe, src + i * bpe, bpe);
  }
}

static uint8_t*
epoch_slot(struct oracle_stream* s, uint32_t e)
{
  return s->pool +
         (uint64_t)e * s->P.total_chunks * s->P.lv[0].lay.chunk_stride * s->bpe;
}

static void
o_morton_to_chunks(struct oracle_stream* s, uint8_t* slot, int l)
{
  const struct o_plan* P = &s->P;
  const uint64_t bpe = s->bpe, n = P->lv[l].lod_nelem;
  const uint8_t* v = s->values + (l ? P->level_end[l - 1] : 0) * bpe;
  for (uint64_t b = 0; b < P->fixed_count; ++b)
    for (uint64_t i = 0; i < n; ++i)
      memcpy(slot + (s->chunk_fixed[l][b] + s->chunk_lut[l][i]) * bpe,
             v + (b * n + i) * bpe,
             bpe);
}

static int
o_fold_dispatch(void* acc, const void* x, uint64_t n, uint32_t count, int level,
                enum dtype dt, int m)
{
  switch (dt) {
#define X(D, T, A, K)                                                          \
  case D:                                                                      \
    fold_##D((T*)acc, (const T*)x, n, count, level, m);                        \
    return 0;
    O_FOR_TYPES(X)
#undef X
  }
  return 1;
}

static int
o_emit_dispatch(void* dst, const void* acc, uint64_t n, uint32_t count,
                enum dtype dt, int m)
{
  switch (dt) {
#define X(D, T, A, K)                                                          \
  case D:                                                                      \
    emit_##D((T*)dst, (const T*)acc, n, count, m);                             \
    return 0;
    O_FOR_TYPES(X)
#undef X
  }
  return 1;
}

static uint64_t
accum_offset(const struct o_plan* P, int lv)
{
  uint64_t o = 0;
  for (int k = 1; k < lv; ++k)
    o += P->fixed_count * P->lv[k].lod_nelem;
  return o;
}

/* One epoch of the LOD pipeline (src/cpu/pipeline.c:195-336). */
static int
o_lod_epoch(struct oracle_stream* s, uint32_t e, uint32_t* mask)
{
  struct o_plan* P = &s->P;
  const uint64_t bpe = s->bpe;
  const uint64_t n0 = P->lv[0].lod_nelem;
  /* gather (src/cpu/lod.cpp:241-267) */
  for (uint64_t b = 0; b < P->fixed_count; ++b)
    for (uint64_t m = 0; m < n0; ++m)
      memcpy(s->values + (b * n0 + m) * bpe,
             s->linear + (s->scatter_fixed[b] + s->scatter_lut[m]) * bpe,
             bpe);
  /* reduce (src/cpu/lod.cpp:269-296) */
  for (int l = 0; l + 1 < P->nlod; ++l) {
    const uint64_t sn = P->lv[l].lod_nelem, dn = P->lv[l + 1].lod_nelem;
    const uint64_t sbeg = l ? P->level_end[l - 1] : 0;
    const uint64_t dbeg = P->level_end[l];
    const uint64_t* ends = P->ends + (P->lod_end[l] - P->lod_end[0]);
    for (uint64_t b = 0; b < P->fixed_count; ++b)
      for (uint64_t i = 0; i < dn; ++i) {
        const uint64_t a = i ? ends[i - 1] : 0, z = ends[i];
        if (oracle_reduce_window(s->values + (dbeg + b * dn + i) * bpe,
                                 s->values + (sbeg + b * sn + a) * bpe,
                                 z - a,
                                 s->cfg.dtype,
                                 s->cfg.reduce_method))
          return 1;
      }
  }
  uint32_t active = (P->append_downsample && s->accum)
                      ? 1u
                      : (uint32_t)((1ull << P->nlod) - 1);
  if (P->append_downsample && s->accum) {
    for (int l = 1; l < P->nlod; ++l) {
      const uint64_t n = P->fixed_count * P->lv[l].lod_nelem;
      if (o_fold_dispatch(s->accum + accum_offset(P, l) * bpe,
                          s->values + P->level_end[l - 1] * bpe,
                          n,
                          s->counts[l],
                          l,
                          s->cfg.dtype,
                          s->cfg.append_reduce_method))
        return 1;
    }
    for (int l = 1; l < P->nlod; ++l) {
      s->counts[l]++;
      if (s->counts[l] >= (1u << l)) {
        const uint64_t n = P->fixed_count * P->lv[l].lod_nelem;
        o_emit_dispatch(s->values + P->level_end[l - 1] * bpe,
                        s->accum + accum_offset(P, l) * bpe,
                        n,
                        s->counts[l],
                        s->cfg.dtype,
                        s->cfg.append_reduce_method);
        s->counts[l] = 0;
        active |= 1u << l;
      }
    }
  }
  uint8_t* slot = epoch_slot(s, e);
  for (int l = 0; l < P->nlod; ++l)
    if (active & (1u << l))
      o_morton_to_chunks(s, slot, l);
  *mask = active;
  return 0;
}

/* ---- codecs (dlopen'd stock libraries) ---- */

typedef size_t (*zstd_c_fn)(void*, size_t, const void*, size_t, int);
typedef size_t (*zstd_d_fn)(void*, size_t, const void*, size_t);
typedef unsigned (*zstd_err_fn)(size_t);
typedef int (*lz4hc_c_fn)(const char*, char*, int, int, int);
typedef int (*lz4_d_fn)(const char*, char*, int, int);

static struct
{
  pthread_once_t once;
  zstd_c_fn zc;
  zstd_d_fn zd;
  zstd_err_fn ze;
  lz4hc_c_fn lc;
  lz4_d_fn ld;
} g_codec = { PTHREAD_ONCE_INIT, 0, 0, 0, 0, 0 };

static void
codec_load(void)
{
  void* z = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL);
  if (z) {
    g_codec.zc = (zstd_c_fn)dlsym(z, "ZSTD_compress");
    g_codec.zd = (zstd_d_fn)dlsym(z, "ZSTD_decompress");
    g_codec.ze = (zstd_err_fn)dlsym(z, "ZSTD_isError");
  }
  void* l = dlopen("liblz4.so.1", RTLD_NOW | RTLD_LOCAL);
  if (l) {
    g_codec.lc = (lz4hc_c_fn)dlsym(l, "LZ4_compress_HC");
    g_codec.ld = (lz4_d_fn)dlsym(l, "LZ4_decompress_safe");
  }
}

int
oracle_codecs_available(void)
{
  pthread_once(&g_codec.once, codec_load);
  return (g_codec.zc && g_codec.zd && g_codec.ze ? 1 : 0) |
         (g_codec.lc && g_codec.ld ? 2 : 0);
}

size_t
oracle_zstd_decompress(void* dst, size_t cap, const void* src, size_t n)
{
  if (!(oracle_codecs_available() & 1))
    return (size_t)-1;
  const size_t r = g_codec.zd(dst, cap, src, n);
  return g_codec.ze(r) ? (size_t)-1 : r;
}

size_t
oracle_lz4_decompress(void* dst, size_t cap, const void* src, size_t n)
{
  if (!(oracle_codecs_available() & 2))
    return (size_t)-1;
  const int r = g_codec.ld((const char*)src, (char*)dst, (int)n, (int)cap);
  return r < 0 ? (size_t)-1 : (size_t)r;
}

/* src/cpu/compress.c:31-110 */
static int
o_compress(struct oracle_stream* s, uint64_t nchunks)
{
  const uint64_t in_stride = s->P.lv[0].lay.chunk_stride * s->bpe;
  const uint64_t chunk_bytes = s->P.lv[0].lay.chunk_elements * s->bpe;
  const uint64_t mo = s->P.max_out;
  const int lvl = s->cfg.codec.level;
  int err = 0;
  if (s->cfg.codec.id != CODEC_NONE && !oracle_codecs_available())
    return 1;
  int64_t i;
#pragma omp parallel for schedule(dynamic) num_threads(s->nthreads) reduction(| : err)
  for (i = 0; i < (int64_t)nchunks; ++i) {
    const uint8_t* in = s->pool + (uint64_t)i * in_stride;
    uint8_t* out = s->comp + (uint64_t)i * mo;
    switch (s->cfg.codec.id) {
      case CODEC_NONE:
        memcpy(out, in, chunk_bytes);
        s->csize[i] = chunk_bytes;
        break;
      case CODEC_LZ4_NON_STANDARD: {
        const int r = g_codec.lc(
          (const char*)in, (char*)out, (int)chunk_bytes, (int)mo, lvl);
        if (r <= 0)
          err |= 1;
        else
          s->csize[i] = (uint64_t)r;
        break;
      }
      case CODEC_ZSTD: {
        const size_t r = g_codec.zc(out, mo, in, chunk_bytes, lvl);
        if (g_codec.ze(r))
          err |= 1;
        else
          s->csize[i] = r;
        break;
      }
      default:
        err |= 1;
    }
  }
  return err;
}

/* crc32c, table driven (src/zarr/crc32c.c:5-28). */
static uint32_t g_crc_tab[256];
static pthread_once_t g_crc_once = PTHREAD_ONCE_INIT;
static void
crc_init(void)
{
  for (uint32_t i = 0; i < 256; ++i) {
    uint32_t c = i;
    for (int j = 0; j < 8; ++j)
      c = (c >> 1) ^ (0x82F63B78u & (0u - (c & 1)));
    g_crc_tab[i] = c;
  }
}

uint32_t
oracle_crc32c(const void* data, size_t len)
{
  pthread_once(&g_crc_once, crc_init);
  uint32_t c = 0xFFFFFFFFu;
  const uint8_t* p = (const uint8_t*)data;
  for (size_t i = 0; i < len; ++i)
    c = g_crc_tab[(c ^ p[i]) & 0xFF] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

/* Write index + crc and finalize every open shard of a level
 * (src/zarr/shard_delivery.c:36-102). */
static int
o_finalize(struct oracle_stream* s, int l)
{
  struct o_shards* ss = &s->shards[l];
  const struct o_level* L = &s->P.lv[l];
  const uint64_t sa = s->cfg.shard_alignment;
  int err = 0;
  for (uint64_t si = 0; si < L->shard_inner_count; ++si) {
    struct o_shard* sh = &ss->sh[si];
    if (!sh->w)
      continue;
    const uint64_t nidx = L->cps_total * 16;
    const uint64_t total = nidx + 4;
    const uint64_t wb = sa ? aup(total, sa) : total;
    const uint64_t pad = wb - total;
    uint8_t* buf = (uint8_t*)calloc(1, wb);
    if (!buf)
      return 1;
    memcpy(buf + pad, sh->index, nidx);
    const uint32_t crc = oracle_crc32c(buf + pad, nidx);
    memcpy(buf + pad + nidx, &crc, 4);
    if (sh->w->write(sh->w, sh->cursor, buf, buf + wb))
      err = 1;
    free(buf);
    if (sh->w->finalize(sh->w))
      err = 1;
    sh->w = NULL;
    sh->cursor = 0;
    memset(sh->index, 0xFF, nidx);
  }
  ss->epoch_in_shard = 0;
  ss->shard_epoch++;
  return err;
}

/* Aggregate one level of a batch in shard order and deliver it
 * (src/cpu/aggregate.c:130-188, src/stream/types.aggregate.c:28-62,
 *  src/zarr/shard_delivery.c:105-204). */
static int
o_aggregate_deliver(struct oracle_stream* s,
                    int l,
                    uint32_t n_active,
                    const uint32_t* pool_epochs)
{
  const struct o_level* L = &s->P.lv[l];
  const uint64_t M = L->lay.chunks_per_epoch, C = L->covering;
  const uint64_t cpi = L->cps_inner;
  const uint64_t nsh = C / cpi;
  const uint64_t bM = (uint64_t)n_active * M, bC = (uint64_t)n_active * C;
  const uint64_t mo = s->P.max_out;
  const uint64_t sa = s->cfg.shard_alignment;
  uint32_t* gather = (uint32_t*)malloc((bM + 1) * sizeof(uint32_t));
  uint32_t* perm = (uint32_t*)malloc((bM + 1) * sizeof(uint32_t));
  uint64_t* sizes = (uint64_t*)calloc(bC + 1, sizeof(uint64_t));
  uint64_t* real = (uint64_t*)calloc(bC + 1, sizeof(uint64_t));
  uint64_t* off = (uint64_t*)calloc(bC + 1, sizeof(uint64_t));
  int rc = 1;
  uint8_t* data = NULL;
  if (!gather || !perm || !sizes || !real || !off)
    goto done;
  for (uint32_t a = 0; a < n_active; ++a)
    for (uint64_t j = 0; j < M; ++j) {
      const uint64_t i = (uint64_t)a * M + j;
      gather[i] =
        (uint32_t)(pool_epochs[a] * s->P.total_chunks + L->chunk_offset + j);
      const uint64_t pos = o_ravel(L->agg_rank, L->agg_shape, L->agg_strides, j);
      perm[i] = (uint32_t)(((pos / cpi) % nsh) * n_active * cpi + pos % cpi +
                           a * cpi);
    }
  for (uint64_t i = 0; i < bM; ++i)
    sizes[perm[i]] = s->csize[gather[i]];
  memcpy(real, sizes, bC * sizeof(uint64_t));
  if (sa > 0) {
    const uint64_t g = (uint64_t)n_active * cpi;
    for (uint64_t sh = 0; sh < bC / g; ++sh) {
      uint64_t t = 0;
      for (uint64_t j = 0; j < g; ++j)
        t += sizes[sh * g + j];
      const uint64_t pad = aup(t, sa) - t;
      sizes[sh * g + g - 1] += pad;
    }
  }
  for (uint64_t i = 0; i < bC; ++i)
    off[i + 1] = off[i] + sizes[i];
  /* the data buffer has alignment slack so aligned writes may read past
   * the last chunk (src/stream/types.aggregate.c:10-26) */
  data = (uint8_t*)calloc(1, off[bC] + (sa ? (nsh + 1) * sa : 0) + 1);
  if (!data)
    goto done;
  for (uint64_t i = 0; i < bM; ++i) {
    const uint64_t nb = s->csize[gather[i]];
    if (nb)
      memcpy(data + off[perm[i]], s->comp + (uint64_t)gather[i] * mo, nb);
  }
  /* deliver */
  {
    struct o_shards* ss = &s->shards[l];
    uint32_t a = 0;
    while (a < n_active) {
      const uint32_t left_shard = (uint32_t)(L->cps_append - ss->epoch_in_shard);
      const uint32_t left_batch = n_active - a;
      const uint32_t run = left_shard < left_batch ? left_shard : left_batch;
      for (uint64_t si = 0; si < L->shard_inner_count; ++si) {
        struct o_shard* sh = &ss->sh[si];
        if (!sh->w) {
          const uint64_t flat = ss->shard_epoch * L->shard_inner_count + si;
          sh->w = s->sink->open(s->sink, (uint8_t)l, flat);
          if (!sh->w)
            goto done;
        }
        const uint64_t j0 = si * n_active * cpi + (uint64_t)a * cpi;
        const uint64_t j1 = j0 + (uint64_t)run * cpi;
        const uint64_t bytes = off[j1] - off[j0];
        if (bytes > 0) {
          const uint8_t* src = data + off[j0];
          const uint64_t wb = sa ? aup(bytes, sa) : bytes;
          if (sh->w->write(sh->w, sh->cursor, src, src + wb))
            goto done;
        }
        for (uint32_t r = 0; r < run; ++r) {
          const uint64_t eis = ss->epoch_in_shard + r;
          const uint64_t js = j0 + (uint64_t)r * cpi;
          for (uint64_t j = js; j < js + cpi; ++j)
            if (real[j] > 0) {
              const uint64_t slot = eis * cpi + (j - js);
              sh->index[2 * slot] = sh->cursor + (off[j] - off[j0]);
              sh->index[2 * slot + 1] = real[j];
            }
        }
        sh->cursor += sa ? aup(bytes, sa) : bytes;
      }
      ss->epoch_in_shard += run;
      a += run;
      if (ss->epoch_in_shard >= L->cps_append)
        if (o_finalize(s, l))
          goto done;
    }
  }
  rc = 0;
done:
  free(gather);
  free(perm);
  free(sizes);
  free(real);
  free(off);
  free(data);
  return rc;
}

/* src/cpu/pipeline.c:113-190 */
static int
o_flush_batch(struct oracle_stream* s, uint32_t n, const uint32_t* masks)
{
  if (o_compress(s, (uint64_t)n * s->P.total_chunks))
    return 1;
  for (int l = 0; l < s->P.nlod; ++l) {
    uint32_t eps[MAX_BATCH_EPOCHS], na = 0;
    for (uint32_t e = 0; e < n; ++e)
      if (masks[e] & (1u << l))
        eps[na++] = e;
    if (!na)
      continue;
    if (s->sink->wait_fence)
      s->sink->wait_fence(s->sink, (uint8_t)l, s->io_done[l]);
    /* The reference keeps a LUT planned for pool epochs (a+1)*period-1 and
     * rebuilds it from the active epochs only when their count differs
     * (src/cpu/pipeline.c:14-31, 152-172).  The two agree except for the
     * final dim-0 drain when K equals the level's period; there the
     * reference reads the previous period's slot. */
    if (g_quirks && na == s->P.lv[l].batch_active) {
      const uint32_t period =
        (s->P.append_downsample && l > 0) ? (1u << l) : 1u;
      for (uint32_t a = 0; a < na; ++a)
        eps[a] = (a + 1) * period - 1;
    }
    if (o_aggregate_deliver(s, l, na, eps))
      return 1;
    if (s->sink->record_fence)
      s->io_done[l] = s->sink->record_fence(s->sink, (uint8_t)l);
  }
  return 0;
}

static int
o_epoch_done(struct oracle_stream* s)
{
  uint32_t mask = 1;
  if (s->P.multiscale && o_lod_epoch(s, s->accumulated, &mask))
    return 1;
  if (s->accumulated >= MAX_BATCH_EPOCHS)
    return 1;
  s->masks[s->accumulated++] = mask;
  return 0;
}

static struct writer_result
o_flush(struct oracle_stream* s);

/* src/cpu/stream.c:528-666 */
static struct writer_result
o_append(struct writer* self, struct slice in)
{
  struct oracle_stream* s = O_SELF(self);
  if (s->flushed)
    return writer_finished_at(in.beg, in.end);
  const uint64_t bpe = s->bpe;
  const uint64_t ee = s->P.lv[0].lay.epoch_elements;
  const uint8_t* src = (const uint8_t*)in.beg;
  const uint8_t* end = (const uint8_t*)in.end;
  while (src < end) {
    if (s->max_cursor > 0 && s->cursor >= s->max_cursor) {
      struct writer_result fr = o_flush(s);
      if (fr.error)
        return writer_error_at(src, end);
      return writer_finished_at(src, end);
    }
    const uint64_t rem_epoch = ee - s->cursor % ee;
    const uint64_t rem_in = (uint64_t)(end - src) / bpe;
    uint64_t n = rem_epoch < rem_in ? rem_epoch : rem_in;
    if (s->max_cursor > 0 && n > s->max_cursor - s->cursor)
      n = s->max_cursor - s->cursor;
    if (n == 0)
      break; /* trailing partial element */
    if (!g_quirks && s->cursor % ee == 0) {
      if (s->P.multiscale)
        memset(s->linear, 0, ee * bpe);
      else
        memset(epoch_slot(s, s->accumulated), 0,
               s->P.total_chunks * s->P.lv[0].lay.chunk_stride * bpe);
    }
    if (s->P.multiscale)
      memcpy(s->linear + (s->cursor % ee) * bpe, src, n * bpe);
    else
      o_transpose(epoch_slot(s, s->accumulated), src, n, bpe, s->cursor,
                  &s->P.lv[0].lay);
    s->cursor += n;
    src += n * bpe;
    if (s->cursor % ee == 0) {
      if (o_epoch_done(s))
        return writer_error_at(src, end);
      if (s->accumulated == s->P.K) {
        if (o_flush_batch(s, s->accumulated, s->masks))
          return writer_error_at(src, end);
        s->accumulated = 0;
        /* CPU chunk strides are never padded, so the reference never clears
         * the pool here (src/cpu/stream.c:623-629). */
      }
      if (s->values)
        memset(s->values, 0, s->P.level_end[s->P.nlod - 1] * bpe);
    }
  }
  return (struct writer_result){ 0, { src, end } };
}

/* src/cpu/stream.c:668-774 */
static struct writer_result
o_flush(struct oracle_stream* s)
{
  const uint64_t ee = s->P.lv[0].lay.epoch_elements;
  if (s->cursor % ee != 0)
    if (o_epoch_done(s))
      return writer_error();
  if (s->accumulated > 0) {
    if (o_flush_batch(s, s->accumulated, s->masks))
      return writer_error();
    s->accumulated = 0;
  }
  if (s->P.append_downsample && s->accum) {
    uint32_t drain = 0;
    for (int l = 1; l < s->P.nlod; ++l)
      if (s->counts[l] > 0) {
        const uint64_t n = s->P.fixed_count * s->P.lv[l].lod_nelem;
        o_emit_dispatch(s->values + s->P.level_end[l - 1] * s->bpe,
                        s->accum + accum_offset(&s->P, l) * s->bpe,
                        n,
                        s->counts[l],
                        s->cfg.dtype,
                        s->cfg.append_reduce_method);
        s->counts[l] = 0;
        o_morton_to_chunks(s, s->pool, l);
        drain |= 1u << l;
      }
    if (drain) {
      s->masks[0] = drain;
      if (o_flush_batch(s, 1, s->masks))
        return writer_error();
    }
  }
  for (int l = 0; l < s->P.nlod; ++l) {
    if (s->sink->wait_fence)
      s->sink->wait_fence(s->sink, (uint8_t)l, s->io_done[l]);
    if (s->shards[l].epoch_in_shard > 0)
      if (o_finalize(s, l))
        return writer_error();
  }
  if (s->sink->update_append) {
    const struct dimension* dims = s->cfg.dimensions;
    const uint8_t na = s->P.na;
    for (int l = 0; l < s->P.nlod; ++l) {
      uint64_t sizes[HALF_MAX_RANK];
      uint64_t inner = 1;
      for (int d = 1; d < s->P.rank; ++d)
        inner *= dims[d].size;
      for (int d = 1; d < na; ++d)
        sizes[d] = dims[d].size;
      uint64_t d0 = inner ? s->cursor / inner : 0;
      if (l > 0 && s->P.append_downsample)
        d0 = (d0 + ((1ull << l) - 1)) >> l;
      sizes[0] = d0;
      if (s->sink->update_append(s->sink, (uint8_t)l, na, sizes))
        return writer_error();
    }
  }
  return writer_ok();
}

static struct writer_result
o_flush_final(struct writer* self)
{
  struct oracle_stream* s = O_SELF(self);
  struct writer_result r = o_flush(s);
  s->flushed = 1;
  return r;
}

/* ---- standalone kernels for unit tests ---- */

int
oracle_reduce_window(void* dst,
                     const void* src,
                     uint64_t n,
                     enum dtype dt,
                     enum lod_reduce_method m)
{
  if (n == 0)
    return 1;
  switch (dt) {
#define X(D, T, A, K)                                                          \
  case D:                                                                      \
    *(T*)dst = reduce_##D((const T*)src, 0, n, (int)m);                        \
    return 0;
    O_FOR_TYPES(X)
#undef X
  }
  return 1;
}

int
oracle_fold(void* accum,
            const void* fresh,
            uint64_t n,
            uint32_t count,
            int level,
            enum dtype dt,
            enum lod_reduce_method m)
{
  return o_fold_dispatch(accum, fresh, n, count, level, dt, (int)m);
}

int
oracle_emit(void* dst,
            const void* accum,
            uint64_t n,
            uint32_t count,
            enum dtype dt,
            enum lod_reduce_method m)
{
  return o_emit_dispatch(dst, accum, n, count, dt, (int)m);
}

/* ---- writer result helpers (same values as src/writer.c:47-82) ---- */

struct writer_result
writer_ok(void)
{
  return (struct writer_result){ 0, { 0, 0 } };
}
struct writer_result
writer_error(void)
{
  return (struct writer_result){ 1, { 0, 0 } };
}
struct writer_result
writer_error_at(const void* b, const void* e)
{
  return (struct writer_result){ 1, { b, e } };
}
struct writer_result
writer_finished_at(const void* b, const void* e)
{
  return (struct writer_result){ 2, { b, e } };
}

/* ---- in-memory sink ---- */

struct o_mem_shard
{
  struct shard_writer base;
  uint8_t level;
  uint64_t index;
  uint8_t* data;
  size_t size, cap;
  int finalized;
};

struct oracle_mem_sink
{
  struct shard_sink base;
  struct o_mem_shard** shards;
  size_t n, cap;
};

static int
mem_write(struct shard_writer* self, uint64_t off, const void* b, const void* e)
{
  struct o_mem_shard* w = (struct o_mem_shard*)self;
  const size_t n = (size_t)((const char*)e - (const char*)b);
  if (off + n > w->cap) {
    size_t c = w->cap ? w->cap : 4096;
    while (c < off + n)
      c *= 2;
    uint8_t* p = (uint8_t*)realloc(w->data, c);
    if (!p)
      return 1;
    memset(p + w->cap, 0, c - w->cap);
    w->data = p;
    w->cap = c;
  }
  memcpy(w->data + off, b, n);
  if (off + n > w->size)
    w->size = off + n;
  return 0;
}

static int
mem_finalize(struct shard_writer* self)
{
  ((struct o_mem_shard*)self)->finalized = 1;
  return 0;
}

static struct shard_writer*
mem_open(struct shard_sink* self, uint8_t level, uint64_t index)
{
  struct oracle_mem_sink* s = (struct oracle_mem_sink*)self;
  for (size_t i = 0; i < s->n; ++i)
    if (s->shards[i]->level == level && s->shards[i]->index == index) {
      s->shards[i]->size = 0;
      s->shards[i]->finalized = 0;
      return &s->shards[i]->base;
    }
  if (s->n == s->cap) {
    size_t c = s->cap ? 2 * s->cap : 16;
    struct o_mem_shard** p =
      (struct o_mem_shard**)realloc(s->shards, c * sizeof(*p));
    if (!p)
      return NULL;
    s->shards = p;
    s->cap = c;
  }
  struct o_mem_shard* w = (struct o_mem_shard*)calloc(1, sizeof(*w));
  if (!w)
    return NULL;
  w->base.write = mem_write;
  w->base.finalize = mem_finalize;
  w->level = level;
  w->index = index;
  s->shards[s->n++] = w;
  return &w->base;
}

struct oracle_mem_sink*
oracle_mem_sink_create(void)
{
  struct oracle_mem_sink* s =
    (struct oracle_mem_sink*)calloc(1, sizeof(struct oracle_mem_sink));
  if (s)
    s->base.open = mem_open;
  return s;
}

void
oracle_mem_sink_destroy(struct oracle_mem_sink* s)
{
  if (!s)
    return;
  for (size_t i = 0; i < s->n; ++i) {
    free(s->shards[i]->data);
    free(s->shards[i]);
  }
  free(s->shards);
  free(s);
}

struct shard_sink*
oracle_mem_sink_base(struct oracle_mem_sink* s)
{
  return &s->base;
}

size_t
oracle_mem_sink_count(const struct oracle_mem_sink* s)
{
  return s->n;
}

int
oracle_mem_sink_at(const struct oracle_mem_sink* s,
                   size_t i,
                   uint8_t* level,
                   uint64_t* index,
                   const uint8_t** data,
                   size_t* size,
                   int* finalized)
{
  if (i >= s->n)
    return 1;
  *level = s->shards[i]->level;
  *index = s->shards[i]->index;
  *data = s->shards[i]->data;
  *size = s->shards[i]->size;
  *finalized = s->shards[i]->finalized;
  return 0;
}

/* ---- discard sink ---- */

struct o_null_sink
{
  struct shard_sink base;
  struct shard_writer w;
  uint64_t bytes;
};

static int
null_write(struct shard_writer* self, uint64_t off, const void* b, const void* e)
{
  (void)off;
  struct o_null_sink* s =
    (struct o_null_sink*)((char*)self - offsetof(struct o_null_sink, w));
  s->bytes += (uint64_t)((const char*)e - (const char*)b);
  return 0;
}

static int
null_finalize(struct shard_writer* self)
{
  (void)self;
  return 0;
}

static struct shard_writer*
null_open(struct shard_sink* self, uint8_t level, uint64_t index)
{
  (void)level;
  (void)index;
  return &((struct o_null_sink*)self)->w;
}

struct shard_sink*
oracle_null_sink_create(void)
{
  struct o_null_sink* s = (struct o_null_sink*)calloc(1, sizeof(*s));
  if (!s)
    return NULL;
  s->base.open = null_open;
  s->w.write = null_write;
  s->w.finalize = null_finalize;
  return &s->base;
}

void
oracle_null_sink_destroy(struct shard_sink* s)
{
  free(s);
}

uint64_t
oracle_null_sink_bytes(const struct shard_sink* s)
{
  return ((const struct o_null_sink*)s)->bytes;
}

/* ---- a stalling writer for writer_append_wait tests ---------------------- */

struct oracle_stalling_writer
{
  struct writer base; /* first: the vtable callbacks recover the object */
  int stalls, fail, calls;
  size_t chunk;
  double times[64];
};

static double
stall_now(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static struct writer_result
stalling_append(struct writer* self, struct slice data)
{
  struct oracle_stalling_writer* w = (struct oracle_stalling_writer*)self;
  if (w->calls < 64)
    w->times[w->calls] = stall_now();
  w->calls++;
  struct writer_result r = { 0, data };
  if (w->calls <= w->stalls)
    return r;
  if (w->fail) {
    r.error = writer_error_fail;
    return r;
  }
  const size_t left = (size_t)((const char*)data.end - (const char*)data.beg);
  const size_t take = (w->chunk && w->chunk < left) ? w->chunk : left;
  r.rest.beg = (const char*)data.beg + take;
  return r;
}

static struct writer_result
stalling_flush(struct writer* self)
{
  (void)self;
  struct writer_result r = { 0, { 0, 0 } };
  return r;
}

struct oracle_stalling_writer*
oracle_stalling_writer_create(int stalls, size_t chunk, int fail)
{
  struct oracle_stalling_writer* w =
    (struct oracle_stalling_writer*)calloc(1, sizeof(*w));
  if (!w)
    return NULL;
  w->base.append = stalling_append;
  w->base.flush = stalling_flush;
  w->stalls = stalls;
  w->chunk = chunk;
  w->fail = fail;
  return w;
}

void
oracle_stalling_writer_destroy(struct oracle_stalling_writer* w)
{
  free(w);
}

struct writer*
oracle_stalling_writer_base(struct oracle_stalling_writer* w)
{
  return &w->base;
}

int
oracle_stalling_writer_calls(const struct oracle_stalling_writer* w)
{
  return w->calls;
}

double
oracle_stalling_writer_time(const struct oracle_stalling_writer* w, int call)
{
  return (call >= 0 && call < 64) ? w->times[call] : 0.0;
}
