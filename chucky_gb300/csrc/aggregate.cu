// (d) Shard aggregation: compressed chunks -> shard-ordered byte runs.
//
// Per level of a batch (src/gpu/aggregate.cu:17-438 and
// src/cpu/aggregate.c:130-188 of the reference):
//   1. sizes in shard order: s[perm[i]] = size[gather[i]], unmapped
//      covering positions are 0;
//   2. the pre-padding sizes are kept for the shard index;
//   3. the last chunk of each shard group (n_active * cps_inner positions)
//      absorbs the padding that rounds the group to the shard alignment,
//      which is written as zeros;
//   4. exclusive scan -> byte offsets (offsets[positions] = total);
//   5. every chunk's bytes are copied to out + offsets[perm[i]].
// Steps 1-4 run in one CTA per level (a few thousand positions); step 5
// spreads 16 KiB pieces of every chunk over the grid (a warp per piece,
// aligned 16-byte stores assembled by funnel shifts, copy.cuh).
#include "copy.cuh"
#include "kernels.hpp"

namespace chucky {

namespace {

constexpr int kScanThreads = 1024;

__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v,
                                                         uint64_t* warp_tot,
                                                         uint64_t& total)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o)
      x += y;
  }
  if (lane == 31)
    warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint64_t t = lane < (blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o)
        t += y;
    }
    warp_tot[lane] = t; // inclusive prefix of warp totals
  }
  __syncthreads();
  const uint64_t before = wid ? warp_tot[wid - 1] : 0;
  total = warp_tot[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads)
agg_layout_k(AggBatch b, uint64_t* scratch, uint64_t scratch_stride)
{
  __shared__ uint64_t warp_tot[32];
  const AggLevel& L = b.lv[blockIdx.x];
  uint64_t* s = scratch + blockIdx.x * scratch_stride;
  for (uint64_t p = threadIdx.x; p < L.positions; p += blockDim.x)
    s[p] = 0;
  __syncthreads();
  for (uint64_t i = threadIdx.x; i < L.n; i += blockDim.x)
    s[L.perm[i]] = b.sizes[L.gather[i]];
  __syncthreads();
  for (uint64_t p = threadIdx.x; p < L.positions; p += blockDim.x)
    L.real_sizes[p] = s[p];
  if (b.alignment > 0 && L.group > 0) {
    __syncthreads();
    for (uint64_t g = threadIdx.x; g < L.positions / L.group;
         g += blockDim.x) {
      uint64_t t = 0;
      for (uint64_t j = 0; j < L.group; ++j)
        t += s[g * L.group + j];
      const uint64_t pad = (t + b.alignment - 1) / b.alignment * b.alignment - t;
      s[g * L.group + L.group - 1] += pad;
    }
  }
  __syncthreads();
  uint64_t carry = 0;
  for (uint64_t base = 0; base < L.positions; base += blockDim.x) {
    const uint64_t p = base + threadIdx.x;
    const uint64_t v = p < L.positions ? s[p] : 0;
    uint64_t tile_total;
    const uint64_t ex = block_exclusive_scan(v, warp_tot, tile_total);
    if (p < L.positions)
      L.offsets[p] = carry + ex;
    carry += tile_total;
  }
  if (threadIdx.x == 0)
    L.offsets[L.positions] = carry;
  // the padding that rounds each shard group up to the alignment is written
  // as zeros (no stale buffer bytes reach the shard files), and so is the
  // alignment's worth of bytes after the batch: a delivery write of a run
  // of epochs is rounded up to the alignment and may read that far past
  // the batch's last byte (src/stream/types.aggregate.c:10-26 allocates
  // the slack, zeroed)
  if (b.alignment > 0 && L.group > 0) {
    __syncthreads();
    for (uint64_t g = 0; g < L.positions / L.group; ++g) {
      const uint64_t last = g * L.group + L.group - 1;
      const uint64_t beg = L.offsets[last] + L.real_sizes[last];
      const uint64_t end = L.offsets[last + 1];
      for (uint64_t q = beg + threadIdx.x; q < end; q += blockDim.x)
        L.out[q] = 0;
    }
    const uint64_t total = L.offsets[L.positions];
    for (uint64_t q = threadIdx.x; q < b.alignment; q += blockDim.x)
      L.out[total + q] = 0;
  }
}

// One warp per 16 KiB piece of one chunk: (chunk, piece) pairs are spread
// over the grid so that a few large chunks still keep every SM busy; the
// copy itself uses aligned 16-byte stores (copy.cuh).
constexpr uint64_t kPiece = 16 << 10;

__global__ void __launch_bounds__(128)
agg_gather_k(AggBatch b, uint64_t total_chunks, uint64_t pieces_per_chunk)
{
  const uint64_t warp = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nwarps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  const unsigned lane = threadIdx.x & 31;
  for (uint64_t w = warp; w < total_chunks * pieces_per_chunk; w += nwarps) {
    uint64_t i = w / pieces_per_chunk;
    const uint64_t piece = w - i * pieces_per_chunk;
    int l = 0;
    while (l < b.nlevels && i >= b.lv[l].n) {
      i -= b.lv[l].n;
      ++l;
    }
    if (l >= b.nlevels)
      return;
    const AggLevel& L = b.lv[l];
    const uint32_t c = L.gather[i];
    const uint64_t n = b.sizes[c];
    const uint64_t off = piece * kPiece;
    if (off >= n)
      continue;
    const uint64_t len = n - off < kPiece ? n - off : kPiece;
    copy_bytes(L.out + L.offsets[L.perm[i]] + off,
               b.comp + c * b.comp_stride + off, len, lane, 32);
  }
}

__global__ void fill_u64_k(uint64_t* p, uint64_t v, uint64_t n)
{
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += uint64_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

// Bytes [start, *total) of each level's device copy to its host slot (the
// part the copy engine's transfer of the expected size did not cover), a
// 64 KiB piece per CTA and step; levels along grid y.
constexpr uint64_t kTailPiece = 64 << 10;

__global__ void __launch_bounds__(256) tail_copy_k(TailCopies t)
{
  const TailCopy& c = t.lv[blockIdx.y];
  const uint64_t total = *c.total + c.extra;
  if (total <= c.start)
    return;
  for (uint64_t p = c.start + blockIdx.x * kTailPiece; p < total;
       p += uint64_t(gridDim.x) * kTailPiece) {
    const uint64_t n = total - p < kTailPiece ? total - p : kTailPiece;
    copy_bytes(c.dst + p, c.src + p, n, threadIdx.x, blockDim.x);
  }
}

// ---- shard index and crc32c ------------------------------------------------

constexpr uint32_t kCrcPoly = 0x82F63B78u; // Castagnoli, reflected
constexpr int kIndexThreads = 128;

// a * b mod P in the reflected representation (bit 31 = x^0); `a` is a
// power of x (never 0).  The combination of segment CRCs through
// multiplication by x^(8 n) mod P is the published method of zlib's
// crc32_combine (M. Adler).
__device__ uint32_t crc_mulmod(uint32_t a, uint32_t b)
{
  uint32_t p = 0;
  for (int i = 0; i < 32; ++i) {
    if (a & (0x80000000u >> i))
      p ^= b;
    b = (b & 1) ? (b >> 1) ^ kCrcPoly : b >> 1;
  }
  return p;
}

// x^(8 n) mod P
__device__ uint32_t crc_xpow8(uint64_t n)
{
  uint32_t p = 0x80000000u, base = 0x00800000u; // x^0, x^8
  while (n) {
    if (n & 1)
      p = crc_mulmod(p, base);
    base = crc_mulmod(base, base);
    n >>= 1;
  }
  return p;
}

// crc32c of the index words idx[0 .. nwords) (u64, little endian), by the
// whole CTA: one segment per thread, combined by thread 0.
__device__ uint32_t index_crc32c(const uint64_t* idx, uint64_t nwords, uint32_t* table,
                                 uint32_t* part)
{
  const unsigned tid = threadIdx.x, nt = blockDim.x;
  const uint64_t per = (nwords + nt - 1) / nt; // words per thread
  const uint64_t w0 = (tid * per < nwords ? tid * per : nwords), w1 = (w0 + per < nwords ? w0 + per : nwords);
  uint32_t c = 0;
  for (uint64_t w = w0; w < w1; ++w) {
    uint64_t v = idx[w];
    for (int k = 0; k < 8; ++k) {
      c = table[(c ^ uint32_t(v)) & 0xFF] ^ (c >> 8);
      v >>= 8;
    }
  }
  part[tid] = c;
  __syncthreads();
  uint32_t crc = 0;
  if (tid == 0) {
    uint32_t st = 0xFFFFFFFFu;
    const uint32_t xfull = crc_xpow8(per * 8);
    for (unsigned t = 0; t < nt; ++t) {
      const uint64_t a = t * per < nwords ? t * per : nwords;
      const uint64_t b = a + per < nwords ? a + per : nwords;
      if (b <= a)
        break;
      const uint32_t x = (b - a == per) ? xfull : crc_xpow8((b - a) * 8);
      st = crc_mulmod(x, st) ^ part[t];
    }
    crc = st ^ 0xFFFFFFFFu;
  }
  __syncthreads();
  return crc;
}

// A CTA per (level, shard) (shards beyond the grid's y extent looped): the
// level's runs in order (each shard's cursor depends on the runs before),
// the entries of a run in parallel.
__global__ void __launch_bounds__(kIndexThreads) index_k(IndexBatch b)
{
  __shared__ uint32_t table[256];
  __shared__ uint32_t part[kIndexThreads];
  __shared__ uint32_t crc_sh;
  const IndexLevel& L = b.lv[blockIdx.x];
  const unsigned tid = threadIdx.x, nt = blockDim.x;
  if (blockIdx.y >= L.shards)
    return;
  for (unsigned i = tid; i < 256; i += nt) {
    uint32_t c = i;
    for (int k = 0; k < 8; ++k)
      c = (c & 1) ? (c >> 1) ^ kCrcPoly : c >> 1;
    table[i] = c;
  }
  __syncthreads();
  const uint64_t sa = b.alignment;
  const uint64_t nidx = L.cps_total * 16, total = nidx + 4;
  const uint64_t pad = L.blob_bytes - total;
  const uint64_t cpi = L.cpi;
  for (uint64_t s = blockIdx.y; s < L.shards; s += gridDim.y) {
    uint64_t* idx = L.index + s * L.cps_total * 2;
    uint64_t cur = L.cursor[s];
    uint32_t nfinal = 0;
    // the shard's final index blob: padding, index, crc32c; then reset
    auto finalize = [&](uint8_t* blob) {
      const uint32_t crc = index_crc32c(idx, L.cps_total * 2, table, part);
      if (tid == 0)
        crc_sh = crc;
      __syncthreads();
      for (uint64_t i = tid; i < pad; i += nt)
        blob[i] = 0;
      if ((pad & 3) == 0) {
        uint32_t* d = reinterpret_cast<uint32_t*>(blob + pad);
        const uint32_t* w = reinterpret_cast<const uint32_t*>(idx);
        for (uint64_t i = tid; i < nidx / 4; i += nt)
          d[i] = w[i];
      } else {
        const uint8_t* src = reinterpret_cast<const uint8_t*>(idx);
        for (uint64_t i = tid; i < nidx; i += nt)
          blob[pad + i] = src[i];
      }
      if (tid < 4)
        blob[pad + nidx + tid] = uint8_t(crc_sh >> (8 * tid));
      __syncthreads();
      for (uint64_t i = tid; i < L.cps_total * 2; i += nt)
        idx[i] = ~uint64_t(0);
      __syncthreads();
    };
    if (L.flush) {
      finalize(L.blobs + s * L.blob_bytes);
      cur = 0;
    } else {
      for (uint32_t r = 0; r < L.n_runs; ++r) {
        const IndexRun R = L.runs[r];
        const uint64_t j0 = s * L.n_active * cpi + uint64_t(R.a0) * cpi;
        const uint64_t j1 = j0 + uint64_t(R.run) * cpi;
        const uint64_t base = L.offsets[j0];
        const uint64_t nbytes = L.offsets[j1] - base;
        for (uint64_t t = tid; t < uint64_t(R.run) * cpi; t += nt) {
          const uint64_t j = j0 + t;
          const uint64_t rs = L.real_sizes[j];
          if (rs > 0) {
            const uint64_t slot = (uint64_t(R.eis0) + t / cpi) * cpi + t % cpi;
            idx[2 * slot] = cur + (L.offsets[j] - base);
            idx[2 * slot + 1] = rs;
          }
        }
        __syncthreads();
        cur += sa ? (nbytes + sa - 1) / sa * sa : nbytes;
        if (R.final) {
          finalize(L.blobs + (uint64_t(nfinal) * L.shards + s) * L.blob_bytes);
          ++nfinal;
          cur = 0;
        }
      }
    }
    if (tid == 0)
      L.cursor[s] = cur;
    __syncthreads();
  }
}

__global__ void stage_copy_k(uint32_t* dst, const uint32_t* src, uint64_t n)
{
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += uint64_t(gridDim.x) * blockDim.x)
    dst[i] = src[i];
}

} // namespace

cudaError_t launch_stage_copy(uint32_t* dst, const uint32_t* src, uint64_t n,
                              cudaStream_t st)
{
  if (!n)
    return cudaSuccess;
  const uint64_t blocks = (n + 255) / 256;
  const uint64_t sms = uint64_t(device_sm_count());
  stage_copy_k<<<int(blocks < sms ? blocks : sms), 256, 0, st>>>(dst, src, n);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_aggregate(const AggBatch& b,
                             uint64_t* scratch,
                             cudaStream_t st)
{
  if (b.nlevels <= 0)
    return cudaSuccess;
  uint64_t stride = 0, total = 0;
  for (int l = 0; l < b.nlevels; ++l) {
    stride = stride > b.lv[l].positions ? stride : b.lv[l].positions;
    total += b.lv[l].n;
  }
  agg_layout_k<<<b.nlevels, kScanThreads, 0, st>>>(b, scratch, stride);
  note_launches(1);
  if (total) {
    const uint64_t ppc = (b.comp_stride + kPiece - 1) / kPiece;
    const uint64_t blocks = (total * ppc + 3) / 4;
    const uint64_t cap = uint64_t(device_sm_count()) * 64;
    const int grid = int(blocks < cap ? blocks : cap);
    agg_gather_k<<<grid, 128, 0, st>>>(b, total, ppc);
    note_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_tail_copy(const TailCopies& t, uint64_t max_bytes, cudaStream_t st)
{
  if (t.n <= 0 || !max_bytes)
    return cudaSuccess;
  const uint64_t pieces = (max_bytes + kTailPiece - 1) / kTailPiece;
  const uint64_t cap = uint64_t(device_sm_count()) * 2;
  const dim3 grid(unsigned(pieces < cap ? pieces : cap), unsigned(t.n));
  tail_copy_k<<<grid, 256, 0, st>>>(t);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_index(const IndexBatch& b, cudaStream_t st)
{
  if (b.nlevels <= 0 || !b.max_shards)
    return cudaSuccess;
  const uint64_t ys = b.max_shards < 65535 ? b.max_shards : 65535;
  const dim3 grid(unsigned(b.nlevels), unsigned(ys));
  index_k<<<grid, kIndexThreads, 0, st>>>(b);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_fill_u64(uint64_t* p, uint64_t v, uint64_t n, cudaStream_t st)
{
  if (!n)
    return cudaSuccess;
  const uint64_t blocks = (n + 255) / 256;
  fill_u64_k<<<int(blocks < 1024 ? blocks : 1024), 256, 0, st>>>(p, v, n);
  note_launches(1);
  return cudaGetLastError();
}

} // namespace chucky
