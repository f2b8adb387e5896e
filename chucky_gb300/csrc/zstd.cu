// (c) zstd encoder: one standard zstd frame per chunk (CODEC_ZSTD).
//
// The reference compresses each chunk into a zstd frame with ZSTD_compress
// on the CPU or nvcomp's batched zstd on the GPU (src/cpu/compress.c:78-93,
// src/gpu/compress.cu:345-358); frames are decoded with ZSTD_decompress.
// This encoder writes the format of RFC 8878 from scratch:
//   frame   : magic, single-segment header with the content size, no
//             checksum, blocks of at most 128 KiB;
//   block   : RLE when every byte is equal, raw when coding does not pay,
//             otherwise a compressed block;
//   literals: Huffman-coded (4 streams, code lengths <= 11 bits, weights
//             sent directly or FSE-compressed with two interleaved states)
//             when that is smaller, else raw / RLE;
//   sequences: LZ77 sequences from the shared warp match finder (lz77.cuh),
//             literal-length / match-length / offset codes with the
//             predefined FSE distributions, extra bits, three interleaved
//             states in one backward bitstream.
// Kernels: find (warp per 16 KiB segment) -> block (CTA per 128 KiB block:
// literal gather + histogram, Huffman build, 4-stream bit packing, sequence
// stream) -> frame (CTA per chunk: frame header + blocks).
#include "kernels_codec.hpp"
#include "launch.cuh"
#include "copy.cuh"
#include "lz77.cuh"

namespace chucky {

namespace {

// 32 KiB blocks: every block builds its own Huffman table serially, so
// smaller blocks put more of them in flight (the table costs ~0.3% ratio)
constexpr uint32_t kBlockLog = 15;
constexpr uint32_t kBlockBytes = 1u << kBlockLog; // 32 KiB
constexpr uint32_t kSegsPerBlock = kBlockBytes / kSegBytes;
constexpr uint32_t kStageBytes = kBlockBytes + 1024;
constexpr int kStreamThreads = 32;                // a warp per Huffman stream
constexpr int kBlockThreads = 4 * kStreamThreads; // >= a warp per segment
static_assert(kBlockThreads >= 32 * int(kSegsPerBlock), "warp per segment");
constexpr int kFindWarps = 4;
constexpr uint32_t kHufMaxBits = 11;
#ifndef CHUCKY_ZSTD_MIN_MATCH
#define CHUCKY_ZSTD_MIN_MATCH 6
#endif
// matches shorter than this cost more as a sequence than as literals
constexpr uint32_t kMinMatch = CHUCKY_ZSTD_MIN_MATCH;

struct ZSeg
{
  uint32_t nseq, trailing, matched; // matched = bytes covered by matches
};

// ---------------------------------------------------------------------------
// bit writer for backward-read streams (written forward, LSB first; the
// decoder starts at the highest set bit of the last byte)
// ---------------------------------------------------------------------------

struct BitOut
{
  uint8_t* p;
  uint64_t acc;
  int n;
  __device__ void init(uint8_t* dst)
  {
    p = dst;
    acc = 0;
    n = 0;
  }
  __device__ __forceinline__ void put(uint64_t v, int bits)
  {
    acc |= (v & ((uint64_t(1) << bits) - 1)) << n;
    n += bits;
    while (n >= 8) {
      *p++ = uint8_t(acc);
      acc >>= 8;
      n -= 8;
    }
  }
  // end mark + padding; returns one past the last byte written
  __device__ uint8_t* close()
  {
    put(1, 1);
    if (n > 0)
      *p++ = uint8_t(acc);
    return p;
  }
};

// ---------------------------------------------------------------------------
// FSE tables (RFC 8878 4.1.1).  The decoder's table spreads symbols with
// step 5/8*size+3 ("less than 1" symbols at the top); state u of symbol s
// is the k-th of its states, x = count + k, reads AL - highbit(x) bits.
// The encoder keeps v = state + size and, for symbol s with count c,
// emits nb low bits of v where nb = AL - h or AL - h - 1 (h = highbit(c)).
// ---------------------------------------------------------------------------

__host__ __device__ __forceinline__ int highbit(uint32_t x)
{
#ifdef __CUDA_ARCH__
  return 31 - __clz(x);
#else
  return 31 - __builtin_clz(x);
#endif
}

struct FseEnc
{
  int al;
  int16_t count[64];  // normalized count per symbol (-1 stored as 1)
  uint8_t first[64];  // index of the symbol's first state in `states`
  uint8_t states[64]; // states of each symbol, ascending, grouped by symbol
};

// Build encoder tables from normalized counts (-1 = "less than 1").
// `spread` and `fill` are 64-entry scratch arrays (shared memory on the
// device: local arrays of one thread would miss L1).
__host__ __device__ inline void fse_build(FseEnc& t,
                                          const int16_t* norm,
                                          int nsym,
                                          int al,
                                          uint8_t* spread,
                                          uint8_t* fill)
{
  const int size = 1 << al;
  int high = size - 1;
  for (int s = 0; s < nsym; ++s)
    if (norm[s] == -1)
      spread[high--] = uint8_t(s);
  const int step = (size >> 1) + (size >> 3) + 3, mask = size - 1;
  int pos = 0;
  for (int s = 0; s < nsym; ++s)
    for (int i = 0; i < norm[s]; ++i) {
      spread[pos] = uint8_t(s);
      do
        pos = (pos + step) & mask;
      while (pos > high);
    }
  int acc = 0;
  for (int s = 0; s < nsym; ++s) {
    t.count[s] = norm[s] == -1 ? 1 : norm[s];
    t.first[s] = uint8_t(acc);
    acc += t.count[s];
  }
  for (int s = 0; s < nsym; ++s)
    fill[s] = t.first[s];
  for (int u = 0; u < size; ++u)
    t.states[fill[spread[u]]++] = uint8_t(u);
  t.al = al;
}

// The three predefined sequence tables, built once on the host.
struct PredefTables
{
  FseEnc ll, ml, of;
};

// v in [size, 2 size): emit bits, move to a state of symbol s.
__device__ __forceinline__ void fse_encode(const FseEnc& t,
                                           uint32_t& v,
                                           int s,
                                           BitOut& bo)
{
  const int c = t.count[s], h = highbit(uint32_t(c));
  int nb = t.al - h;
  if ((v >> nb) < uint32_t(c))
    --nb;
  bo.put(v, nb);
  const uint32_t x = v >> nb;
  v = t.states[t.first[s] + (x - c)] + (1u << t.al);
}

__device__ __forceinline__ uint32_t fse_init(const FseEnc& t, int s)
{
  return t.states[t.first[s]] + (1u << t.al);
}

// Predefined distributions (RFC 8878 3.1.1.3.2.2).
static const int16_t kLLNormH[36] = { 4, 3, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2,
                                     2, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2,
                                     2, 3, 2, 1, 1, 1, 1, 1, -1, -1, -1, -1 };
static const int16_t kMLNormH[53] = { 1, 4, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1 };
static const int16_t kOFNormH[29] = { 1, 1, 1, 1, 1, 1, 2, 2, 2, 1,
                                     1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, -1, -1, -1, -1, -1 };

__constant__ uint32_t kLLBase[36] = { 0,  1,  2,   3,   4,   5,    6,    7,
                                      8,  9,  10,  11,  12,  13,   14,   15,
                                      16, 18, 20,  22,  24,  28,   32,   40,
                                      48, 64, 128, 256, 512, 1024, 2048, 4096,
                                      8192, 16384, 32768, 65536 };
__constant__ uint8_t kLLBits[36] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 3, 3,
                                     4, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16 };
__constant__ uint32_t kMLBase[53] = {
  3,  4,  5,  6,  7,  8,  9,  10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20,
  21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 33, 34, 35, 37, 39, 41,
  43, 47, 51, 59, 67, 83, 99, 131, 259, 515, 1027, 2051, 4099, 8195, 16387,
  32771, 65539
};
__constant__ uint8_t kMLBits[53] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 3, 3, 4, 4,
                                     5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16 };

__device__ __forceinline__ int ll_code(uint32_t ll)
{
  if (ll < 16)
    return int(ll);
  if (ll >= 64)
    return highbit(ll) + 19;
  // 16..63
  int c = 16;
  while (c < 35 && kLLBase[c + 1] <= ll)
    ++c;
  return c;
}

__device__ __forceinline__ int ml_code(uint32_t ml)
{
  const uint32_t mb = ml - 3;
  if (mb < 32)
    return int(mb);
  if (mb >= 128)
    return highbit(mb) + 36;
  int c = 32;
  while (c < 52 && kMLBase[c + 1] <= ml)
    ++c;
  return c;
}

// ---------------------------------------------------------------------------
// find
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(32 * kFindWarps)
zstd_find_k(CodecBatch b, Seq* seqs, ZSeg* meta)
{
  __shared__ uint16_t tables[kFindWarps][1 << kHashLog];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t seg = uint64_t(blockIdx.x) * kFindWarps + w;
  if (seg >= b.n_chunks * b.segs_per_chunk)
    return;
  const uint64_t chunk = seg / b.segs_per_chunk;
  const uint32_t k = uint32_t(seg % b.segs_per_chunk);
  const uint8_t* base = b.in + b.id(chunk) * b.in_stride;
  const uint32_t s0 = k * kSegBytes;
  const uint32_t s1 = min(b.chunk_bytes, s0 + kSegBytes);
  Seq* out = seqs + seg * kMaxSeqPerSeg;
  const SegInfo info =
    lz77_parse_segment(base, s0, s1, s1, s1, tables[w], out, kMinMatch);
  __syncwarp();
  uint32_t matched = 0;
  for (uint32_t i = lane; i < info.nseq; i += 32)
    matched += out[i].match;
  for (int o = 16; o; o >>= 1)
    matched += __shfl_xor_sync(0xffffffffu, matched, o);
  if (lane == 0)
    meta[seg] = ZSeg{ info.nseq, info.trailing, matched };
}

// ---------------------------------------------------------------------------
// Huffman (thread 0 of the block CTA)
// ---------------------------------------------------------------------------

// Working arrays of the serial Huffman build, kept in shared memory (local
// memory of one thread is interleaved with every other thread's frame and
// would miss L1 on every access).
struct HuffScratch
{
  uint32_t rank_start[16], count_w[16], whist[16];
  int16_t norm[16];
  uint8_t spread[64], fill[64];
  uint16_t sym[256];
  uint32_t f[512];
  int16_t parent[512];
  uint8_t depth[512];
  uint8_t w[256];
};

struct Huff
{
  uint32_t cl[256];    // code | length << 16 (one load per symbol)
  uint16_t code[256];
  uint8_t len[256];
  int max_bits;
  int last;            // highest symbol with a code
  uint8_t desc[320];   // tree description (header byte + payload)
  int desc_len;
  uint64_t bits;       // sum of code lengths over the literals
};

// Code lengths limited to kHufMaxBits, complete prefix code.  Two-queue
// Huffman on the sorted leaves, then clamp + Kraft repair.
__device__ bool huff_lengths(const uint32_t* freq,
                             const uint16_t* sorted,
                             int n,
                             Huff& h,
                             HuffScratch& x)
{
  // `sorted`: the n symbols with freq > 0, ascending by (freq, symbol)
  uint16_t* sym = x.sym;
  uint32_t* f = x.f;
  int16_t* parent = x.parent;
  if (n < 2)
    return false;
  for (int i = 0; i < n; ++i)
    sym[i] = sorted[i];
  for (int i = 0; i < n; ++i)
    f[i] = freq[sym[i]];
  int leaf = 0, inode = n, next = n;
  for (int k = 0; k < n - 1; ++k) {
    int pick[2];
    for (int t = 0; t < 2; ++t) {
      if (leaf < n && (inode >= next || f[leaf] <= f[inode]))
        pick[t] = leaf++;
      else
        pick[t] = inode++;
    }
    f[next] = f[pick[0]] + f[pick[1]];
    parent[pick[0]] = parent[pick[1]] = int16_t(next);
    ++next;
  }
  uint8_t* depth = x.depth;
  depth[next - 1] = 0;
  for (int i = next - 2; i >= 0; --i)
    depth[i] = uint8_t(depth[parent[i]] + 1);
  for (int s = 0; s < 256; ++s)
    h.len[s] = 0;
  int maxlen = 0;
  for (int i = 0; i < n; ++i) {
    int L = depth[i];
    if (L > int(kHufMaxBits))
      L = kHufMaxBits;
    h.len[sym[i]] = uint8_t(L);
    maxlen = L > maxlen ? L : maxlen;
  }
  // Kraft repair at maxlen: sum of 2^(maxlen-len) must equal 2^maxlen
  const uint32_t full = 1u << maxlen;
  uint32_t kraft = 0;
  for (int i = 0; i < n; ++i)
    kraft += 1u << (maxlen - h.len[sym[i]]);
  // over-full: lengthen the least frequent codes shorter than maxlen
  while (kraft > full) {
    for (int i = 0; i < n && kraft > full; ++i) {
      const int s = sym[i];
      if (h.len[s] < maxlen) {
        kraft -= 1u << (maxlen - h.len[s] - 1);
        h.len[s]++;
      }
    }
  }
  // under-full: shorten the most frequent codes that still fit
  for (int i = n - 1; i >= 0 && kraft < full; --i) {
    const int s = sym[i];
    while (h.len[s] > 1 && kraft + (1u << (maxlen - h.len[s])) <= full) {
      kraft += 1u << (maxlen - h.len[s]);
      h.len[s]--;
    }
  }
  if (kraft != full)
    return false;
  h.max_bits = 0;
  for (int s = 0; s < 256; ++s)
    h.max_bits = h.len[s] > h.max_bits ? h.len[s] : h.max_bits;
  return true;
}

// Canonical codes in zstd's order: by weight ascending (longest code
// first), then by symbol (RFC 8878 4.2.1.3).
__device__ void huff_codes(Huff& h, uint32_t* rank_start, uint32_t* count_w)
{
  const int mb = h.max_bits;
  for (int i = 0; i < 16; ++i)
    rank_start[i] = count_w[i] = 0;
  for (int s = 0; s < 256; ++s)
    if (h.len[s])
      count_w[mb + 1 - h.len[s]]++;
  uint32_t acc = 0;
  for (int w = 1; w <= mb; ++w) {
    rank_start[w] = acc;
    acc += count_w[w] << (w - 1);
  }
  h.last = 0;
  for (int s = 0; s < 256; ++s)
    if (h.len[s]) {
      const int w = mb + 1 - h.len[s];
      h.code[s] = uint16_t(rank_start[w] >> (w - 1));
      rank_start[w] += 1u << (w - 1);
      h.last = s;
    }
}

// Normalize a histogram of weights to 2^al, every present symbol >= 1 and
// no symbol above half the table (so every state reads >= 1 bit and the
// decoder's end-of-stream test fires exactly after the last weight).
__device__ void norm_weights(const uint32_t* hist, int nsym, int al, int16_t* norm)
{
  const int size = 1 << al, half = size / 2;
  uint32_t total = 0;
  int present = 0;
  for (int s = 0; s < nsym; ++s) {
    total += hist[s];
    present += hist[s] > 0;
  }
  int sum = 0;
  for (int s = 0; s < nsym; ++s) {
    int c = 0;
    if (hist[s]) {
      c = int((uint64_t(hist[s]) * size + total / 2) / total);
      c = c < 1 ? 1 : (c > half ? half : c);
    }
    norm[s] = int16_t(c);
    sum += c;
  }
  if (present == 1) { // a second symbol takes the other half
    for (int s = 0; s < nsym; ++s)
      if (!hist[s]) {
        norm[s] = int16_t(size - sum);
        sum = size;
        break;
      }
  }
  while (sum > size) { // take from the largest
    int best = -1;
    for (int s = 0; s < nsym; ++s)
      if (norm[s] > 1 && (best < 0 || norm[s] > norm[best]))
        best = s;
    norm[best]--;
    --sum;
  }
  while (sum < size) { // give to the most under-represented that has room
    int best = -1;
    for (int s = 0; s < nsym; ++s)
      if (hist[s] && norm[s] < half &&
          (best < 0 || uint64_t(hist[s]) * uint64_t(norm[best]) >
                         uint64_t(hist[best]) * uint64_t(norm[s])))
        best = s;
    if (best < 0) // everything capped: an absent symbol takes the rest
      for (int s = 0; s < nsym && best < 0; ++s)
        if (!hist[s] && norm[s] < half)
          best = s;
    norm[best]++;
    ++sum;
  }
}

// FSE table description (RFC 8878 4.1.1), forward bitstream.
__device__ int write_ncount(uint8_t* out, const int16_t* norm, int nsym, int al)
{
  uint64_t acc = uint64_t(al - 5);
  int n = 4, len = 0;
  int remaining = (1 << al) + 1, threshold = 1 << al, nb = al + 1;
  bool prev0 = false;
  int s = 0;
  auto flush = [&]() {
    while (n >= 8) {
      out[len++] = uint8_t(acc);
      acc >>= 8;
      n -= 8;
    }
  };
  while (s < nsym && remaining > 1) {
    if (prev0) {
      int start = s;
      while (s < nsym && !norm[s])
        ++s;
      while (s >= start + 24) {
        start += 24;
        acc |= uint64_t(0xFFFF) << n;
        n += 16;
        flush();
      }
      while (s >= start + 3) {
        start += 3;
        acc |= uint64_t(3) << n;
        n += 2;
      }
      acc |= uint64_t(s - start) << n;
      n += 2;
      flush();
    }
    int count = norm[s++];
    const int mx = (2 * threshold - 1) - remaining;
    remaining -= count < 0 ? -count : count;
    count++;
    if (count >= threshold)
      count += mx;
    acc |= uint64_t(count) << n;
    n += nb;
    n -= count < mx;
    prev0 = count == 1;
    while (remaining < threshold) {
      nb--;
      threshold >>= 1;
    }
    flush();
  }
  if (n > 0)
    out[len++] = uint8_t(acc);
  return len;
}

// Tree description: direct 4-bit weights when <= 128 weights, else FSE.
__device__ bool huff_describe(Huff& h, HuffScratch& x, FseEnc& t)
{
  const int mb = h.max_bits, nw = h.last; // explicit weights: symbols < last
  uint8_t* w = x.w;
  for (int s = 0; s < nw; ++s)
    w[s] = h.len[s] ? uint8_t(mb + 1 - h.len[s]) : 0;
  if (nw <= 128) {
    h.desc[0] = uint8_t(127 + nw);
    for (int i = 0; i < (nw + 1) / 2; ++i) {
      const uint8_t hi = w[2 * i], lo = 2 * i + 1 < nw ? w[2 * i + 1] : 0;
      h.desc[1 + i] = uint8_t(hi << 4 | lo);
    }
    h.desc_len = 1 + (nw + 1) / 2;
    return true;
  }
  // FSE-compressed weights, accuracy log 6, two interleaved states
  uint32_t* hist = x.whist;
  for (int i = 0; i < 16; ++i)
    hist[i] = 0;
  int maxw = 0;
  for (int s = 0; s < nw; ++s) {
    hist[w[s]]++;
    maxw = w[s] > maxw ? w[s] : maxw;
  }
  const int nsym = maxw + 2 <= 13 ? maxw + 2 : 13; // room for a spare symbol
  int16_t* norm = x.norm;
  const int al = 6;
  norm_weights(hist, nsym, al, norm);
  fse_build(t, norm, nsym, al, x.spread, x.fill);
  uint8_t* out = h.desc + 1;
  int len = write_ncount(out, norm, nsym, al);
  BitOut bo;
  bo.init(out + len);
  uint32_t v1, v2;
  int i = nw;
  if (nw & 1) {
    v1 = fse_init(t, w[--i]);
    v2 = fse_init(t, w[--i]);
    fse_encode(t, v1, w[--i], bo);
  } else {
    v2 = fse_init(t, w[--i]);
    v1 = fse_init(t, w[--i]);
  }
  while (i > 0) {
    fse_encode(t, v2, w[--i], bo);
    fse_encode(t, v1, w[--i], bo);
  }
  bo.put(v2 - (1u << al), al);
  bo.put(v1 - (1u << al), al);
  const uint8_t* end = bo.close();
  len = int(end - out);
  if (len >= 128)
    return false;
  h.desc[0] = uint8_t(len);
  h.desc_len = 1 + len;
  return true;
}

// ---------------------------------------------------------------------------
// block
// ---------------------------------------------------------------------------

struct BlockShared
{
  uint32_t hist[256];
  uint32_t whist[kSegsPerBlock][256]; // per-warp histograms (merged)
  uint16_t sorted[256];               // used symbols by (count, symbol)
  uint32_t nsym;
  PredefTables pre;                   // predefined sequence tables
  FseEnc tw;                          // Huffman weights table
  HuffScratch hx;
  Huff huff;
  uint32_t seg_nseq[kSegsPerBlock];
  uint32_t seg_carry[kSegsPerBlock];
  uint32_t seg_litout[kSegsPerBlock]; // literal buffer offset of seg start
  uint32_t nseq, nlit;
  uint32_t stream_bits[4];
  uint32_t stream_pos[4]; // byte offset of each Huffman stream in staging
  uint32_t lit_mode;      // 0 raw, 1 rle, 2 huffman
  uint32_t lit_hdr;       // literals section header bytes
  uint32_t lit_size;      // literals section bytes (header included)
  uint32_t all_same;
};

__device__ __forceinline__ void put_le(uint8_t* p, uint64_t v, int n)
{
  for (int i = 0; i < n; ++i)
    p[i] = uint8_t(v >> (8 * i));
}

// Visit lits[hi-1], lits[hi-2], ..., lits[lo] (descending), reading the
// shared-memory literal buffer 16 bytes at a time.
template<typename F>
__device__ __forceinline__ void for_each_desc(const uint8_t* lits,
                                              uint32_t lo,
                                              uint32_t hi,
                                              F&& f)
{
  uint32_t a = hi;
  while (a > lo) {
    const uint32_t wi = (a - 1) >> 4;
    const uint4 w = reinterpret_cast<const uint4*>(lits)[wi];
    const uint32_t wlo = max(lo, wi << 4);
    for (uint32_t x = a; x > wlo; --x) {
      const uint32_t o = (x - 1) & 15;
      const uint32_t word = o < 4 ? w.x : (o < 8 ? w.y : (o < 12 ? w.z : w.w));
      f(uint8_t(word >> ((o & 3) * 8)));
    }
    a = wlo;
  }
}

// Copy n literal bytes in[src..) -> lits[dst..) with one warp and count them
// in `hist`; the body moves whole aligned 32-bit words of the input.
__device__ __forceinline__ void gather_run(const uint8_t* in,
                                           uint32_t src,
                                           uint32_t n,
                                           uint8_t* lits,
                                           uint32_t dst,
                                           uint32_t* hist,
                                           unsigned lane)
{
  const uint32_t lead = (4 - (src & 3)) & 3;
  const uint32_t h = n < lead ? n : lead;
  if (lane < h) {
    const uint8_t c = in[src + lane];
    lits[dst + lane] = c;
    atomicAdd(&hist[c], 1u);
  }
  const uint32_t nw = (n - h) >> 2;
  const uint32_t* w = reinterpret_cast<const uint32_t*>(in + src + h);
  for (uint32_t i = lane; i < nw; i += 32) {
    const uint32_t v = w[i];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint8_t c = uint8_t(v >> (8 * k));
      lits[dst + h + 4 * i + k] = c;
      atomicAdd(&hist[c], 1u);
    }
  }
  for (uint32_t t = h + 4 * nw + lane; t < n; t += 32) {
    const uint8_t c = in[src + t];
    lits[dst + t] = c;
    atomicAdd(&hist[c], 1u);
  }
}

__global__ void __launch_bounds__(kBlockThreads)
zstd_block_k(CodecBatch b,
             const __grid_constant__ PredefTables pre,
             const Seq* seqs,
             const ZSeg* meta,
             uint8_t* stage_all,
             uint32_t* block_sizes,
             uint32_t blocks_per_chunk)
{
  __shared__ BlockShared S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t blk = blockIdx.x;
  const uint64_t chunk = blk / blocks_per_chunk;
  const uint32_t bi = uint32_t(blk % blocks_per_chunk);
  const uint8_t* in = b.in + b.id(chunk) * b.in_stride;
  const uint32_t b0 = bi * kBlockBytes;
  const uint32_t b1 = min(b.chunk_bytes, b0 + kBlockBytes);
  const uint32_t bsize = b1 - b0;
  const uint32_t seg0 = b0 / kSegBytes;
  const uint32_t nsegs = (bsize + kSegBytes - 1) / kSegBytes;
  const uint64_t segbase = chunk * b.segs_per_chunk + seg0;
  CHUCKY_DYN_SHARED(uint8_t, lits); // this block's literals
  uint8_t* stage = stage_all + blk * kStageBytes;

  for (int i = tid; i < 256 * int(kSegsPerBlock); i += blockDim.x)
    (&S.whist[0][0])[i] = 0;
  // the three predefined sequence tables (built once on the host)
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&pre);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&S.pre);
    for (int i = tid; i < int(sizeof(PredefTables) / 4); i += blockDim.x)
      dst[i] = src[i];
  }
  if (tid == 0) {
    uint32_t carry = 0, matched_before = 0, nseq = 0;
    for (uint32_t k = 0; k < nsegs; ++k) {
      const ZSeg m = meta[segbase + k];
      const uint32_t s0 = b0 + k * kSegBytes;
      S.seg_nseq[k] = m.nseq;
      S.seg_carry[k] = carry;
      S.seg_litout[k] = (s0 - b0) - matched_before; // literal slot of s0
      matched_before += m.matched;
      nseq += m.nseq;
      carry = m.nseq ? m.trailing : carry + m.trailing;
    }
    S.nseq = nseq;
    S.nlit = bsize - matched_before;
    S.all_same = 1;
  }
  __syncthreads();

  // RLE block test
  {
    // chunks are 16-byte aligned and blocks start at multiples of 128 KiB
    const uint8_t first = in[b0];
    const uint32_t pat = first * 0x01010101u;
    bool same = true;
    const uint32_t nv = bsize / 16;
    const uint4* v = reinterpret_cast<const uint4*>(in + b0);
    for (uint32_t i = tid; i < nv && same; i += blockDim.x) {
      const uint4 q = v[i];
      same = q.x == pat && q.y == pat && q.z == pat && q.w == pat;
    }
    for (uint32_t i = nv * 16 + tid; i < bsize && same; i += blockDim.x)
      same = in[b0 + i] == first;
    if (!same)
      S.all_same = 0;
  }

  // gather literals: warp k copies the literal bytes that lie inside its
  // own segment (the bytes before each match and after the last one), so
  // all warps work even when most segments have no match at all
  if (uint32_t(warp) < nsegs) {
    const uint32_t k = warp;
    const uint32_t s0 = b0 + k * kSegBytes;
    const uint32_t s1 = min(b1, s0 + kSegBytes);
    const Seq* sq = seqs + (segbase + k) * kMaxSeqPerSeg;
    const uint32_t nq = S.seg_nseq[k];
    uint32_t src = s0, dst = S.seg_litout[k];
    uint32_t* hist = S.whist[warp];
    for (uint32_t base = 0; base < nq; base += 32) {
      const uint32_t i = base + lane;
      uint32_t ll = 0, used = 0;
      if (i < nq) {
        const Seq q = sq[i];
        ll = q.lit; // this segment's own literals (no carry)
        used = ll + q.match;
      }
      uint32_t ex_in = used, ex_out = ll;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t a = __shfl_up_sync(0xffffffffu, ex_in, o);
        const uint32_t c = __shfl_up_sync(0xffffffffu, ex_out, o);
        if (lane >= o) {
          ex_in += a;
          ex_out += c;
        }
      }
      const uint32_t tot_in = __shfl_sync(0xffffffffu, ex_in, 31);
      const uint32_t tot_out = __shfl_sync(0xffffffffu, ex_out, 31);
      ex_in -= used;
      ex_out -= ll;
      unsigned pend = __ballot_sync(0xffffffffu, ll > 0);
      while (pend) {
        const int j = __ffs(pend) - 1;
        pend &= pend - 1;
        const uint32_t n = __shfl_sync(0xffffffffu, ll, j);
        const uint32_t si = __shfl_sync(0xffffffffu, ex_in, j);
        const uint32_t di = __shfl_sync(0xffffffffu, ex_out, j);
        gather_run(in, src + si, n, lits, dst + di, hist, lane);
      }
      src += tot_in;
      dst += tot_out;
    }
    // trailing literals of the segment (all of it when nothing matched)
    gather_run(in, src, s1 - src, lits, dst, hist, lane);
  }
  __syncthreads();
  for (int i = tid; i < 256; i += blockDim.x) {
    uint32_t t = 0;
    for (uint32_t w = 0; w < kSegsPerBlock; ++w)
      t += S.whist[w][i];
    S.hist[i] = t;
  }
  __syncthreads();
  // rank the used symbols by (count, symbol) in parallel for the Huffman
  // build (one comparison pass per symbol instead of a serial sort)
  for (int i = tid; i < 256; i += blockDim.x) {
    const uint32_t fi = S.hist[i];
    if (fi) {
      int rank = 0;
      for (int j = 0; j < 256; ++j) {
        const uint32_t fj = S.hist[j];
        rank += fj && (fj < fi || (fj == fi && j < i));
      }
      S.sorted[rank] = uint16_t(i);
    }
  }
  if (tid == 0) {
    uint32_t n = 0;
    for (int i = 0; i < 256; ++i)
      n += S.hist[i] > 0;
    S.nsym = n;
  }
  __syncthreads();

  const uint32_t nlit = S.nlit, nseq = S.nseq;
  if (tid == 0) {
    // literals section mode (the exact Huffman size decides below)
    S.lit_mode = 0;
    if (nlit > 0 && S.nsym == 1)
      S.lit_mode = 1;
    else if (nlit >= 256 &&
             huff_lengths(S.hist, S.sorted, S.nsym, S.huff, S.hx)) {
      huff_codes(S.huff, S.hx.rank_start, S.hx.count_w);
      if (huff_describe(S.huff, S.hx, S.tw))
        S.lit_mode = 2;
    }
  }
  __syncthreads();
  for (int c = tid; c < 256; c += blockDim.x)
    S.huff.cl[c] = uint32_t(S.huff.code[c]) | (uint32_t(S.huff.len[c]) << 16);
  __syncthreads();

  // ---- Huffman streams: bit lengths per stream (64 threads per stream)
  const uint32_t per = (nlit + 3) / 4;
  if (S.lit_mode == 2) {
    const int st = tid / kStreamThreads, t = tid % kStreamThreads;
    const uint32_t a0 = st * per;
    const uint32_t a1 = st == 3 ? nlit : min(nlit, a0 + per);
    const uint32_t m = a1 - a0;
    // this thread's share of the stream in writing order (reversed)
    const uint32_t q0 = uint32_t(uint64_t(m) * t / kStreamThreads);
    const uint32_t q1 = uint32_t(uint64_t(m) * (t + 1) / kStreamThreads);
    uint32_t bits = 0;
    const uint32_t* cl = S.huff.cl;
    for_each_desc(lits, a1 - q1, a1 - q0,
                  [&](uint8_t c) { bits += cl[c] >> 16; });
    // exclusive scan over the stream's warp
    uint32_t before = bits;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, before, o);
      if (t >= o)
        before += y;
    }
    if (t == kStreamThreads - 1)
      S.stream_bits[st] = before;
    before -= bits;
    __syncthreads();
    if (tid == 0) {
      // literals section layout
      uint32_t ssz[4], tot = 0;
      for (int s = 0; s < 4; ++s) {
        ssz[s] = S.stream_bits[s] / 8 + 1; // end mark + padding
        tot += ssz[s];
      }
      const uint32_t csize = S.huff.desc_len + 6 + tot;
      const uint32_t big = max(nlit, csize);
      const uint32_t hdr = big < 1024 ? 3 : (big < 16384 ? 4 : 5);
      S.lit_hdr = hdr;
      S.lit_size = hdr + csize;
      uint32_t pos = 3 + hdr + S.huff.desc_len + 6;
      for (int s = 0; s < 4; ++s) {
        S.stream_pos[s] = pos;
        pos += ssz[s];
      }
      if (csize + hdr >= nlit + 3) // not worth it
        S.lit_mode = 0;
      else {
        uint8_t* o = stage + 3;
        const uint32_t sf = hdr == 3 ? 1 : (hdr == 4 ? 2 : 3);
        const int nbits = hdr == 3 ? 10 : (hdr == 4 ? 14 : 18);
        const uint64_t h = 2u | (sf << 2) | (uint64_t(nlit) << 4) |
                           (uint64_t(csize) << (4 + nbits));
        put_le(o, h, hdr);
        o += hdr;
        for (int i = 0; i < S.huff.desc_len; ++i)
          o[i] = S.huff.desc[i];
        o += S.huff.desc_len;
        put_le(o, ssz[0], 2);
        put_le(o + 2, ssz[1], 2);
        put_le(o + 4, ssz[2], 2);
      }
    }
    // zero the stream area before the bit packing ORs into it
    __syncthreads();
    if (S.lit_mode == 2) {
      const uint32_t z0 = S.stream_pos[0];
      const uint32_t z1 = S.lit_size + 3;
      for (uint32_t i = z0 + tid; i < z1 + 4; i += blockDim.x)
        stage[i] = 0;
    }
    __syncthreads();
    if (S.lit_mode == 2) {
      uint8_t* sp = stage + S.stream_pos[st];
      // Bits of this thread: [before, before + bits) of the stream.  Whole
      // 32-bit words inside that range belong to this thread alone and are
      // stored plainly; the first and last (shared) words are OR-ed in.
      uint32_t* wbase = reinterpret_cast<uint32_t*>(
        reinterpret_cast<uintptr_t>(sp) & ~uintptr_t(3));
      const uint64_t skew = uint64_t(reinterpret_cast<uintptr_t>(sp) & 3) * 8;
      const uint64_t start = before + skew;
      uint64_t word = start >> 5;
      int fill = int(start & 31);
      const bool first_shared = fill != 0;
      bool first = true;
      uint64_t acc = 0;
      const uint32_t* cl = S.huff.cl;
      for_each_desc(lits, a1 - q1, a1 - q0, [&](uint8_t c) {
        const uint32_t e = cl[c];
        acc |= uint64_t(e & 0xFFFF) << fill;
        fill += int(e >> 16);
        if (fill >= 32) {
          if (first && first_shared)
            atomicOr(wbase + word, uint32_t(acc));
          else
            wbase[word] = uint32_t(acc);
          first = false;
          acc >>= 32;
          fill -= 32;
          ++word;
        }
      });
      if (t == kStreamThreads - 1) { // end mark after the stream's last bit
        acc |= uint64_t(1) << fill;
        fill += 1;
        if (fill >= 32) {
          if (first && first_shared)
            atomicOr(wbase + word, uint32_t(acc));
          else
            wbase[word] = uint32_t(acc);
          acc >>= 32;
          fill -= 32;
          ++word;
        }
      }
      if (fill > 0)
        atomicOr(wbase + word, uint32_t(acc));
    }
  } else if (tid == 0 && nlit > 0 && S.lit_mode == 0) {
    // nothing to lay out yet (raw literals below)
  }
  __syncthreads();

  // ---- raw / rle literals section
  if (S.lit_mode != 2) {
    const uint32_t hdr = nlit < 32 ? 1 : (nlit < 4096 ? 2 : 3);
    if (tid == 0) {
      const uint32_t type = S.lit_mode; // 0 raw, 1 rle
      uint64_t h;
      if (hdr == 1)
        h = type | (uint64_t(nlit) << 3);
      else if (hdr == 2)
        h = type | (1u << 2) | (uint64_t(nlit) << 4);
      else
        h = type | (3u << 2) | (uint64_t(nlit) << 4);
      put_le(stage + 3, h, int(hdr));
      S.lit_hdr = hdr;
      S.lit_size = hdr + (S.lit_mode == 1 ? 1 : nlit);
    }
    if (S.lit_mode == 1) {
      if (tid == 0)
        stage[3 + hdr] = lits[0];
    } else {
      for (uint32_t i = tid; i < nlit; i += blockDim.x)
        stage[3 + hdr + i] = lits[i];
    }
  }
  __syncthreads();

  // ---- sequences section (thread 0)
  if (tid == 0) {
    uint8_t* o = stage + 3 + S.lit_size;
    // every sequence takes at most 9 bytes of the bitstream
    const bool fits = 3 + uint64_t(S.lit_size) + 8 + 9 * uint64_t(nseq) <
                      kStageBytes;
    if (!fits)
      o = stage; // contents unused: the block is written raw below
    bool bad = false;
    if (nseq < 128)
      *o++ = uint8_t(nseq);
    else if (nseq < 0x7F00) {
      *o++ = uint8_t((nseq >> 8) + 128);
      *o++ = uint8_t(nseq);
    } else {
      *o++ = 255;
      put_le(o, nseq - 0x7F00, 2);
      o += 2;
    }
    if (nseq && fits) {
      *o++ = 0; // predefined LL, OF and ML tables
      const FseEnc& tll = S.pre.ll;
      const FseEnc& tml = S.pre.ml;
      const FseEnc& tof = S.pre.of;
      BitOut bo;
      bo.init(o);
      // walk the sequences backwards across segments
      uint32_t vll = 0, vml = 0, vof = 0;
      bool first = true;
      for (int k = int(nsegs) - 1; k >= 0 && !bad; --k) {
        const Seq* sq = seqs + (segbase + k) * kMaxSeqPerSeg;
        for (int i = int(S.seg_nseq[k]) - 1; i >= 0; --i) {
          const Seq q = sq[i];
          const uint32_t ll = q.lit + (i == 0 ? S.seg_carry[k] : 0);
          const uint32_t off = q.offset + 3;
          const int lc = ll_code(ll), mc = ml_code(q.match);
          const int oc = highbit(off);
          if (oc > 28 || q.match < 3 || q.offset == 0) { // cannot happen
            bad = true;
            break;
          }
          if (first) {
            vll = fse_init(tll, lc);
            vml = fse_init(tml, mc);
            vof = fse_init(tof, oc);
            first = false;
          } else {
            fse_encode(tof, vof, oc, bo);
            fse_encode(tml, vml, mc, bo);
            fse_encode(tll, vll, lc, bo);
          }
          bo.put(ll - kLLBase[lc], kLLBits[lc]);
          bo.put(q.match - kMLBase[mc], kMLBits[mc]);
          bo.put(off - (1u << oc), oc);
        }
      }
      bo.put(vml - 64, 6);
      bo.put(vof - 32, 5);
      bo.put(vll - 64, 6);
      o = bo.close();
    }
    uint32_t csize = (fits && !bad) ? uint32_t(o - (stage + 3)) : bsize;
    const bool last = b1 == b.chunk_bytes;
    uint32_t total;
    if (S.all_same) { // RLE block: one byte
      put_le(stage, (last ? 1u : 0u) | (1u << 1) | (bsize << 3), 3);
      stage[3] = in[b0];
      total = 4;
    } else if (csize >= bsize) { // raw block
      put_le(stage, (last ? 1u : 0u) | (bsize << 3), 3);
      total = 3 + bsize;
      S.lit_mode = 3; // marks "copy input" for the threads below
    } else {
      put_le(stage, (last ? 1u : 0u) | (2u << 1) | (csize << 3), 3);
      total = 3 + csize;
    }
    block_sizes[blk] = total;
  }
  __syncthreads();
  if (S.lit_mode == 3 && !S.all_same)
    for (uint32_t i = tid; i < bsize; i += blockDim.x)
      stage[3 + i] = in[b0 + i];
}

// ---------------------------------------------------------------------------
// frame: header + blocks
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256)
zstd_frame_k(CodecBatch b,
             const uint8_t* stage_all,
             const uint32_t* block_sizes,
             uint32_t blocks_per_chunk)
{
  __shared__ uint32_t offs[1024];
  const uint64_t chunk = blockIdx.x;
  uint8_t* out = b.out + b.id(chunk) * b.out_stride;
  const uint32_t n = b.chunk_bytes;
  if (threadIdx.x == 0) {
    // magic, descriptor (single segment), frame content size
    put_le(out, 0xFD2FB528u, 4);
    uint32_t h;
    if (n < 256) {
      out[4] = 0x20; // FCS flag 0, single segment
      out[5] = uint8_t(n);
      h = 6;
    } else if (n < 65536 + 256) {
      out[4] = 0x60; // FCS flag 1 (2 bytes, value - 256)
      put_le(out + 5, n - 256, 2);
      h = 7;
    } else {
      out[4] = 0xA0; // FCS flag 2 (4 bytes)
      put_le(out + 5, n, 4);
      h = 9;
    }
    uint32_t acc = h;
    for (uint32_t k = 0; k < blocks_per_chunk && k < 1024; ++k) {
      offs[k] = acc;
      acc += block_sizes[chunk * blocks_per_chunk + k];
    }
    b.out_sizes[b.id(chunk)] = acc;
  }
  __syncthreads();
  for (uint32_t k = 0; k < blocks_per_chunk; ++k) {
    const uint8_t* src = stage_all + (chunk * blocks_per_chunk + k) * kStageBytes;
    const uint32_t sz = block_sizes[chunk * blocks_per_chunk + k];
    copy_bytes(out + offs[k], src, sz, threadIdx.x, blockDim.x);
  }
}

} // namespace

size_t zstd_scratch_bytes(uint64_t n_chunks, uint32_t chunk_bytes)
{
  const uint64_t segs = n_chunks * ((chunk_bytes + kSegBytes - 1) / kSegBytes);
  const uint64_t blocks =
    n_chunks * ((chunk_bytes + kBlockBytes - 1) / kBlockBytes);
  return segs * (kMaxSeqPerSeg * sizeof(Seq) + sizeof(ZSeg)) +
         blocks * (kStageBytes + sizeof(uint32_t)) + 1024;
}

cudaError_t launch_zstd(CodecBatch b, void* scratch, cudaStream_t st)
{
  if (!b.n_chunks)
    return cudaSuccess;
  b.segs_per_chunk = (b.chunk_bytes + kSegBytes - 1) / kSegBytes;
  const uint32_t bpc = (b.chunk_bytes + kBlockBytes - 1) / kBlockBytes;
  if (bpc > 1024)
    return cudaErrorInvalidValue; // chunks above 128 MiB
  const uint64_t segs = b.n_chunks * b.segs_per_chunk;
  const uint64_t blocks = b.n_chunks * bpc;
  uint8_t* p = static_cast<uint8_t*>(scratch);
  Seq* seqs = reinterpret_cast<Seq*>(p);
  p += segs * kMaxSeqPerSeg * sizeof(Seq);
  ZSeg* meta = reinterpret_cast<ZSeg*>(p);
  p += segs * sizeof(ZSeg);
  p = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
  uint8_t* stage = p;
  p += blocks * kStageBytes;
  uint32_t* bsizes = reinterpret_cast<uint32_t*>(p);
  cudaError_t e;
  note_launches(3);
  CHUCKY_LAUNCH(zstd_find_k, unsigned((segs + kFindWarps - 1) / kFindWarps), 32 * kFindWarps, 0, st, b, seqs, meta);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  static const PredefTables pre = [] {
    PredefTables t{};
    uint8_t spread[64], fill[64];
    fse_build(t.ll, kLLNormH, 36, 6, spread, fill);
    fse_build(t.ml, kMLNormH, 53, 6, spread, fill);
    fse_build(t.of, kOFNormH, 29, 5, spread, fill);
    return t;
  }();
  CHUCKY_LAUNCH(zstd_block_k, unsigned(blocks), kBlockThreads, kBlockBytes + 16, st, b, pre, seqs, meta,
                                                           stage, bsizes, bpc);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  CHUCKY_LAUNCH(zstd_frame_k, unsigned(b.n_chunks), 256, 0, st, b, stage, bsizes, bpc);
  return cudaGetLastError();
}

} // namespace chucky
