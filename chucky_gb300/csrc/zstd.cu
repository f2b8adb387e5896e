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
#include "zstd_format.cuh"

namespace chucky {

namespace {

// 8 KiB blocks: a CTA per block, whose serial parts (the three FSE state
// chains) grow with the block's sequences
constexpr uint32_t kBlockLog = 13;
constexpr uint32_t kBlockBytes = 1u << kBlockLog; // 8 KiB
constexpr uint32_t kSegsPerBlock = kBlockBytes / kSegBytes;
// staging of one compressed block: a block that carries its chunk's
// Huffman description is never replaced by a raw block, so it must fit
// however large it comes out (literals <= 11/8 of their bytes, sequences
// <= 9 bytes each)
constexpr uint32_t kStageBytes = 3 * kBlockBytes + 1024;
constexpr int kStreamThreads = 32;                // a warp per Huffman stream
constexpr int kBlockThreads = 4 * kStreamThreads; // >= a warp per segment
constexpr int kTableThreads = 256;                // a thread per symbol
static_assert(kBlockThreads >= 32 * int(kSegsPerBlock), "warp per segment");
static_assert(kStreamThreads % 32 == 0, "whole warps per stream");
// fewest literals coded with the chunk's Huffman table
constexpr uint32_t kMinHufLits = 64;
// chunks at least this large share one Huffman description: the first
// block that codes literals with it carries it, later blocks refer to it
// (treeless literals); smaller chunks describe the table in every block
constexpr uint32_t kTreelessMinChunk = 64u << 10;
constexpr uint32_t kHufMaxBits = 11;
#ifndef CHUCKY_ZSTD_MIN_MATCH
#define CHUCKY_ZSTD_MIN_MATCH 8
#endif
// Matches shorter than this cost about as much as a sequence (predefined
// FSE codes of its three fields plus the offset's extra bits, about 30
// bits) as their bytes cost as Huffman-coded literals, and every match
// restarts the dense probing of the parser.  8 bytes: on 12-bit sensor
// frames the encoders run 1.45x faster with a better ratio than with 6,
// on the u16/f32 cubes 5 % faster for 0.06 % of ratio.
constexpr uint32_t kMinMatch = CHUCKY_ZSTD_MIN_MATCH;

// Per chunk: 256 literal counts of a 1-in-4 sample of the literal bytes,
// then a 256-bit map of every literal byte value present.
constexpr uint32_t kHistWords = 256 + 8;

struct ZSeg
{
  uint32_t nseq, trailing, matched; // matched = bytes covered by matches
  // bits 0-7 first literal byte, bit 8 every literal equals it (or none);
  // bits 16-23 first input byte, bit 24 every input byte equals it
  uint32_t flags;
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

// Literal-length and match-length codes (RFC 8878 3.1.1.3.2.1.1): the
// base-value tables in closed form.
__host__ __device__ __forceinline__ int ll_code(uint32_t ll)
{
  if (ll < 16)
    return int(ll);
  if (ll >= 64)
    return highbit(ll) + 19;
  if (ll < 24)
    return 16 + int((ll - 16) >> 1);
  if (ll < 32)
    return 20 + int((ll - 24) >> 2);
  if (ll < 48)
    return 22 + int((ll - 32) >> 3);
  return 24;
}

__host__ __device__ __forceinline__ int ml_code(uint32_t ml) // ml >= 3
{
  const uint32_t mb = ml - 3;
  if (mb < 32)
    return int(mb);
  if (mb >= 128)
    return highbit(mb) + 36;
  if (mb < 40)
    return 32 + int((mb - 32) >> 1);
  if (mb < 48)
    return 36 + int((mb - 40) >> 2);
  if (mb < 64)
    return 38 + int((mb - 48) >> 3);
  if (mb < 96)
    return 40 + int((mb - 64) >> 4);
  return 42;
}

template<int kStates>
struct FseEncT
{
  int al;
  int16_t count[64];        // normalized count per symbol (-1 stored as 1)
  uint16_t first[64];       // index of the symbol's first state in `states`
  uint8_t states[kStates];  // states of each symbol, ascending, grouped by symbol
};
using FseEnc = FseEncT<64>;  // accuracy log <= 6: Huffman weights
using SeqEnc = FseEncT<256>; // accuracy log <= 8: sequence codes
constexpr int kSeqMaxLog = 8;

// Build encoder tables from normalized counts (-1 = "less than 1").
// `spread` (1 << al entries) and `fill` (nsym entries) are scratch arrays
// (shared memory on the device: local arrays of one thread would miss L1).
template<int kStates>
__host__ __device__ inline void fse_build(FseEncT<kStates>& t,
                                          const int16_t* norm,
                                          int nsym,
                                          int al,
                                          uint8_t* spread,
                                          uint16_t* fill)
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
    t.first[s] = uint16_t(acc);
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
  SeqEnc ll, ml, of;
};

template<int kStates>
__device__ __forceinline__ uint32_t fse_init(const FseEncT<kStates>& t, int s)
{
  return t.states[t.first[s]] + (1u << t.al);
}

// ---------------------------------------------------------------------------
// find
// ---------------------------------------------------------------------------

// One CTA per region, a warp per segment.  Besides the sequences, every
// segment leaves its literal bytes, compacted, in its slot of `litbuf`
// (kSegBytes each), adds them to its chunk's literal histogram
// (`chunk_hist`, kHistWords per chunk, zeroed before the launch) and
// records whether its input and its literals are single-valued.
// Levels 3 and up parse with the wide window (the 7 regions before each
// one: matches up to 112-128 KiB back) and accept matches from
// kMinMatchWide bytes; levels below with the region's own window.
constexpr uint32_t kZstdWideBack = 7;
constexpr int kZstdWideLog = 14;
#ifndef CHUCKY_ZSTD_MIN_MATCH_WIDE
#define CHUCKY_ZSTD_MIN_MATCH_WIDE 4
#endif
constexpr uint32_t kMinMatchWide = CHUCKY_ZSTD_MIN_MATCH_WIDE;
__host__ __device__ inline bool zstd_wide(int level) { return level >= 3; }
// Per-chunk counts of the sequence codes (levels with the wide window):
// LL codes at 0, ML codes at kSeqHistML, OF codes at kSeqHistOF; a word
// set when a sequence cannot be coded.
constexpr uint32_t kSeqHistML = 36, kSeqHistOF = 36 + 53, kSeqHistBad = 36 + 53 + 32;
constexpr uint32_t kSeqHistWords = 128;

__global__ void __launch_bounds__(32 * kSegsPerRegion)
zstd_find_k(CodecBatch b,
            Seq* seqs,
            ZSeg* meta,
            uint32_t* chunk_hist,
            uint8_t* litbuf,
            uint32_t regions_per_chunk,
            const uint16_t* wide_tables, // null: the region's own window only
            uint32_t* seq_hist)          // null: no sequence-code histograms
{
  __shared__ __align__(16) uint16_t tables[kSegsPerRegion][1 << kHashLog];
  __shared__ uint32_t seg_nseq[kSegsPerRegion], seg_trail[kSegsPerRegion];
  __shared__ uint32_t shist[kSeqHistWords];
  CHUCKY_DYN_SHARED(uint32_t, words); // kRegionStageWords
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t chunk = blockIdx.x / regions_per_chunk;
  const uint32_t r0 = (blockIdx.x % regions_per_chunk) * kRegionBytes;
  const uint8_t* base = b.in_at(chunk);
  const uint32_t r1 = min(b.chunk_bytes, r0 + kRegionBytes);
  lz77_stage_region(base, r0, r1, words, threadIdx.x, blockDim.x);
  const uint32_t s0 = r0 + w * kSegBytes;
  const bool has = s0 < r1;
  const uint32_t s1 = has ? min(r1, s0 + kSegBytes) : s0;
  const uint64_t seg = chunk * b.segs_per_chunk + s0 / kSegBytes;
  Seq* out = seqs + (has ? seg : 0) * kMaxSeqPerSeg;
  SegInfo info{ 0, 0 };
  if (has) {
    const WideWindow W{ base,
                        wide_tables ? wide_tables + chunk * regions_per_chunk *
                                                      wide_entries(kZstdWideLog)
                                    : nullptr,
                        uint32_t(r0 / kRegionBytes), kZstdWideBack,
                        (kZstdWideBack + 1) * kRegionBytes, kZstdWideLog };
    const uint32_t mm = wide_tables ? kMinMatchWide
                                    : (b.min_match >= 4 ? uint32_t(b.min_match) : kMinMatch);
    info = lz77_parse_segment(words, r0, s0, s1, s1, s1, tables[w], out, mm,
                              wide_tables ? &W : nullptr,
                              b.strength > 0 ? b.strength : kSearchStrength);
  }
  if (lane == 0) {
    seg_nseq[w] = info.nseq;
    seg_trail[w] = info.trailing;
  }
  if (seq_hist)
    for (int i = threadIdx.x; i < int(kSeqHistWords); i += blockDim.x)
      shist[i] = 0;
  __syncthreads(); // the region is no longer needed as history
  if (seq_hist && has) {
    // codes of the segment's sequences (as the block kernel forms them:
    // the first takes the literals carried from the block's earlier
    // segments since its last sequence), counted per CTA
    uint32_t carry = 0;
    for (int k = w - w % int(kSegsPerBlock); k < w; ++k)
      carry = seg_nseq[k] ? seg_trail[k] : carry + seg_trail[k];
    for (uint32_t i0 = 0; i0 < info.nseq; i0 += 32) {
      const uint32_t i = i0 + lane;
      const bool v = i < info.nseq;
      unsigned code[3] = { ~0u, ~0u, ~0u };
      if (v) {
        const Seq x = out[i];
        const uint32_t ll = x.lit + (i == 0 ? carry : 0), ml = x.match, off = x.offset + 3;
        const int oc = highbit(off);
        if (oc > 28 || ml < 3 || off <= 3)
          shist[kSeqHistBad] = 1;
        code[0] = unsigned(ll_code(ll));
        code[1] = kSeqHistML + unsigned(ml < 3 ? 0 : ml_code(ml));
        code[2] = kSeqHistOF + unsigned(oc);
      }
#pragma unroll
      for (int t = 0; t < 3; ++t) { // lanes past the sequences carry ~0u
        const unsigned peers = __match_any_sync(0xffffffffu, code[t]);
        if (v && lane == __ffs(int(peers)) - 1)
          atomicAdd(&shist[code[t]], uint32_t(__popc(peers)));
      }
    }
  }
  uint32_t* bitmap = reinterpret_cast<uint32_t*>(tables[w]);
  uint32_t* hist = bitmap + (kSegBytes / 32 + 31) / 32 * 32; // after the bitmap
  uint32_t* pres = hist + 256;
  static_assert((kSegBytes / 32 + 31) / 32 * 32 + 256 + 8 <= (1u << kHashLog) / 2,
                "bitmap, histogram and presence map fit in a warp's table");
  for (int i = lane; i < 256 + 8; i += 32)
    hist[i] = 0;
  __syncwarp();
  if (has) {
    uint32_t matched = 0;
    for (uint32_t i = lane; i < info.nseq; i += 32)
      matched += out[i].match;
    for (int o = 16; o; o >>= 1)
      matched += __shfl_xor_sync(0xffffffffu, matched, o);
    // single-valued input?
    const uint8_t* sb = reinterpret_cast<const uint8_t*>(words) + (s0 - r0);
    const uint32_t n = s1 - s0;
    const uint8_t in0 = sb[0];
    const uint32_t pat = in0 * 0x01010101u;
    const uint32_t* sw = words + (s0 - r0) / 4;
    // (without matches the literals are the input: the literal pass below
    // answers it)
    bool same = true;
    if (info.nseq) {
      for (uint32_t i = lane; i < n / 4; i += 32)
        same &= sw[i] == pat;
      for (uint32_t i = n / 4 * 4 + lane; i < n; i += 32)
        same &= sb[i] == in0;
    }
    bool in_same = __all_sync(0xffffffffu, same);
    // literals: compacted in place, counted, copied out
    const uint32_t nlit =
      lz77_compact_literals(words, r0, s0, s1, out, info.nseq, bitmap);
    __syncwarp();
    // literal statistics, a word (4 bytes) per lane and step: every value
    // present marks the presence map (one atomic the first time it is seen
    // by this warp), one byte per word, rotating through the four byte
    // positions, is counted; and whether the literals are all one value
    const uint8_t lit0 = nlit ? sb[0] : 0;
    const uint32_t pat0 = lit0 * 0x01010101u;
    same = true;
    const uint32_t* lw = reinterpret_cast<const uint32_t*>(sb);
    for (uint32_t i = lane; i < (nlit + 3) / 4; i += 32) {
      const uint32_t v = lw[i];
      const uint32_t nb = min(4u, nlit - 4 * i); // bytes of this word in use
      const uint32_t keep = nb == 4 ? 0xFFFFFFFFu : (1u << (8 * nb)) - 1;
      same &= ((v ^ pat0) & keep) == 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (uint32_t(k) < nb) {
          const uint32_t c = (v >> (8 * k)) & 255;
          const uint32_t bit = 1u << (c & 31);
          if (!(pres[c >> 5] & bit))
            atomicOr(pres + (c >> 5), bit);
        }
      }
      const uint32_t k = i & 3;
      if (k < nb)
        atomicAdd(hist + ((v >> (8 * k)) & 255), 1u);
    }
    const bool lit_same = __all_sync(0xffffffffu, same);
    if (!info.nseq)
      in_same = lit_same;
    const uint4* src = reinterpret_cast<const uint4*>(sb);
    uint4* dst = reinterpret_cast<uint4*>(litbuf + seg * kSegBytes);
    for (uint32_t i = lane; i < (nlit + 15) / 16; i += 32)
      dst[i] = src[i];
    if (lane == 0)
      meta[seg] = ZSeg{ info.nseq, info.trailing, matched,
                        uint32_t(lit0) | (lit_same ? 1u << 8 : 0u) |
                          (uint32_t(in0) << 16) | (in_same ? 1u << 24 : 0u) };
  }
  // the CTA's literal statistics, added to its chunk's once
  __syncthreads();
  uint32_t* ch = chunk_hist + chunk * kHistWords;
  for (int i = threadIdx.x; i < int(kHistWords); i += blockDim.x) {
    uint32_t t = 0;
    for (int v = 0; v < int(kSegsPerRegion); ++v) {
      const uint32_t x =
        (reinterpret_cast<uint32_t*>(tables[v]) + (kSegBytes / 32 + 31) / 32 * 32)[i];
      t = i < 256 ? t + x : t | x;
    }
    if (t) {
      if (i < 256)
        atomicAdd(ch + i, t);
      else
        atomicOr(ch + i, t);
    }
  }
  if (seq_hist) // the CTA's code counts, added to its chunk's
    for (int i = threadIdx.x; i < int(kSeqHistWords); i += blockDim.x)
      if (shist[i]) {
        if (i == int(kSeqHistBad))
          seq_hist[chunk * kSeqHistWords + i] = 1;
        else
          atomicAdd(seq_hist + chunk * kSeqHistWords + i, shist[i]);
      }
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

// Normalize a histogram of weights to 2^al, every present symbol >= 1 and
// no symbol above half the table (so every state reads >= 1 bit and the
// decoder's end-of-stream test fires exactly after the last weight).
__device__ void norm_weights(const uint32_t* hist_s, int nsym, int al, int16_t* norm_s)
{
  // nsym <= 16: counts and the result live in registers (every index below
  // is a compile-time constant after unrolling), so the serial loops do not
  // wait on shared memory
  const int size = 1 << al, half = size / 2;
  uint32_t hist[16];
  int norm[16];
  uint32_t total = 0;
  int present = 0;
#pragma unroll
  for (int s = 0; s < 16; ++s) {
    hist[s] = s < nsym ? hist_s[s] : 0u;
    total += hist[s];
    present += hist[s] > 0;
  }
  int sum = 0;
#pragma unroll
  for (int s = 0; s < 16; ++s) {
    int c = 0;
    if (hist[s]) {
      // weight counts (<= 256) times the table size (<= 64): 32 bits do
      c = int((hist[s] * uint32_t(size) + total / 2) / total);
      c = c < 1 ? 1 : (c > half ? half : c);
    }
    norm[s] = c;
    sum += c;
  }
  if (present == 1) { // a second symbol takes the other half
    bool done = false;
#pragma unroll
    for (int s = 0; s < 16; ++s)
      if (!done && s < nsym && !hist[s]) {
        norm[s] = size - sum;
        sum = size;
        done = true;
      }
  }
  while (sum > size) { // take from the largest
    int best = -1, bv = 0;
#pragma unroll
    for (int s = 0; s < 16; ++s)
      if (norm[s] > 1 && (best < 0 || norm[s] > bv)) {
        best = s;
        bv = norm[s];
      }
#pragma unroll
    for (int s = 0; s < 16; ++s)
      if (s == best)
        norm[s]--;
    --sum;
  }
  while (sum < size) { // give to the most under-represented that has room
    int best = -1;
    uint32_t bh = 0;
    int bn = 0;
#pragma unroll
    for (int s = 0; s < 16; ++s)
      if (hist[s] && norm[s] < half &&
          (best < 0 || uint64_t(hist[s]) * uint64_t(bn) > uint64_t(bh) * uint64_t(norm[s]))) {
        best = s;
        bh = hist[s];
        bn = norm[s];
      }
    if (best < 0) // everything capped: an absent symbol takes the rest
#pragma unroll
      for (int s = 0; s < 16; ++s)
        if (best < 0 && s < nsym && !hist[s] && norm[s] < half)
          best = s;
#pragma unroll
    for (int s = 0; s < 16; ++s)
      if (s == best)
        norm[s]++;
    ++sum;
  }
#pragma unroll
  for (int s = 0; s < 16; ++s)
    if (s < nsym)
      norm_s[s] = int16_t(norm[s]);
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

// FSE bookkeeping of the weights description (the state chain runs on one
// thread; the bits are then packed by all threads).
struct WeightChain
{
  uint16_t enc[256]; // per step: low bits | bit count << 8
  uint32_t nsteps, ncount_len, fin1, fin2, maxw, warp_bits[8];
  uint32_t high;            // highest position of the regular symbols
  uint32_t spread_ballot0;  // valid walk positions among the first 32
};

// ---------------------------------------------------------------------------
// block
// ---------------------------------------------------------------------------

// Huffman table of a chunk's literals, built once per chunk
// (zstd_table_k) and used by every block of the chunk.
struct ChunkTable
{
  uint32_t cl[256];    // code | length << 16; 0 for absent symbols
  uint8_t desc[320];   // tree description (header byte + payload)
  uint32_t desc_len;
  uint32_t ok;         // a usable table exists and beats raw literals
  uint32_t carrier;    // block carrying the description (treeless chunks);
                       // ~0u: every Huffman block carries it
};

// Literal count and single-valuedness of block `bi` of a chunk from its
// segments' metadata.
__device__ __forceinline__ void block_literals(const ZSeg* meta,
                                               uint64_t seg_first,
                                               uint32_t chunk_bytes,
                                               uint32_t bi,
                                               uint32_t& nlit,
                                               bool& same)
{
  const uint32_t b0 = bi * kBlockBytes;
  const uint32_t b1 = min(chunk_bytes, b0 + kBlockBytes);
  const uint32_t nsegs = (b1 - b0 + kSegBytes - 1) / kSegBytes;
  const uint64_t sb = seg_first + b0 / kSegBytes;
  nlit = 0;
  same = true;
  int byte = -1;
  for (uint32_t k = 0; k < nsegs; ++k) {
    const ZSeg m = meta[sb + k];
    const uint32_t s0 = b0 + k * kSegBytes;
    const uint32_t nl = min(b1, s0 + kSegBytes) - s0 - m.matched;
    nlit += nl;
    if (nl) {
      if (byte < 0)
        byte = int(m.flags & 0xFF);
      same &= ((m.flags >> 8) & 1) && (m.flags & 0xFF) == uint32_t(byte);
    }
  }
}

// Whether block literals are coded with the chunk's Huffman table.
__device__ __forceinline__ bool block_uses_table(bool table_ok, uint32_t nlit, bool same)
{
  return table_ok && !same && nlit >= kMinHufLits;
}

struct TableShared
{
  alignas(16) uint32_t hist[256];
  uint16_t sorted[256]; // used symbols by (count, symbol)
  uint32_t nsym, total;
  uint32_t ok;
  unsigned long long bits; // coded size of the chunk's literals
  uint32_t carrier;
  WeightChain wc;
  FseEnc tw;            // Huffman weights table
  HuffScratch hx;
  Huff huff;
};

struct BlockShared
{
  uint32_t cl[256];                   // the chunk's Huffman codes
  PredefTables seqt;                  // the chunk's sequence tables (LL, ML, OF)
  uint32_t seq_modes;                 // modes byte of a block with sequences
  uint32_t seq_desc;                  // description bytes after it (carrier)
  uint32_t seg_nseq[kSegsPerBlock];
  uint32_t seg_seq0[kSegsPerBlock];   // block index of the segment's first sequence
  uint32_t seg_carry[kSegsPerBlock];
  uint32_t seg_litout[kSegsPerBlock]; // literal buffer offset of seg start
  uint32_t nseq, nlit;
  uint32_t stream_bits[4];
  uint32_t stream_pos[4]; // byte offset of each Huffman stream in staging
  uint32_t lit_mode;      // 0 raw, 1 rle, 2 huffman
  uint32_t lit_hdr;       // literals section header bytes
  uint32_t lit_size;      // literals section bytes (header included)
  uint32_t lit_same;      // every literal equals the first
  uint32_t lit_missing;   // a literal has no code in the chunk's table
  uint32_t with_desc;     // the literals section describes the table
  uint32_t forced;        // description carrier: never a raw block
  uint32_t all_same;
  // sequences section
  uint32_t ll_base[36], ml_base[53];
  uint8_t ll_bits[36], ml_bits[53];
  uint32_t final_state[3];    // LL, ML, OF states after the last step
  uint32_t warp_bits[kBlockThreads / 32];
  uint32_t seq_bad;
  uint32_t seq_csize;         // compressed block bytes (after the header)
};

__device__ __forceinline__ void put_le(uint8_t* p, uint64_t v, int n)
{
  for (int i = 0; i < n; ++i)
    p[i] = uint8_t(v >> (8 * i));
}

// Bit packing into a stream shared by many threads (zstd's backward-read
// bitstreams are written forward, least significant bit first; the decoder
// starts at the end mark).  Each thread owns a contiguous bit range
// [start, start + n) of the stream at `p` (zeroed beforehand).  Words
// wholly inside the range are stored plainly; the first (shared with the
// bytes or thread before) and the last are OR-ed in.
struct BitPack
{
  uint32_t* w;
  uint64_t acc, word;
  int fill;
  bool first;
  __device__ void init(uint8_t* p, uint32_t start_bit)
  {
    w = reinterpret_cast<uint32_t*>(reinterpret_cast<uintptr_t>(p) & ~uintptr_t(3));
    const uint64_t pos = uint64_t(reinterpret_cast<uintptr_t>(p) & 3) * 8 + start_bit;
    word = pos >> 5;
    fill = int(pos & 31);
    first = fill != 0;
    acc = 0;
  }
  // n <= 32
  __device__ __forceinline__ void put(uint32_t v, int n)
  {
    acc |= (uint64_t(v) & ((uint64_t(1) << n) - 1)) << fill;
    fill += n;
    if (fill >= 32) {
      if (first)
        atomicOr(w + word, uint32_t(acc));
      else
        w[word] = uint32_t(acc);
      first = false;
      acc >>= 32;
      fill -= 32;
      ++word;
    }
  }
  __device__ void flush()
  {
    if (fill > 0)
      atomicOr(w + word, uint32_t(acc));
  }
};

// Literal length (with the carry into a segment's first sequence), match
// length and offset value (offset + 3, no repeat offsets) of block
// sequence j.
__device__ __forceinline__ void seq_at(const BlockShared& S,
                                       const Seq* seqs,
                                       uint64_t segbase,
                                       uint32_t nsegs,
                                       uint32_t j,
                                       uint32_t& ll,
                                       uint32_t& ml,
                                       uint32_t& off)
{
  uint32_t k = 0;
  while (k + 1 < nsegs && j >= S.seg_seq0[k + 1])
    ++k;
  const uint32_t i = j - S.seg_seq0[k];
  const Seq q = seqs[(segbase + k) * kMaxSeqPerSeg + i];
  ll = q.lit + (i == 0 ? S.seg_carry[k] : 0);
  ml = q.match;
  off = q.offset + 3;
}

// Low bits of FSE state u (v = u + table size) when encoding `sym`.
template<int kStates, typename F>
__device__ __forceinline__ int state_bits(const FseEncT<kStates>& t, uint32_t u, int sym,
                                          F& put)
{
  const uint32_t v = u + (1u << t.al);
  const int c = t.count[sym];
  int nb = t.al - highbit(uint32_t(c));
  if ((v >> nb) < uint32_t(c))
    --nb;
  put(v, nb);
  return nb;
}

// Bits of block sequence j in stream order (RFC 8878 3.1.1.3.2.1): for all
// but the block's last sequence (the stream's first) the OF, ML and LL
// state bits, then the LL, ML and OF extra bits.  `st` holds the state each
// sequence starts from ([3][nseq]: LL, ML, OF).  Returns the bit count.
template<typename F>
__device__ __forceinline__ uint32_t seq_emit(const BlockShared& S,
                                             const Seq* seqs,
                                             uint64_t segbase,
                                             uint32_t nsegs,
                                             uint32_t nseq,
                                             const uint8_t* st,
                                             uint32_t j,
                                             F&& put)
{
  uint32_t ll, ml, off;
  seq_at(S, seqs, segbase, nsegs, j, ll, ml, off);
  const int lc = ll_code(ll), mc = ml_code(ml);
  const int oc = highbit(off);
  uint32_t bits = 0;
  if (j + 1 < nseq) {
    bits += state_bits(S.seqt.of, st[2 * nseq + j], oc, put);
    bits += state_bits(S.seqt.ml, st[nseq + j], mc, put);
    bits += state_bits(S.seqt.ll, st[j], lc, put);
  }
  const int lb = S.ll_bits[lc], mb = S.ml_bits[mc];
  put(ll - S.ll_base[lc], lb);
  put(ml - S.ml_base[mc], mb);
  put(off - (1u << oc), oc);
  return bits + lb + mb + oc;
}

// Visit lits[hi-1], lits[hi-2], ..., lits[lo] (descending): the unaligned
// ends byte by byte through f1, every whole aligned 16-byte word of the
// shared-memory literal buffer at once through f16 (which takes its bytes
// 15, 14, ..., 0).
template<typename F1, typename F16>
__device__ __forceinline__ void visit_desc(const uint8_t* lits,
                                           uint32_t lo,
                                           uint32_t hi,
                                           F1&& f1,
                                           F16&& f16)
{
  uint32_t a = hi;
  while (a > lo && (a & 15))
    f1(lits[--a]);
  while (a >= lo + 16) {
    a -= 16;
    f16(*reinterpret_cast<const uint4*>(lits + a));
  }
  while (a > lo)
    f1(lits[--a]);
}

// One CTA per chunk: the length-limited Huffman code of the chunk's
// literal histogram and its tree description (thread 0 builds, the rest
// rank the symbols and publish the table).
// Tree description (RFC 8878 4.2.1): direct 4-bit weights for up to 128
// weights, else the weights FSE-compressed (accuracy log 6, two
// interleaved states).  x.w holds the weights of symbols 0 .. h.last - 1.
// All threads of the CTA call it; it sets T.ok to 0 when the description
// does not fit.
__device__ void huff_describe(TableShared& T, int tid)
{
  Huff& h = T.huff;
  HuffScratch& x = T.hx;
  WeightChain& c = T.wc;
  const int nw = h.last;
  const uint8_t* w = x.w;
  const int lane = tid & 31, warp = tid >> 5;
  if (nw <= 128) {
    if (tid < (nw + 1) / 2) {
      const uint8_t hi = w[2 * tid], lo = 2 * tid + 1 < nw ? w[2 * tid + 1] : 0;
      h.desc[1 + tid] = uint8_t(hi << 4 | lo);
    }
    if (tid == 0) {
      h.desc[0] = uint8_t(127 + nw);
      h.desc_len = 1 + (nw + 1) / 2;
    }
    __syncthreads();
    return;
  }
  if (tid < 16)
    x.whist[tid] = 0;
  if (tid == 0)
    c.maxw = 0;
  __syncthreads();
  {
    // weight histogram and largest weight: one shared atomic per distinct
    // weight and warp (a few weights shared by many symbols serialise)
    const uint32_t key = tid < nw ? uint32_t(w[tid]) : ~0u;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (tid < nw && lane == __ffs(int(peers)) - 1)
      atomicAdd(&x.whist[key], uint32_t(__popc(peers)));
    uint32_t mx = tid < nw ? uint32_t(w[tid]) : 0u;
    for (int o = 16; o; o >>= 1)
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0 && mx)
      atomicMax(&c.maxw, mx);
  }
  __syncthreads();
  constexpr int al = 6;
  uint8_t* out = h.desc + 1;
  const int nsym = int(c.maxw) + 2 <= 13 ? int(c.maxw) + 2 : 13; // room for a spare symbol
  constexpr int size = 1 << al;
  FseEnc& t = T.tw;
  if (tid == 0) {
    norm_weights(x.whist, nsym, al, x.norm);
    // counts, first states, and the top positions of "less than 1" symbols
    int acc = 0, high = size - 1;
    for (int sy = 0; sy < nsym; ++sy) {
      t.count[sy] = x.norm[sy] == -1 ? 1 : x.norm[sy];
      t.first[sy] = uint8_t(acc);
      acc += t.count[sy];
      if (x.norm[sy] == -1)
        x.spread[high--] = uint8_t(sy);
    }
    c.high = uint32_t(high);
    t.al = al;
    c.ncount_len = uint32_t(write_ncount(out, x.norm, nsym, al));
    c.nsteps = uint32_t(nw - 2);
  }
  __syncthreads();
  // The symbol spread of fse_build in parallel: position j of the walk
  // (j * step mod size) is the rank-th valid one (<= high), and the rank-th
  // valid position goes to the symbol whose cumulative count covers it.
  constexpr int step = (size >> 1) + (size >> 3) + 3;
  static_assert(size == 64, "two warps walk the table");
  if (warp == 0) { // valid walk positions among the first 32
    const uint32_t pos = uint32_t(tid * step) & (size - 1);
    const unsigned m = __ballot_sync(0xffffffffu, pos <= c.high);
    if (lane == 0)
      c.spread_ballot0 = m;
  }
  __syncthreads();
  if (tid < size) {
    const uint32_t pos = uint32_t(tid * step) & (size - 1);
    const bool valid = pos <= c.high;
    const unsigned m = __ballot_sync(0xffffffffu, valid);
    const uint32_t rank =
      __popc(m & ((1u << lane) - 1)) + (warp == 1 ? __popc(c.spread_ballot0) : 0);
    if (valid) {
      int sy = 0;
      uint32_t cum = 0;
      for (; sy < nsym; ++sy) {
        const uint32_t n = x.norm[sy] > 0 ? uint32_t(x.norm[sy]) : 0;
        if (rank < cum + n)
          break;
        cum += n;
      }
      x.spread[pos] = uint8_t(sy);
    }
  }
  __syncthreads();
  // states of each symbol in increasing position order
  if (tid < size) {
    const int sy = x.spread[tid];
    int before = 0;
    for (int u = 0; u < tid; ++u)
      before += x.spread[u] == sy;
    t.states[t.first[sy] + before] = uint8_t(tid);
  }
  __syncthreads();
  // The two interleaved state chains, last weight first, one lane each:
  // the chain initialised with weight nw-1 encodes the even steps (weights
  // nw-3, nw-5, ...), the one initialised with weight nw-2 the odd steps
  // (nw-4, nw-6, ...).  Each step's bits are recorded for the packing
  // below.  The stream closes with state 2 then state 1, where state 1 is
  // the even-step chain when nw is odd and the odd-step chain when even.
  if (tid < 2) {
    const FseEnc& t = T.tw;
    const int par = tid; // 0: even steps, 1: odd steps
    uint32_t v = fse_init(t, w[nw - 1 - par]);
    // the next step's weight, count and first state are loaded a step
    // ahead (they do not depend on the state), so each step waits on one
    // shared-memory load: the state transition
    int idx = nw - 3 - par;
    int s_n = idx >= 0 ? w[idx] : 0;
    int cnt_n = t.count[s_n], first_n = t.first[s_n];
    for (int k = par; idx >= 0; k += 2, idx -= 2) {
      const int cnt = cnt_n, first = first_n;
      if (idx >= 2) {
        s_n = w[idx - 2];
        cnt_n = t.count[s_n];
        first_n = t.first[s_n];
      }
      int nb = al - highbit(uint32_t(cnt));
      if ((v >> nb) < uint32_t(cnt))
        --nb;
      c.enc[k] = uint16_t((v & ((1u << nb) - 1)) | (uint32_t(nb) << 8));
      v = t.states[first + ((v >> nb) - cnt)] + (1u << al);
    }
    const bool state1 = (nw & 1) ? par == 0 : par == 1;
    if (state1)
      c.fin1 = v - (1u << al);
    else
      c.fin2 = v - (1u << al);
  }
  __syncthreads();
  // pack: thread k writes step k's bits at the sum of the steps before it
  const uint32_t ns = c.nsteps, len = c.ncount_len;
  const uint32_t e = uint32_t(tid) < ns ? c.enc[tid] : 0;
  const uint32_t nb = e >> 8;
  uint32_t before = nb;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, before, o);
    if (lane >= o)
      before += y;
  }
  if (lane == 31)
    c.warp_bits[warp] = before;
  before -= nb;
  for (uint32_t i = 1 + len + tid; i < sizeof(h.desc); i += blockDim.x)
    h.desc[i] = 0;
  __syncthreads();
  uint32_t total = 0;
  for (int v = 0; v < kTableThreads / 32; ++v) {
    if (v < warp)
      before += c.warp_bits[v];
    total += c.warp_bits[v];
  }
  const uint32_t bytes = (total + 2 * al + 1 + 7) / 8;
  const bool fits = 1 + len + bytes + 4 <= sizeof(h.desc) && len + bytes < 128;
  if (fits && (uint32_t(tid) < ns || (ns == 0 && tid == 0))) {
    BitPack bp;
    bp.init(out + len, before);
    bp.put(e & 0xFF, int(nb));
    if (uint32_t(tid) + 1 == ns || ns == 0) { // final states, end mark
      bp.put(c.fin2, al);
      bp.put(c.fin1, al);
      bp.put(1, 1);
    }
    bp.flush();
  }
  __syncthreads();
  if (tid == 0) {
    if (fits) {
      h.desc[0] = uint8_t(len + bytes);
      h.desc_len = int(1 + len + bytes);
    } else {
      T.ok = 0;
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kTableThreads)
zstd_table_k(CodecBatch b,
             const uint32_t* chunk_hist,
             const ZSeg* meta,
             ChunkTable* tables,
             uint32_t blocks_per_chunk)
{
  static_assert(kTableThreads >= 256, "a thread per symbol");
  __shared__ TableShared T;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t chunk = blockIdx.x;
  HuffScratch& x = T.hx;
  Huff& h = T.huff;
  if (tid < 256) {
    // four times the sampled count, and at least 1 for every value present
    const uint32_t* ch = chunk_hist + chunk * kHistWords;
    T.hist[tid] = 4 * ch[tid] + ((ch[256 + (tid >> 5)] >> (tid & 31)) & 1);
    h.len[tid] = 0;
  }
  if (tid < 16)
    x.count_w[tid] = x.whist[tid] = 0;
  if (tid == 0)
    T.nsym = T.total = 0;
  __syncthreads();
  // rank the used symbols by (count, symbol); count them
  if (tid < 256) {
    const uint32_t fi = T.hist[tid];
    if (fi) {
      // four counts per shared load
      int rank = 0;
      const uint4* h4 = reinterpret_cast<const uint4*>(T.hist);
#pragma unroll 8
      for (int q = 0; q < 64; ++q) {
        const uint4 v = h4[q];
        const uint32_t fv[4] = { v.x, v.y, v.z, v.w };
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const uint32_t fj = fv[u];
          const int j = 4 * q + u;
          rank += fj && (fj < fi || (fj == fi && j < tid));
        }
      }
      T.sorted[rank] = uint16_t(tid);
    }
  }
  {
    // the used symbols and their total count: warp sums, one shared atomic
    // per warp (256 on one address serialise)
    const uint32_t fi = tid < 256 ? T.hist[tid] : 0;
    uint32_t cnt = fi ? 1u : 0u, tot = fi;
    for (int o = 16; o; o >>= 1) {
      cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (lane == 0 && cnt) {
      atomicAdd(&T.nsym, cnt);
      atomicAdd(&T.total, tot);
    }
  }
  __syncthreads();
  const int n = int(T.nsym);
  const bool build = n >= 2 && T.total >= 256;
  // Huffman tree by the two-queue method on the sorted leaves (serial):
  // leaves 0 .. n-1 (ascending count), internal nodes n .. 2n-2 (root)
  if (build && tid < n)
    x.f[tid] = T.hist[T.sorted[tid]];
  __syncthreads();
  if (build && tid == 0) {
    uint32_t* f = x.f;
    int16_t* parent = x.parent;
    // The first two entries of both queues stay in registers (empty: ~0u),
    // so taking an entry never waits for a shared-memory load: the entry
    // after the new head is loaded then and needed one take later.
    int leaf = 0, inode = n, next = n;
    uint32_t fl = f[0], fl2 = n > 1 ? f[1] : ~0u, fi = ~0u, fi2 = ~0u;
    for (int k = 0; k < n - 1; ++k) {
      int pick[2];
      uint32_t val[2];
      for (int t = 0; t < 2; ++t) {
        if (fl <= fi) { // ties take the leaf
          pick[t] = leaf;
          val[t] = fl;
          ++leaf;
          fl = fl2;
          fl2 = leaf + 1 < n ? f[leaf + 1] : ~0u;
        } else {
          pick[t] = inode;
          val[t] = fi;
          ++inode;
          fi = fi2;
          fi2 = inode + 1 < next ? f[inode + 1] : ~0u;
        }
      }
      const uint32_t sum = val[0] + val[1];
      f[next] = sum;
      parent[pick[0]] = parent[pick[1]] = int16_t(next);
      if (inode == next) // the internal queue was empty: this node heads it
        fi = sum;
      else if (inode + 1 == next) // it is the queue's second entry
        fi2 = sum;
      ++next;
    }
    parent[2 * n - 2] = int16_t(2 * n - 2); // the root is its own parent
  }
  __syncthreads();
  if (!build) {
    if (tid == 0)
      T.ok = 0;
  } else {
    // leaf depths by pointer jumping (depth <= 255 < 2^8)
    const int nodes = 2 * n - 1;
    uint8_t* dist = x.depth;
    for (int i = tid; i < nodes; i += blockDim.x)
      dist[i] = i == nodes - 1 ? 0 : 1;
    __syncthreads();
    for (int r = 0; r < 8; ++r) {
      int16_t np[2];
      uint8_t nd[2];
      for (int k = 0; k < 2; ++k) {
        const int i = tid + k * int(blockDim.x);
        if (i < nodes) {
          const int p = x.parent[i];
          nd[k] = uint8_t(dist[i] + dist[p]);
          np[k] = x.parent[p];
        }
      }
      __syncthreads();
      for (int k = 0; k < 2; ++k) {
        const int i = tid + k * int(blockDim.x);
        if (i < nodes) {
          dist[i] = nd[k];
          x.parent[i] = np[k];
        }
      }
      __syncthreads();
    }
    // lengths per depth, leaves deeper than kHufMaxBits clamped: one
    // shared atomic per depth and warp
    {
      const uint32_t d = tid < n ? uint32_t(dist[tid]) : 0u;
      const uint32_t key = tid < n ? (d > kHufMaxBits ? kHufMaxBits : d) : ~0u;
      const unsigned peers = __match_any_sync(0xffffffffu, key);
      if (tid < n && lane == __ffs(int(peers)) - 1)
        atomicAdd(&x.count_w[key], uint32_t(__popc(peers)));
    }
    __syncthreads();
    if (tid == 0) {
      // The clamped leaves overfill the code by `excess` units of
      // 2^-kHufMaxBits.  Each step splits the deepest leaf above the limit
      // into two leaves one level down, one of them taken from the limit
      // (as zlib's gen_bitlen repairs its length counts): one unit less.
      uint32_t* bl = x.count_w;
      constexpr int M = int(kHufMaxBits);
      // the counts stay in registers through the repair (every index
      // below is a compile-time constant after unrolling)
      uint32_t r[M + 1];
#pragma unroll
      for (int L = 0; L <= M; ++L)
        r[L] = bl[L];
      uint32_t units = 0;
#pragma unroll
      for (int L = 1; L <= M; ++L)
        units += r[L] << (M - L);
      for (uint32_t excess = units - (1u << M); int(excess) > 0; --excess) {
        int bits = 0; // the deepest level above the limit with a leaf
#pragma unroll
        for (int L = 1; L < M; ++L)
          if (r[L])
            bits = L;
        if (bits == 0 || r[M] == 0)
          break;
#pragma unroll
        for (int L = 1; L < M; ++L)
          if (L == bits) {
            r[L]--;
            r[L + 1] += 2;
          }
        r[M]--;
      }
#pragma unroll
      for (int L = 0; L <= M; ++L)
        bl[L] = r[L];
      int mb = 0;
      uint32_t kraft = 0;
      for (int L = 1; L <= int(kHufMaxBits); ++L)
        if (bl[L])
          mb = L;
      for (int L = 1; L <= mb; ++L)
        kraft += bl[L] << (mb - L);
      h.max_bits = mb;
      T.ok = kraft == (1u << mb) && bl[0] == 0 ? 1 : 0;
      // rank_start[w]: canonical start of weight w = mb + 1 - length
      uint32_t acc = 0;
      for (int w = 1; w <= mb; ++w) {
        x.rank_start[w] = acc;
        acc += bl[mb + 1 - w] << (w - 1);
      }
    }
    __syncthreads();
    // the least frequent symbols get the longest codes
    if (T.ok && tid < n) {
      uint32_t cum = 0;
      int L = int(kHufMaxBits);
      for (; L > 0; --L) {
        cum += x.count_w[L];
        if (uint32_t(tid) < cum)
          break;
      }
      h.len[T.sorted[tid]] = uint8_t(L);
    }
    __syncthreads();
    // canonical codes in zstd's order: by weight, then by symbol
    const int mb = h.max_bits;
    const int sym = tid; // < 256
    const int len = sym < 256 ? h.len[sym] : 0;
    const int wt = len ? mb + 1 - len : 0;
    uint32_t* cnt = x.f; // [warps][16] counts per weight
    uint32_t below = 0;
    for (int w = 1; w <= mb; ++w) {
      const unsigned m = __ballot_sync(0xffffffffu, wt == w);
      if (wt == w)
        below = __popc(m & ((1u << lane) - 1));
      if (lane == 0)
        cnt[warp * 16 + w] = __popc(m);
    }
    __syncthreads();
    if (sym < 256 && len > 0) {
      for (int v = 0; v < warp; ++v)
        below += cnt[v * 16 + wt];
      h.code[sym] = uint16_t((x.rank_start[wt] >> (wt - 1)) + below);
    }
    // the highest coded symbol; weights of the symbols below it
    if (tid == 0)
      h.last = 0;
    __syncthreads();
    {
      // warp maximum first: one shared atomic per warp
      uint32_t mx = sym < 256 && len > 0 ? uint32_t(sym) : 0u;
      for (int o = 16; o; o >>= 1)
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0 && mx)
        atomicMax(&h.last, mx);
    }
    // (h.last is read after the barrier below)
    __syncthreads();
    if (sym < h.last)
      x.w[sym] = uint8_t(wt);
    __syncthreads();
    if (T.ok)
      huff_describe(T, tid);
    // worth it: the coded literals (and one description) beat raw bytes
    if (tid == 0)
      T.bits = 0;
    __syncthreads();
    {
      // one shared atomic per warp: 256 on one address serialise
      unsigned long long cb =
        T.ok && sym < 256 && len > 0 ? (unsigned long long)T.hist[sym] * uint32_t(len) : 0;
      for (int o = 16; o; o >>= 1)
        cb += __shfl_xor_sync(0xffffffffu, cb, o);
      if (lane == 0 && cb)
        atomicAdd(&T.bits, cb);
    }
    __syncthreads();
    if (tid == 0 && T.ok)
      T.ok = T.bits / 8 + uint32_t(h.desc_len) + 16 < uint64_t(T.total);
  }
  // the description carrier: the chunk's first block coding its literals
  // with the table
  if (tid == 0)
    T.carrier = ~0u;
  __syncthreads();
  if (T.ok && b.chunk_bytes >= kTreelessMinChunk) {
    const uint64_t seg_first = chunk * b.segs_per_chunk;
    for (uint32_t bi = tid; bi < blocks_per_chunk; bi += blockDim.x) {
      uint32_t nlit;
      bool same;
      block_literals(meta, seg_first, b.chunk_bytes, bi, nlit, same);
      if (block_uses_table(true, nlit, same))
        atomicMin(&T.carrier, bi);
    }
  }
  __syncthreads();
  ChunkTable& ct = tables[chunk];
  if (tid < 256)
    ct.cl[tid] = T.ok ? uint32_t(h.code[tid]) | (uint32_t(h.len[tid]) << 16) : 0;
  const int dl = T.ok ? h.desc_len : 0;
  for (int i = tid; i < dl; i += blockDim.x)
    ct.desc[i] = h.desc[i];
  if (tid == 0) {
    ct.desc_len = uint32_t(dl);
    ct.ok = T.ok;
    ct.carrier = T.carrier;
  }
}

// ---- adaptive sequence tables (levels with the wide window) ---------------
//
// The wide window's parse yields many short matches whose codes are far from
// the predefined distributions.  A CTA per chunk counts the chunk's
// literal-length, match-length and offset codes and normalizes each
// histogram into an FSE table (RFC 8878 4.1.1) wherever that beats the
// predefined table, description included.  The chunk's first block with
// sequences that is not an RLE block (the carrier, never replaced by a raw
// block) describes the tables (FSE_Compressed mode); every later block
// refers to them (Repeat mode).  A repeated table is the one of the previous
// compressed block with sequences, which is the carrier or a block that
// repeated it.

struct ChunkSeq
{
  SeqEnc t[3];          // LL, ML, OF encoders
  uint8_t desc[3][96];  // descriptions of the described tables (LL, ML, OF)
  uint32_t desc_len[3];
  uint32_t mode[3];     // 0 predefined, 2 described by the carrier
  uint32_t carrier;     // block describing the tables; ~0u: none
};

struct SeqTabShared
{
  uint32_t hist[kSeqHistWords];
  uint32_t carrier;
  int16_t norm[3][64];
  uint8_t spread[3][256];
  uint16_t fill[3][64];
  ChunkSeq cs;
};

// Normalize counts to 2^al (al large enough that 2^al >= 2 nsym): every
// present symbol >= 1, no "less than 1" symbols; a lone symbol shares the
// table with an absent one, so that no table is single-valued.  nsym >= 2.
__device__ void norm_seq(const uint32_t* hist, int nsym, int al, int16_t* norm)
{
  const int size = 1 << al;
  uint64_t total = 0;
  int present = 0, only = 0;
  for (int s = 0; s < nsym; ++s) {
    total += hist[s];
    if (hist[s]) {
      ++present;
      only = s;
    }
  }
  int sum = 0;
  for (int s = 0; s < nsym; ++s) {
    int c = 0;
    if (hist[s]) {
      c = int((uint64_t(hist[s]) * uint64_t(size) + total / 2) / total);
      c = c < 1 ? 1 : c;
    }
    norm[s] = int16_t(c);
    sum += c;
  }
  if (present == 1) {
    for (int s = 0; s < nsym; ++s)
      norm[s] = 0;
    norm[only] = int16_t(size - 1);
    norm[only == 0 ? 1 : 0] = 1;
    return;
  }
  while (sum > size) { // take from the largest
    int best = -1;
    for (int s = 0; s < nsym; ++s)
      if (norm[s] > 1 && (best < 0 || norm[s] > norm[best]))
        best = s;
    norm[best]--;
    --sum;
  }
  while (sum < size) { // give to the most under-represented
    int best = -1;
    for (int s = 0; s < nsym; ++s)
      if (hist[s] && (best < 0 || uint64_t(hist[s]) * uint64_t(norm[best]) >
                                    uint64_t(hist[best]) * uint64_t(norm[s])))
        best = s;
    norm[best]++;
    ++sum;
  }
}

// Coded bits of a histogram under normalized counts of accuracy log al
// (a count of -1 codes like 1).
__device__ float fse_cost(const uint32_t* hist, int nhist, const int16_t* norm, int nsym,
                          int al)
{
  float c = 0.f;
  for (int s = 0; s < nhist; ++s)
    if (hist[s]) {
      if (s >= nsym)
        return 3.0e38f;
      const int n = norm[s] < 1 ? 1 : norm[s];
      c += float(hist[s]) * (float(al) - log2f(float(n)));
    }
  return c;
}

__global__ void __launch_bounds__(kTableThreads)
zstd_seqtab_k(CodecBatch b,
              const ZSeg* meta,
              const uint32_t* seq_hist,
              ChunkSeq* out,
              uint32_t blocks_per_chunk)
{
  __shared__ SeqTabShared T;
  const int tid = threadIdx.x;
  const uint64_t chunk = blockIdx.x;
  for (int i = tid; i < int(kSeqHistWords); i += blockDim.x)
    T.hist[i] = seq_hist[chunk * kSeqHistWords + i];
  if (tid == 0)
    T.carrier = ~0u;
  __syncthreads();
  // the carrier: the first block with sequences that is not an RLE block
  // (its segments' records, as the block kernel reads them)
  const uint64_t seg_first = chunk * b.segs_per_chunk;
  for (uint32_t bi = tid; bi < blocks_per_chunk; bi += blockDim.x) {
    const uint32_t b0 = bi * kBlockBytes;
    const uint32_t b1 = min(b.chunk_bytes, b0 + kBlockBytes);
    const uint32_t nsegs = (b1 - b0 + kSegBytes - 1) / kSegBytes;
    const uint64_t sb = seg_first + b0 / kSegBytes;
    const uint32_t in0 = (meta[sb].flags >> 16) & 0xFF;
    uint32_t nseq = 0, all_same = 1;
    for (uint32_t k = 0; k < nsegs; ++k) {
      const ZSeg m = meta[sb + k];
      all_same &= (m.flags >> 24) & (((m.flags >> 16) & 0xFF) == in0);
      nseq += m.nseq;
    }
    if (nseq && !all_same)
      atomicMin(&T.carrier, bi);
  }
  __syncthreads();
  if (tid < 3) { // a thread per table
    const int t = tid;
    const int nhist = t == 0 ? 36 : (t == 1 ? 53 : 32);
    const int pre_n = t == 0 ? 36 : (t == 1 ? 53 : 29);
    const int pre_al = t == 2 ? 5 : 6;
    const int16_t* pre = t == 0 ? kLLNormD : (t == 1 ? kMLNormD : kOFNormD);
    const uint32_t* h = T.hist + (t == 0 ? 0 : (t == 1 ? kSeqHistML : kSeqHistOF));
    uint64_t total = 0;
    int last = -1;
    for (int s = 0; s < nhist; ++s) {
      total += h[s];
      if (h[s])
        last = s;
    }
    SeqEnc& e = T.cs.t[t];
    uint32_t mode = 0;
    if (!T.hist[kSeqHistBad] && T.carrier != ~0u && last >= 0) {
      const int nsym = last + 1 > 2 ? last + 1 : 2;
      const uint32_t tot32 = total > 0xFFFFFFFFull ? 0xFFFFFFFFu : uint32_t(total);
      int al = tot32 > 32 ? highbit(tot32) - 2 : 5;
      const int lo = highbit(uint32_t(nsym - 1)) + 2;
      al = al < lo ? lo : al;
      al = al < 5 ? 5 : (al > kSeqMaxLog ? kSeqMaxLog : al);
      norm_seq(h, nsym, al, T.norm[t]);
      const int dl = write_ncount(T.cs.desc[t], T.norm[t], nsym, al);
      const float custom = fse_cost(h, nhist, T.norm[t], nsym, al) + 8.f * float(dl);
      const float predefined = fse_cost(h, nhist, pre, pre_n, pre_al);
      if (custom + 32.f < predefined) {
        mode = 2;
        fse_build(e, T.norm[t], nsym, al, T.spread[t], T.fill[t]);
        T.cs.desc_len[t] = uint32_t(dl);
      }
    }
    if (mode == 0) {
      fse_build(e, pre, pre_n, pre_al, T.spread[t], T.fill[t]);
      T.cs.desc_len[t] = 0;
    }
    T.cs.mode[t] = mode;
  }
  __syncthreads();
  if (tid == 0)
    T.cs.carrier = T.cs.mode[0] | T.cs.mode[1] | T.cs.mode[2] ? T.carrier : ~0u;
  __syncthreads();
  static_assert(sizeof(ChunkSeq) % 4 == 0, "word copy");
  const uint32_t* src = reinterpret_cast<const uint32_t*>(&T.cs);
  uint32_t* dst = reinterpret_cast<uint32_t*>(out + chunk);
  for (int i = tid; i < int(sizeof(ChunkSeq) / 4); i += blockDim.x)
    dst[i] = src[i];
}

// 12 CTAs per SM (40 registers, a few spilled): the block kernel waits at
// its phase barriers, and more resident CTAs cover those waits (measured
// 3 % faster on the cube workload than 8 CTAs with 64 registers)
#ifndef CHUCKY_BLOCK_MIN_CTAS
#define CHUCKY_BLOCK_MIN_CTAS 12
#endif
__global__ void __launch_bounds__(kBlockThreads, CHUCKY_BLOCK_MIN_CTAS)
zstd_block_k(CodecBatch b,
             const __grid_constant__ PredefTables pre,
             const Seq* seqs,
             const ZSeg* meta,
             const ChunkTable* tables,
             const ChunkSeq* cseq, // adaptive sequence tables; null: predefined
             const uint8_t* litbuf,
             uint8_t* stage_all,
             uint32_t* block_sizes,
             uint32_t blocks_per_chunk)
{
  __shared__ BlockShared S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t blk = blockIdx.x;
  const uint64_t chunk = blk / blocks_per_chunk;
  const uint32_t bi = uint32_t(blk % blocks_per_chunk);
  const uint8_t* in = b.in_at(chunk);
  const uint32_t b0 = bi * kBlockBytes;
  const uint32_t b1 = min(b.chunk_bytes, b0 + kBlockBytes);
  const uint32_t bsize = b1 - b0;
  const uint32_t seg0 = b0 / kSegBytes;
  const uint32_t nsegs = (bsize + kSegBytes - 1) / kSegBytes;
  const uint64_t segbase = chunk * b.segs_per_chunk + seg0;
  CHUCKY_DYN_SHARED(uint8_t, lits); // this block's literals
  uint8_t* stage = stage_all + blk * kStageBytes;

  const ChunkTable& ct = tables[chunk];
  for (int c = tid; c < 256; c += blockDim.x)
    S.cl[c] = ct.cl[c];
  // the three sequence tables: the chunk's (adaptive) or the predefined
  // ones (built once on the host)
  {
    static_assert(sizeof(PredefTables) == 3 * sizeof(SeqEnc), "LL, ML, OF in a row");
    const uint32_t* src = cseq ? reinterpret_cast<const uint32_t*>(cseq[chunk].t)
                               : reinterpret_cast<const uint32_t*>(&pre);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&S.seqt);
    for (int i = tid; i < int(sizeof(PredefTables) / 4); i += blockDim.x)
      dst[i] = src[i];
  }
  if (tid == 0) {
    // modes byte (LL, OF, ML in bits 7-6, 5-4, 3-2): a described table is
    // FSE_Compressed in the carrier and Repeat after it
    uint32_t modes = 0, desc = 0;
    if (cseq && cseq[chunk].carrier != ~0u) {
      const ChunkSeq& c = cseq[chunk];
      const bool carrier = bi == c.carrier;
      const uint32_t m = carrier ? 2u : 3u;
      modes = (c.mode[0] ? m << 6 : 0u) | (c.mode[2] ? m << 4 : 0u) |
              (c.mode[1] ? m << 2 : 0u);
      if (carrier)
        desc = c.desc_len[0] + c.desc_len[1] + c.desc_len[2];
    }
    S.seq_modes = modes;
    S.seq_desc = desc;
  }
  for (int i = tid; i < 53; i += blockDim.x) {
    S.ml_base[i] = kMLBase[i];
    S.ml_bits[i] = kMLBits[i];
    if (i < 36) {
      S.ll_base[i] = kLLBase[i];
      S.ll_bits[i] = kLLBits[i];
    }
  }
  if (tid == 0) {
    // the block's segment records, loaded together
    ZSeg ms[kSegsPerBlock];
#pragma unroll
    for (uint32_t k = 0; k < kSegsPerBlock; ++k)
      if (k < nsegs)
        ms[k] = meta[segbase + k];
    uint32_t carry = 0, matched_before = 0, nseq = 0;
#pragma unroll
    for (uint32_t k = 0; k < kSegsPerBlock; ++k) {
      if (k >= nsegs)
        break;
      const ZSeg m = ms[k];
      const uint32_t s0 = b0 + k * kSegBytes;
      S.seg_nseq[k] = m.nseq;
      S.seg_seq0[k] = nseq;
      S.seg_carry[k] = carry;
      S.seg_litout[k] = (s0 - b0) - matched_before; // literal slot of s0
      matched_before += m.matched;
      nseq += m.nseq;
      carry = m.nseq ? m.trailing : carry + m.trailing;
    }
    S.nseq = nseq;
    S.nlit = bsize - matched_before;
    // single-valued input (RLE block) and literals (RLE literals section)
    uint32_t all_same = 1, lit_same = 1;
    int lit_byte = -1;
    const uint32_t in0 = (ms[0].flags >> 16) & 0xFF;
#pragma unroll
    for (uint32_t k = 0; k < kSegsPerBlock; ++k) {
      if (k >= nsegs)
        break;
      const ZSeg m = ms[k];
      const uint32_t s0 = b0 + k * kSegBytes;
      const uint32_t nl = min(b1, s0 + kSegBytes) - s0 - m.matched;
      all_same &= (m.flags >> 24) & ((m.flags >> 16) & 0xFF) == in0;
      if (nl) {
        if (lit_byte < 0)
          lit_byte = int(m.flags & 0xFF);
        lit_same &= (m.flags >> 8) & ((m.flags & 0xFF) == uint32_t(lit_byte));
      }
    }
    S.all_same = all_same;
    S.lit_same = lit_same;
    S.lit_missing = 0;
    S.seq_bad = 0;
  }
  __syncthreads();

  // literals: a warp per segment copies the segment's compacted literals
  if (uint32_t(warp) < nsegs) {
    const uint32_t k = warp;
    const uint32_t s0 = b0 + k * kSegBytes;
    const uint32_t nl = min(b1, s0 + kSegBytes) - s0 - meta[segbase + k].matched;
    copy_bytes(lits + S.seg_litout[k], litbuf + (segbase + k) * kSegBytes, nl, lane, 32);
  }
  __syncthreads();
  const uint32_t nlit = S.nlit, nseq = S.nseq;
  if (tid == 0) {
    // literals section mode (the exact Huffman size decides below).  In a
    // treeless chunk the carrier block describes the table and is always
    // kept as a compressed block; later blocks refer to its description.
    S.lit_mode = 0;
    S.with_desc = 1;
    S.forced = 0;
    if (nlit > 0 && S.lit_same)
      S.lit_mode = 1;
    else if (block_uses_table(ct.ok, nlit, false)) {
      S.lit_mode = 2;
      if (ct.carrier != ~0u) {
        S.with_desc = bi == ct.carrier;
        S.forced = bi == ct.carrier;
      }
    }
    // the block describing the chunk's sequence tables stays compressed too
    if (S.seq_desc)
      S.forced = 1;
  }
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
    uint32_t bits = 0, missing = 0; // missing: a literal without a code
    const uint32_t* cl = S.cl;
    visit_desc(
      lits, a1 - q1, a1 - q0,
      [&](uint8_t c) {
        const uint32_t L = cl[c] >> 16;
        bits += L;
        missing |= L == 0;
      },
      [&](const uint4& w) {
        uint32_t s4[4] = { 0, 0, 0, 0 };
        const uint32_t v[4] = { w.x, w.y, w.z, w.w };
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const uint32_t L = cl[(v[i] >> (8 * k)) & 255] >> 16;
            s4[i] += L;
            missing |= L == 0;
          }
        bits += s4[0] + s4[1] + s4[2] + s4[3];
      });
    if (missing) // the chunk's table does not cover these literals
      S.lit_missing = 1;
    // exclusive scan over the stream's threads (whole warps)
    uint32_t before = bits;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, before, o);
      if (lane >= o)
        before += y;
    }
    if (lane == 31)
      S.warp_bits[warp] = before;
    before -= bits;
    __syncthreads();
    constexpr int kStreamWarps = kStreamThreads / 32;
    for (int w = st * kStreamWarps; w < warp; ++w)
      before += S.warp_bits[w];
    if (tid < 4) {
      uint32_t sb = 0;
      for (int w = 0; w < kStreamWarps; ++w)
        sb += S.warp_bits[tid * kStreamWarps + w];
      S.stream_bits[tid] = sb;
    }
    __syncthreads();
    if (tid == 0) {
      // literals section layout
      uint32_t ssz[4], tot = 0;
      for (int s = 0; s < 4; ++s) {
        ssz[s] = S.stream_bits[s] / 8 + 1; // end mark + padding
        tot += ssz[s];
      }
      const uint32_t dlen = S.with_desc ? ct.desc_len : 0;
      const uint32_t csize = dlen + 6 + tot;
      const uint32_t big = max(nlit, csize);
      const uint32_t hdr = big < 1024 ? 3 : (big < 16384 ? 4 : 5);
      S.lit_hdr = hdr;
      S.lit_size = hdr + csize;
      uint32_t pos = 3 + hdr + dlen + 6;
      for (int s = 0; s < 4; ++s) {
        S.stream_pos[s] = pos;
        pos += ssz[s];
      }
      // not worth it / a literal without a code (the carrier keeps its
      // table: later blocks of the chunk depend on its description)
      if (!S.forced && (csize + hdr >= nlit + 3 || S.lit_missing))
        S.lit_mode = 0;
      else {
        uint8_t* o = stage + 3;
        const uint32_t sf = hdr == 3 ? 1 : (hdr == 4 ? 2 : 3);
        const int nbits = hdr == 3 ? 10 : (hdr == 4 ? 14 : 18);
        const uint32_t type = S.with_desc ? 2u : 3u; // compressed / treeless
        const uint64_t h = type | (sf << 2) | (uint64_t(nlit) << 4) |
                           (uint64_t(csize) << (4 + nbits));
        put_le(o, h, hdr);
        o += hdr + dlen; // the description is copied by all threads below
        put_le(o, ssz[0], 2);
        put_le(o + 2, ssz[1], 2);
        put_le(o + 4, ssz[2], 2);
      }
    }
    // copy the tree description; zero the stream area before the bit
    // packing ORs into it (16-byte stores between byte-wise ends)
    __syncthreads();
    if (S.lit_mode == 2) {
      const uint32_t dlen = S.with_desc ? ct.desc_len : 0;
      for (uint32_t i = tid; i < dlen; i += blockDim.x)
        stage[3 + S.lit_hdr + i] = ct.desc[i];
      const uint32_t z0 = S.stream_pos[0];
      const uint32_t z1 = S.lit_size + 3 + 4;
      const uint32_t v0 = min(z1, (z0 + 15) & ~15u), v1 = max(v0, z1 & ~15u);
      if (tid < v0 - z0)
        stage[z0 + tid] = 0;
      if (tid < z1 - v1)
        stage[v1 + tid] = 0;
      uint4* zv = reinterpret_cast<uint4*>(stage + v0);
      for (uint32_t i = tid; i < (v1 - v0) / 16; i += blockDim.x)
        zv[i] = make_uint4(0, 0, 0, 0);
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
      const uint32_t* cl = S.cl;
      auto flush = [&]() {
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
      };
      // codes are at most 11 bits: two fit before a flush (fill < 54)
      auto put = [&](uint32_t e) {
        acc |= uint64_t(e & 0xFFFF) << fill;
        fill += int(e >> 16);
      };
      visit_desc(
        lits, a1 - q1, a1 - q0,
        [&](uint8_t c) {
          put(cl[c]);
          flush();
        },
        [&](const uint4& w) {
          const uint32_t v[4] = { w.w, w.z, w.y, w.x };
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            put(cl[v[i] >> 24]);
            put(cl[(v[i] >> 16) & 255]);
            flush();
            put(cl[(v[i] >> 8) & 255]);
            put(cl[v[i] & 255]);
            flush();
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

  // ---- sequences section.  The three FSE state chains (LL, ML, OF) are
  // serial by nature: lanes 0-2 of warp 0 walk them side by side and record
  // the state every sequence starts from.  Everything else -- codes, bit
  // counts, the block-wide scan of bit positions and the bit packing -- runs
  // on all threads.  The literal buffer is free again (the literals are in
  // staging) and holds the per-sequence codes, then the states.
  uint8_t* scode = lits; // [3][nseq]: LL, ML, OF codes -> states (in place)
  for (uint32_t j = tid; j < nseq; j += blockDim.x) {
    uint32_t ll, ml, off;
    seq_at(S, seqs, segbase, nsegs, j, ll, ml, off);
    const int oc = highbit(off);
    if (oc > 28 || ml < 3 || off <= 3)
      S.seq_bad = 1;
    scode[j] = uint8_t(ll_code(ll));
    scode[nseq + j] = uint8_t(ml < 3 ? 0 : ml_code(ml));
    scode[2 * nseq + j] = uint8_t(oc);
  }
  __syncthreads();
  if (warp == 0 && lane < 3 && nseq) {
    const SeqEnc& t = lane == 0 ? S.seqt.ll : (lane == 1 ? S.seqt.ml : S.seqt.of);
    uint8_t* a = scode + lane * nseq;
    const uint32_t size = 1u << t.al;
    uint32_t v = t.states[t.first[a[nseq - 1]]] + size;
    for (int j = int(nseq) - 2; j >= 0; --j) {
      const int sym = a[j];
      a[j] = uint8_t(v - size);
      const int c = t.count[sym];
      int nb = t.al - highbit(uint32_t(c));
      if ((v >> nb) < uint32_t(c))
        --nb;
      v = t.states[t.first[sym] + ((v >> nb) - c)] + size;
    }
    S.final_state[lane] = v - size;
  }
  __syncthreads();
  // sequence p of the stream is block sequence nseq - 1 - p (written
  // backwards); thread tid packs the stream sequences [p0, p1)
  const uint32_t p0 = uint32_t(uint64_t(nseq) * tid / kBlockThreads);
  const uint32_t p1 = uint32_t(uint64_t(nseq) * (tid + 1) / kBlockThreads);
  uint32_t my_bits = 0;
  for (uint32_t p = p0; p < p1; ++p)
    my_bits += seq_emit(S, seqs, segbase, nsegs, nseq, scode, nseq - 1 - p,
                        [](uint32_t, int) {});
  uint32_t before = my_bits;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, before, o);
    if (lane >= o)
      before += y;
  }
  if (lane == 31)
    S.warp_bits[warp] = before;
  before -= my_bits;
  __syncthreads();
  uint32_t total_bits = 0;
  for (int w = 0; w < kBlockThreads / 32; ++w) {
    if (w < warp)
      before += S.warp_bits[w];
    total_bits += S.warp_bits[w];
  }
  // header: sequence count, then the modes byte and (carrier) the table
  // descriptions
  const uint32_t seq_at0 = 3 + S.lit_size;
  const uint32_t nhdr =
    nseq == 0 ? 1 : (nseq < 128 ? 2 : (nseq < 0x7F00 ? 3 : 4)) + S.seq_desc;
  const uint32_t bs0 = seq_at0 + nhdr; // first byte of the bitstream
  // final states and the end mark
  const uint32_t fin_bits = uint32_t(S.seqt.ll.al + S.seqt.ml.al + S.seqt.of.al);
  const uint32_t nbytes = nseq ? (total_bits + fin_bits + 1 + 7) / 8 : 0;
  const bool fits = bs0 + nbytes + 4 <= kStageBytes && !S.seq_bad;
  if (fits) {
    if (tid == 0) {
      uint8_t* o = stage + seq_at0;
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
      if (nseq) {
        *o++ = uint8_t(S.seq_modes);
        if (S.seq_desc) { // descriptions in the order LL, OF, ML
          const ChunkSeq& c = cseq[chunk];
          const int order[3] = { 0, 2, 1 };
          for (int k = 0; k < 3; ++k)
            for (uint32_t i = 0; i < c.desc_len[order[k]]; ++i)
              *o++ = c.desc[order[k]][i];
        }
      }
    }
    const uint32_t z1 = bs0 + nbytes + 4;
    const uint32_t v0 = min(z1, (bs0 + 15) & ~15u), v1 = max(v0, z1 & ~15u);
    if (tid < v0 - bs0)
      stage[bs0 + tid] = 0;
    if (tid < z1 - v1)
      stage[v1 + tid] = 0;
    uint4* zv = reinterpret_cast<uint4*>(stage + v0);
    for (uint32_t i = tid; i < (v1 - v0) / 16; i += blockDim.x)
      zv[i] = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  if (fits && nseq) {
    BitPack bp;
    bp.init(stage + bs0, before);
    for (uint32_t p = p0; p < p1; ++p)
      seq_emit(S, seqs, segbase, nsegs, nseq, scode, nseq - 1 - p,
               [&](uint32_t v, int n) { bp.put(v, n); });
    if (p1 == nseq && p1 > p0) { // the stream's last sequence: states, end mark
      bp.put(S.final_state[1], S.seqt.ml.al);
      bp.put(S.final_state[2], S.seqt.of.al);
      bp.put(S.final_state[0], S.seqt.ll.al);
      bp.put(1, 1);
    }
    bp.flush();
  }
  if (tid == 0)
    S.seq_csize = fits ? bs0 + nbytes - 3 : 0xFFFFFFFFu;
  __syncthreads();
  if (tid == 0) {
    // a carrier stays compressed even when larger than its input (it
    // always fits the staging, see kStageBytes)
    const uint32_t csize = S.seq_csize; // ~0u: did not fit
    const bool last = b1 == b.chunk_bytes;
    uint32_t total;
    if (S.all_same) { // RLE block: one byte
      put_le(stage, (last ? 1u : 0u) | (1u << 1) | (bsize << 3), 3);
      stage[3] = in[b0];
      total = 4;
    } else if (csize == 0xFFFFFFFFu || (!S.forced && csize >= bsize)) { // raw block
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

// Frame header size for a chunk of n bytes (single segment, content size).
__device__ __forceinline__ uint32_t frame_header_bytes(uint32_t n)
{
  return n < 256 ? 6 : (n < 65536 + 256 ? 7 : 9);
}

// One CTA per block: place the block at its offset in the chunk's frame
// (header + the sizes of the blocks before it); block 0 also writes the
// frame header and the last block the chunk's compressed size.
__global__ void __launch_bounds__(256)
zstd_frame_k(CodecBatch b,
             const uint8_t* stage_all,
             const uint32_t* block_sizes,
             uint32_t blocks_per_chunk)
{
  __shared__ uint32_t off;
  const uint64_t blk = blockIdx.x;
  const uint64_t chunk = blk / blocks_per_chunk;
  const uint32_t k = uint32_t(blk % blocks_per_chunk);
  uint8_t* out = b.out_at(chunk);
  const uint32_t n = b.chunk_bytes;
  const uint32_t* sizes = block_sizes + chunk * blocks_per_chunk;
  if (threadIdx.x < 32) {
    const unsigned lane = threadIdx.x;
    uint32_t acc = 0;
    for (uint32_t i = lane; i < k; i += 32)
      acc += sizes[i];
    for (int o = 16; o; o >>= 1)
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const uint32_t h = frame_header_bytes(n);
      off = h + acc;
      if (k == 0) { // magic, descriptor (single segment), frame content size
        put_le(out, 0xFD2FB528u, 4);
        if (h == 6) {
          out[4] = 0x20; // FCS flag 0
          out[5] = uint8_t(n);
        } else if (h == 7) {
          out[4] = 0x60; // FCS flag 1 (2 bytes, value - 256)
          put_le(out + 5, n - 256, 2);
        } else {
          out[4] = 0xA0; // FCS flag 2 (4 bytes)
          put_le(out + 5, n, 4);
        }
      }
      if (k + 1 == blocks_per_chunk)
        *b.size_at(chunk) = h + acc + sizes[k];
    }
  }
  __syncthreads();
  copy_bytes(out + off, stage_all + blk * kStageBytes, sizes[k], threadIdx.x,
             blockDim.x);
}

} // namespace

size_t zstd_scratch_bytes(uint64_t n_chunks, uint32_t chunk_bytes, int level)
{
  const uint64_t wide =
    zstd_wide(level)
      ? n_chunks * ((uint64_t(chunk_bytes) + kRegionBytes - 1) / kRegionBytes) *
            wide_entries(kZstdWideLog) * 2 + 256
      : 0;
  const uint64_t segs = n_chunks * ((chunk_bytes + kSegBytes - 1) / kSegBytes);
  const uint64_t blocks =
    n_chunks * ((chunk_bytes + kBlockBytes - 1) / kBlockBytes);
  const uint64_t adaptive =
    zstd_wide(level) ? n_chunks * (sizeof(ChunkSeq) + kSeqHistWords * sizeof(uint32_t)) + 256
                     : 0;
  return segs * (kMaxSeqPerSeg * sizeof(Seq) + sizeof(ZSeg) + kSegBytes) +
         blocks * (kStageBytes + sizeof(uint32_t)) +
         n_chunks * (kHistWords * sizeof(uint32_t) + sizeof(ChunkTable)) + 2048 + wide +
         adaptive;
}

cudaError_t launch_zstd(CodecBatch b, void* scratch, cudaStream_t st)
{
  if (!b.n_chunks)
    return cudaSuccess;
  b.segs_per_chunk = (b.chunk_bytes + kSegBytes - 1) / kSegBytes;
  const uint32_t bpc = (b.chunk_bytes + kBlockBytes - 1) / kBlockBytes;
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
  p += blocks * sizeof(uint32_t);
  p = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
  uint32_t* hist = reinterpret_cast<uint32_t*>(p);
  p += b.n_chunks * kHistWords * sizeof(uint32_t);
  ChunkTable* tables = reinterpret_cast<ChunkTable*>(p);
  p += b.n_chunks * sizeof(ChunkTable);
  p = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
  uint8_t* litbuf = p; // segs * kSegBytes, read up to 20 bytes past a slot
  p += segs * kSegBytes + 64;
  const uint32_t rpc = (b.chunk_bytes + kRegionBytes - 1) / kRegionBytes;
  cudaError_t e;
  if ((e = cudaMemsetAsync(hist, 0, b.n_chunks * kHistWords * sizeof(uint32_t), st)) !=
      cudaSuccess)
    return e;
  uint16_t* wide = nullptr;
  ChunkSeq* cseq = nullptr;
  uint32_t* seq_hist = nullptr;
  if (zstd_wide(b.level)) { // region tables of the wide window, sequence tables
    wide = reinterpret_cast<uint16_t*>((reinterpret_cast<uintptr_t>(p) + 255) &
                                       ~uintptr_t(255));
    const uintptr_t c = reinterpret_cast<uintptr_t>(wide + uint64_t(b.n_chunks) * rpc *
                                                             wide_entries(kZstdWideLog));
    cseq = reinterpret_cast<ChunkSeq*>((c + 255) & ~uintptr_t(255));
    seq_hist = reinterpret_cast<uint32_t*>(cseq + b.n_chunks);
    if ((e = cudaMemsetAsync(seq_hist, 0, b.n_chunks * kSeqHistWords * sizeof(uint32_t),
                             st)) != cudaSuccess)
      return e;
    note_launches(1);
    if ((e = lz77_launch_index(b, wide, rpc, kZstdWideLog, st)) != cudaSuccess)
      return e;
  }
  note_launches(4);
  CHUCKY_LAUNCH(zstd_find_k, unsigned(b.n_chunks * rpc), 32 * kSegsPerRegion,
                kRegionStageWords * sizeof(uint32_t), st, b, seqs, meta, hist, litbuf,
                rpc, static_cast<const uint16_t*>(wide), seq_hist);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  static const PredefTables pre = [] {
    PredefTables t{};
    uint8_t spread[64];
    uint16_t fill[64];
    fse_build(t.ll, kLLNormH, 36, 6, spread, fill);
    fse_build(t.ml, kMLNormH, 53, 6, spread, fill);
    fse_build(t.of, kOFNormH, 29, 5, spread, fill);
    return t;
  }();
  CHUCKY_LAUNCH(zstd_table_k, unsigned(b.n_chunks), kTableThreads, 0, st, b, hist, meta,
                tables, bpc);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  if (cseq) {
    note_launches(1);
    CHUCKY_LAUNCH(zstd_seqtab_k, unsigned(b.n_chunks), kTableThreads, 0, st, b, meta,
                  static_cast<const uint32_t*>(seq_hist), cseq, bpc);
    if ((e = cudaGetLastError()) != cudaSuccess)
      return e;
  }
  CHUCKY_LAUNCH(zstd_block_k, unsigned(blocks), kBlockThreads, kBlockBytes + 16, st, b,
                pre, seqs, meta, tables, static_cast<const ChunkSeq*>(cseq), litbuf, stage,
                bsizes, bpc);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  CHUCKY_LAUNCH(zstd_frame_k, unsigned(blocks), 256, 0, st, b, stage, bsizes, bpc);
  return cudaGetLastError();
}

} // namespace chucky
