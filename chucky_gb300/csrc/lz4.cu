// (c) LZ4 block encoder: one raw LZ4 block per chunk (CODEC_LZ4_NON_STANDARD).
//
// The reference compresses each chunk into a raw block with LZ4_compress_HC
// on the CPU or nvcomp's batched LZ4 on the GPU
// (src/cpu/compress.c:55-76, src/gpu/compress.cu:330-343); blocks are
// decoded with LZ4_decompress_safe and the known chunk size.  This encoder
// writes the LZ4 block format (token, literal length, literals, 16-bit
// offset, match length; last sequence literals only; last 5 bytes literal;
// last match starting >= 12 bytes before the end) in three passes:
//   find : warp-parallel greedy match finding per 4 KiB segment, matches
//          reaching back across the 16 KiB region (lz77.cuh)
//   plan : a warp per chunk carries each segment's trailing literals into
//          the next segment's first sequence and places every segment in
//          the output (segmented scans over the segments)
//   emit : a warp writes its segment's sequences at that place.
#include "kernels_codec.hpp"
#include "copy.cuh"
#include "launch.cuh"
#include "lz77.cuh"

namespace chucky {

namespace {

// warps per CTA of the plan and emit kernels (a chunk / a segment each);
// 2 measured 1 % (emit) and 12 % (plan) faster than 4 or 8 on sensor chunks
constexpr int kWarps = 2;

__host__ __device__ __forceinline__ uint32_t ext_len(uint32_t x)
{
  return x >= 15 ? (x - 15) / 255 + 1 : 0;
}

__host__ __device__ __forceinline__ uint32_t lit_part(uint32_t ll)
{
  return 1 + ll + ext_len(ll);
}

__host__ __device__ __forceinline__ uint32_t match_part(uint32_t ml)
{
  return 2 + ext_len(ml - 4);
}

struct SegMeta
{
  uint32_t nseq, trailing;
  uint32_t first_lit; // literal length of sequence 0 (before carry)
  uint32_t body;      // bytes of all sequences except sequence 0's literals
  uint32_t carry_in;  // literals carried in from earlier segments
  uint64_t out_off;   // byte offset of this segment's output in the chunk
  uint64_t tail_dst;  // output offset of this segment's trailing literals
  uint64_t final_off; // last segment: offset of the literal-only sequence
  uint32_t final_ll;  // last segment: its literal count
};

// Levels 2 and up parse with the wide window (the 3 regions before each
// one, LZ4's 64 KiB reach); level 0 and 1 with the region's own window.
constexpr uint32_t kLz4WideBack = 3;
constexpr int kLz4WideLog = 15;
__host__ __device__ inline bool lz4_wide(int level) { return level >= 2; }

// One CTA per region, a warp per segment of it.
__global__ void __launch_bounds__(32 * kSegsPerRegion)
lz4_find_k(CodecBatch b,
           Seq* seqs,
           SegMeta* meta,
           uint32_t regions_per_chunk,
           const uint16_t* wide_tables) // null: the region's own window only
{
  __shared__ __align__(16) uint16_t tables[kSegsPerRegion][1 << kHashLog];
  CHUCKY_DYN_SHARED(uint32_t, words); // kRegionStageWords
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t chunk = blockIdx.x / regions_per_chunk;
  const uint32_t r0 = (blockIdx.x % regions_per_chunk) * kRegionBytes;
  const uint8_t* base = b.in_at(chunk);
  const uint32_t n = b.chunk_bytes;
  const uint32_t r1 = min(n, r0 + kRegionBytes);
  lz77_stage_region(base, r0, r1, words, threadIdx.x, blockDim.x);
  const uint32_t s0 = r0 + w * kSegBytes;
  if (s0 >= r1)
    return;
  const uint64_t seg = chunk * b.segs_per_chunk + s0 / kSegBytes;
  const uint32_t s1 = min(n, s0 + kSegBytes);
  const bool last = s1 == n;
  uint32_t start_limit = s1, match_end = s1;
  if (last) {
    start_limit = n > 12 ? n - 12 : 0;
    match_end = n > 5 ? n - 5 : 0;
    if (start_limit < s0)
      start_limit = s0;
  }
  Seq* out = seqs + seg * kMaxSeqPerSeg;
  // the wide window: the 3 regions before (LZ4 offsets reach 65535 back)
  const WideWindow W{ base,
                      wide_tables ? wide_tables + chunk * regions_per_chunk *
                                                    wide_entries(kLz4WideLog)
                                  : nullptr,
                      uint32_t(r0 / kRegionBytes), kLz4WideBack, 65535u, kLz4WideLog };
  const SegInfo info = lz77_parse_segment(
    words, r0, s0, s1, start_limit, match_end, tables[w], out,
    b.min_match > 4 ? uint32_t(b.min_match) : 4u, wide_tables ? &W : nullptr,
    b.strength > 0 ? b.strength : kSearchStrength);
  __syncwarp();
  // encoded size of everything but sequence 0's literal part
  uint32_t body = 0;
  for (uint32_t i = lane; i < info.nseq; i += 32) {
    const Seq s = out[i];
    body += match_part(s.match) + (i ? lit_part(s.lit) : 0);
  }
  for (int o = 16; o; o >>= 1)
    body += __shfl_xor_sync(0xffffffffu, body, o);
  if (lane == 0) {
    SegMeta m{};
    m.nseq = info.nseq;
    m.trailing = info.trailing;
    m.first_lit = info.nseq ? out[0].lit : 0;
    m.body = body;
    meta[seg] = m;
  }
}

// Place every segment's sequences, and every trailing literal run, in the
// chunk's output.  Trailing literals of a segment (all of it when it has no
// match) belong to the literal field of the next sequence: the first
// sequence of a later segment, or the final literal-only sequence.
//
// A warp per chunk, 32 segments per step.  Forward pass: the literals
// carried into each segment are a segmented sum of the trailing counts (a
// segment with matches restarts the run with its own trailing literals),
// and the output offsets an exclusive sum of the segments' sizes.  Reverse
// pass: each segment's trailing literals go to the literal field of the
// next segment with matches (or of the final sequence), after the run's
// earlier contributions.
__global__ void __launch_bounds__(32 * kWarps)
lz4_plan_k(CodecBatch b, SegMeta* meta)
{
  constexpr unsigned kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint64_t chunk = uint64_t(blockIdx.x) * kWarps + (threadIdx.x >> 5);
  if (chunk >= b.n_chunks)
    return; // the whole warp
  SegMeta* m = meta + chunk * b.segs_per_chunk;
  const uint32_t S = b.segs_per_chunk;
  uint32_t carry = 0; // literals pending before the group
  uint64_t off = 0;   // output bytes before the group
  for (uint32_t g = 0; g < S; g += 32) {
    const uint32_t k = g + lane;
    const bool valid = k < S;
    uint32_t tr = 0, fl = 0, body = 0;
    bool has = false;
    if (valid) {
      has = m[k].nseq != 0;
      tr = m[k].trailing;
      fl = m[k].first_lit;
      body = m[k].body;
    }
    // carry out of segment k, counted from the group start unless a
    // segment with matches in [g, k] restarted the run
    uint32_t x = tr;
    bool f = has;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t xp = __shfl_up_sync(kAll, x, o);
      const bool fp = __shfl_up_sync(kAll, f, o);
      if (lane >= o) {
        if (!f)
          x += xp;
        f = f || fp;
      }
    }
    const uint32_t cout = f ? x : carry + x;
    uint32_t cin = __shfl_up_sync(kAll, cout, 1);
    if (lane == 0)
      cin = carry;
    const uint64_t c = has ? uint64_t(lit_part(fl + cin)) + body : 0;
    uint64_t inc = c;
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(kAll, inc, o);
      if (lane >= o)
        inc += y;
    }
    if (valid) {
      m[k].carry_in = cin;
      m[k].out_off = off + inc - c;
    }
    off += __shfl_sync(kAll, inc, 31);
    carry = __shfl_sync(kAll, cout, 31); // lanes past S add nothing
  }
  if (lane == 0) {
    m[S - 1].final_off = off;
    m[S - 1].final_ll = carry;
    *b.size_at(chunk) = off + lit_part(carry);
  }
  __syncwarp();
  // literal field of the run that ends at the final sequence
  uint64_t next_field = off + 1 + ext_len(carry);
  const uint32_t ngroups = (S + 31) / 32;
  for (uint32_t gi = ngroups; gi-- > 0;) {
    const uint32_t k = gi * 32 + lane;
    const bool valid = k < S;
    bool has = false;
    uint64_t field = 0;
    uint32_t in_run = 0; // place of the segment's tail within its run
    if (valid) {
      has = m[k].nseq != 0;
      const uint32_t cin = m[k].carry_in;
      if (has)
        field = m[k].out_off + 1 + ext_len(m[k].first_lit + cin);
      else
        in_run = cin;
    }
    const unsigned hm = __ballot_sync(kAll, has);
    const unsigned above = lane == 31 ? 0u : hm & (kAll << (lane + 1));
    const uint64_t f_above = __shfl_sync(kAll, field, above ? __ffs(int(above)) - 1 : 0);
    if (valid)
      m[k].tail_dst = (above ? f_above : next_field) + in_run;
    const uint64_t f_first = __shfl_sync(kAll, field, hm ? __ffs(int(hm)) - 1 : 0);
    if (hm)
      next_field = f_first;
  }
}

__device__ __forceinline__ uint8_t* put_len(uint8_t* o, uint32_t extra)
{
  // extra = length - 15 (length >= 15): 255-runs then the remainder
  while (extra >= 255) {
    *o++ = 255;
    extra -= 255;
  }
  *o++ = uint8_t(extra);
  return o;
}

__global__ void __launch_bounds__(32 * kWarps)
lz4_emit_k(CodecBatch b, const Seq* seqs, const SegMeta* meta)
{
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t seg = uint64_t(blockIdx.x) * kWarps + w;
  if (seg >= b.n_chunks * b.segs_per_chunk)
    return;
  const uint64_t chunk = seg / b.segs_per_chunk;
  const uint32_t k = uint32_t(seg % b.segs_per_chunk);
  const SegMeta m = meta[seg];
  const bool last = k + 1 == b.segs_per_chunk;
  const uint8_t* in = b.in_at(chunk);
  uint8_t* out = b.out_at(chunk);
  const Seq* s = seqs + seg * kMaxSeqPerSeg;
  const uint32_t s0 = k * kSegBytes;
  const uint32_t s1 = min(b.chunk_bytes, s0 + kSegBytes);
  uint64_t pos = m.out_off;
  uint32_t src = s0; // input position of this segment's next own literal
  for (uint32_t base = 0; base < m.nseq; base += 32) {
    const uint32_t i = base + lane;
    Seq q{ 0, 0, 0 };
    uint32_t sz = 0, carry = 0;
    if (i < m.nseq) {
      q = s[i];
      if (i == 0)
        carry = m.carry_in; // written by the segments they came from
      sz = lit_part(q.lit + carry) + match_part(q.match);
    }
    // exclusive scans of output size and consumed own input
    uint32_t ex = sz, in_ex = q.lit + q.match;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t a = __shfl_up_sync(0xffffffffu, ex, o);
      const uint32_t c = __shfl_up_sync(0xffffffffu, in_ex, o);
      if (lane >= o) {
        ex += a;
        in_ex += c;
      }
    }
    const uint32_t tot = __shfl_sync(0xffffffffu, ex, 31);
    const uint32_t in_tot = __shfl_sync(0xffffffffu, in_ex, 31);
    ex -= sz;
    in_ex -= q.lit + q.match;
    const uint32_t ll = q.lit + carry;
    uint8_t* o = out + pos + ex;
    const uint32_t hdr = 1 + ext_len(ll);
    const bool long_lits = q.lit > 64;
    if (i < m.nseq) {
      const uint32_t ml4 = q.match - 4;
      o[0] = uint8_t((min(ll, 15u) << 4) | min(ml4, 15u));
      if (ll >= 15)
        put_len(o + 1, ll - 15);
      if (!long_lits)
        for (uint32_t j = 0; j < q.lit; ++j)
          o[hdr + carry + j] = in[src + in_ex + j];
      uint8_t* t = o + hdr + ll;
      t[0] = uint8_t(q.offset);
      t[1] = uint8_t(q.offset >> 8);
      if (ml4 >= 15)
        put_len(t + 2, ml4 - 15);
    }
    // long literal runs: copied by the whole warp
    unsigned pending = __ballot_sync(0xffffffffu, i < m.nseq && long_lits);
    while (pending) {
      const int j = __ffs(pending) - 1;
      pending &= pending - 1;
      const uint32_t n = __shfl_sync(0xffffffffu, q.lit, j);
      const uint32_t lo = __shfl_sync(0xffffffffu, ex, j);
      const uint32_t li = __shfl_sync(0xffffffffu, in_ex, j);
      const uint32_t h = __shfl_sync(0xffffffffu, hdr + carry, j);
      copy_bytes(out + pos + lo + h, in + src + li, n, lane, 32);
    }
    pos += tot;
    src += in_tot;
  }
  // this segment's trailing literals go into a later literal field
  copy_bytes(out + m.tail_dst, in + src, s1 - src, lane, 32);
  if (last && lane == 0) { // header of the final literal-only sequence
    uint8_t* f = out + m.final_off;
    f[0] = uint8_t(min(m.final_ll, 15u) << 4);
    if (m.final_ll >= 15)
      put_len(f + 1, m.final_ll - 15);
  }
}

} // namespace

// Saturates at SIZE_MAX when the product would overflow, so a caller that
// compares the result with a fixed capacity rejects absurd chunk counts.
size_t lz4_scratch_bytes(uint64_t n_chunks, uint32_t chunk_bytes, int level)
{
  const uint64_t rpc = (uint64_t(chunk_bytes) + kRegionBytes - 1) / kRegionBytes;
  const uint64_t per_chunk = ((uint64_t(chunk_bytes) + kSegBytes - 1) / kSegBytes) *
                               (kMaxSeqPerSeg * sizeof(Seq) + sizeof(SegMeta)) +
                             (lz4_wide(level) ? rpc * wide_entries(kLz4WideLog) * 2 + 256 : 0);
  if (per_chunk && n_chunks > (SIZE_MAX - 512) / per_chunk)
    return SIZE_MAX;
  return n_chunks * per_chunk + 512;
}

cudaError_t launch_lz4(CodecBatch b, void* scratch, cudaStream_t st)
{
  if (!b.n_chunks)
    return cudaSuccess;
  b.segs_per_chunk = (b.chunk_bytes + kSegBytes - 1) / kSegBytes;
  const uint64_t segs = b.n_chunks * b.segs_per_chunk;
  const uint32_t rpc = (b.chunk_bytes + kRegionBytes - 1) / kRegionBytes;
  Seq* seqs = static_cast<Seq*>(scratch);
  // SegMeta holds a 64-bit field: start it on a 256-byte boundary
  const uintptr_t m = reinterpret_cast<uintptr_t>(seqs + segs * kMaxSeqPerSeg);
  SegMeta* meta = reinterpret_cast<SegMeta*>((m + 255) & ~uintptr_t(255));
  const unsigned grid = unsigned((segs + kWarps - 1) / kWarps);
  cudaError_t e;
  uint16_t* wide = nullptr;
  if (lz4_wide(b.level)) { // region tables after the segment metadata
    const uintptr_t t = reinterpret_cast<uintptr_t>(meta + segs);
    wide = reinterpret_cast<uint16_t*>((t + 255) & ~uintptr_t(255));
    note_launches(1);
    if ((e = lz77_launch_index(b, wide, rpc, kLz4WideLog, st)) != cudaSuccess)
      return e;
  }
  note_launches(3);
  CHUCKY_LAUNCH(lz4_find_k, unsigned(b.n_chunks * rpc), 32 * kSegsPerRegion,
                kRegionStageWords * sizeof(uint32_t), st, b, seqs, meta, rpc,
                static_cast<const uint16_t*>(wide));
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  CHUCKY_LAUNCH(lz4_plan_k, unsigned((b.n_chunks + kWarps - 1) / kWarps), 32 * kWarps, 0,
                st, b, meta);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  CHUCKY_LAUNCH(lz4_emit_k, grid, 32 * kWarps, 0, st, b, seqs, meta);
  return cudaGetLastError();
}

} // namespace chucky
