// (c) LZ4 block encoder: one raw LZ4 block per chunk (CODEC_LZ4_NON_STANDARD).
//
// The reference compresses each chunk into a raw block with LZ4_compress_HC
// on the CPU or nvcomp's batched LZ4 on the GPU
// (src/cpu/compress.c:55-76, src/gpu/compress.cu:330-343); blocks are
// decoded with LZ4_decompress_safe and the known chunk size.  This encoder
// writes the LZ4 block format (token, literal length, literals, 16-bit
// offset, match length; last sequence literals only; last 5 bytes literal;
// last match starting >= 12 bytes before the end) in three passes:
//   find : warp-parallel greedy match finding per 16 KiB segment (lz77.cuh)
//   plan : per chunk, carry each segment's trailing literals into the next
//          segment's first sequence and place every segment in the output
//   emit : a warp writes its segment's sequences at that place.
#include "kernels_codec.hpp"
#include "launch.cuh"
#include "lz77.cuh"

namespace chucky {

namespace {

constexpr int kWarps = 4;

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
};

__global__ void __launch_bounds__(32 * kWarps)
lz4_find_k(CodecBatch b, Seq* seqs, SegMeta* meta)
{
  __shared__ uint16_t tables[kWarps][1 << kHashLog];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t seg = uint64_t(blockIdx.x) * kWarps + w;
  if (seg >= b.n_chunks * b.segs_per_chunk)
    return;
  const uint64_t chunk = seg / b.segs_per_chunk;
  const uint32_t k = uint32_t(seg % b.segs_per_chunk);
  const uint8_t* base = b.in + b.id(chunk) * b.in_stride;
  const uint32_t n = b.chunk_bytes;
  const uint32_t s0 = k * kSegBytes;
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
  const SegInfo info =
    lz77_parse_segment(base, s0, s1, start_limit, match_end, tables[w], out);
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

__global__ void lz4_plan_k(CodecBatch b, SegMeta* meta)
{
  const uint64_t chunk = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (chunk >= b.n_chunks)
    return;
  SegMeta* m = meta + chunk * b.segs_per_chunk;
  uint64_t off = 0;
  uint32_t carry = 0;
  for (uint32_t k = 0; k < b.segs_per_chunk; ++k) {
    m[k].carry_in = carry;
    m[k].out_off = off;
    if (m[k].nseq) {
      off += lit_part(m[k].first_lit + carry) + m[k].body;
      carry = m[k].trailing;
    } else {
      carry += m[k].trailing;
    }
  }
  off += lit_part(carry); // final literal-only sequence
  b.out_sizes[b.id(chunk)] = off;
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

// Copy n bytes with the warp (byte per lane).
__device__ __forceinline__ void warp_bytes(uint8_t* dst,
                                           const uint8_t* src,
                                           uint32_t n)
{
  for (uint32_t i = threadIdx.x & 31; i < n; i += 32)
    dst[i] = src[i];
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
  if (!m.nseq && !last)
    return; // its literals travel with the next segment
  const uint8_t* in = b.in + b.id(chunk) * b.in_stride;
  uint8_t* out = b.out + b.id(chunk) * b.out_stride;
  const Seq* s = seqs + seg * kMaxSeqPerSeg;
  const uint32_t s0 = k * kSegBytes;
  uint64_t pos = m.out_off;
  uint32_t src = s0 - m.carry_in; // first literal of the next sequence
  for (uint32_t base = 0; base < m.nseq; base += 32) {
    const uint32_t i = base + lane;
    Seq q{ 0, 0, 0 };
    uint32_t sz = 0;
    if (i < m.nseq) {
      q = s[i];
      if (i == 0)
        q.lit += m.carry_in;
      sz = lit_part(q.lit) + match_part(q.match);
    }
    // exclusive scans of output size and consumed input
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
    uint8_t* o = out + pos + ex;
    const uint8_t* lits = in + src + in_ex;
    const bool long_lits = q.lit > 64;
    if (i < m.nseq) {
      const uint32_t ml4 = q.match - 4;
      *o++ = uint8_t((min(q.lit, 15u) << 4) | min(ml4, 15u));
      if (q.lit >= 15)
        o = put_len(o, q.lit - 15);
      if (!long_lits)
        for (uint32_t j = 0; j < q.lit; ++j)
          o[j] = lits[j];
      o += q.lit;
      o[0] = uint8_t(q.offset);
      o[1] = uint8_t(q.offset >> 8);
      o += 2;
      if (ml4 >= 15)
        put_len(o, ml4 - 15);
    }
    // long literal runs: copied by the whole warp
    unsigned pending = __ballot_sync(0xffffffffu, i < m.nseq && long_lits);
    while (pending) {
      const int j = __ffs(pending) - 1;
      pending &= pending - 1;
      const uint32_t ll = __shfl_sync(0xffffffffu, q.lit, j);
      const uint32_t lo = __shfl_sync(0xffffffffu, ex, j);
      const uint32_t li = __shfl_sync(0xffffffffu, in_ex, j);
      const uint32_t hdr = 1 + ext_len(ll);
      warp_bytes(out + pos + lo + hdr, in + src + li, ll);
    }
    pos += tot;
    src += in_tot;
  }
  if (last) {
    // final literal-only sequence: everything from `src` to the chunk end
    const uint32_t ll = b.chunk_bytes - src;
    uint8_t* o = out + pos;
    if (lane == 0) {
      o[0] = uint8_t(min(ll, 15u) << 4);
      if (ll >= 15)
        put_len(o + 1, ll - 15);
    }
    warp_bytes(o + 1 + ext_len(ll), in + src, ll);
  }
}

} // namespace

size_t lz4_scratch_bytes(uint64_t n_chunks, uint32_t chunk_bytes)
{
  const uint64_t segs = n_chunks * ((chunk_bytes + kSegBytes - 1) / kSegBytes);
  return segs * (kMaxSeqPerSeg * sizeof(Seq) + sizeof(SegMeta)) + 512;
}

cudaError_t launch_lz4(CodecBatch b, void* scratch, cudaStream_t st)
{
  if (!b.n_chunks)
    return cudaSuccess;
  b.segs_per_chunk = (b.chunk_bytes + kSegBytes - 1) / kSegBytes;
  const uint64_t segs = b.n_chunks * b.segs_per_chunk;
  Seq* seqs = static_cast<Seq*>(scratch);
  // SegMeta holds a 64-bit field: start it on a 256-byte boundary
  const uintptr_t m = reinterpret_cast<uintptr_t>(seqs + segs * kMaxSeqPerSeg);
  SegMeta* meta = reinterpret_cast<SegMeta*>((m + 255) & ~uintptr_t(255));
  const unsigned grid = unsigned((segs + kWarps - 1) / kWarps);
  cudaError_t e;
  note_launches(3);
  CHUCKY_LAUNCH(lz4_find_k, grid, 32 * kWarps, 0, st, b, seqs, meta);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  CHUCKY_LAUNCH(lz4_plan_k, unsigned((b.n_chunks + 127) / 128), 128, 0, st, b, meta);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return e;
  CHUCKY_LAUNCH(lz4_emit_k, grid, 32 * kWarps, 0, st, b, seqs, meta);
  return cudaGetLastError();
}

} // namespace chucky
