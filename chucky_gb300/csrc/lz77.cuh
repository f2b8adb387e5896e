// Warp-parallel greedy LZ77 match finder shared by the LZ4 and zstd encoders.
//
// A chunk is cut into regions of kRegionBytes and each region into segments
// of kSegBytes.  One CTA of kSegsPerRegion warps takes one region: all its
// threads stage the region's bytes in shared memory (lz77_stage_region),
// then warp w parses segment w of the region with a private hash table
// (kHashLog-bit hash of 4 bytes -> last position, 16-bit positions relative
// to the region).  Before parsing, a warp enters the positions of the
// kHistorySegs segments of the region before its own into its table
// (insert only), so its matches may reach back into them, as a single
// sequential parse would; the segments are parsed side by side.
//
// The segment is scanned in windows of 32 positions, one per lane (with a
// stride that grows by one for every 2^kSearchStrength literals since the
// last match, as fast LZ77 parsers skip through incompressible data).  Every
// lane hashes the 4 bytes at its position, probes the table, verifies the
// candidate (or, for runs and periods of 1, 2 or 4 bytes, the lane 1, 2 or
// 4 positions back in the same window) and measures the match on its own,
// up to kLaneExtend bytes; then all 32 positions enter the table.  The
// greedy parse then takes, within the window, the lowest position at or
// after the parse point with a match of at least `min_match` bytes, as many
// times as the window allows (a chain walk over per-lane links to the next
// hit after each match); a match that reaches kLaneExtend bytes is
// extended by the whole warp, 32 bytes per step.  Windows inside a long
// match are skipped.  Matches end inside their segment and start inside
// it or its history.  (When lanes of one window share a hash slot the
// hardware keeps one of their stores.)
//
// Output per segment: sequences (literal length, match length, offset) in
// scratch, the sequence count and the trailing literal count.
#pragma once

#include <stdint.h>

namespace chucky {

constexpr int kSegLog = 12;
constexpr uint32_t kSegBytes = 1u << kSegLog; // 4 KiB: one warp's parse
constexpr int kRegionLog = 14;
constexpr uint32_t kRegionBytes = 1u << kRegionLog; // 16 KiB: match window
constexpr uint32_t kSegsPerRegion = kRegionBytes / kSegBytes;
constexpr int kHashLog = 10;
constexpr uint32_t kMaxSeqPerSeg = kSegBytes / 4 + 1;
// 32-bit words of a staged region: the region plus a spare vector for reads
// that straddle its end.
constexpr uint32_t kRegionStageWords = kRegionBytes / 4 + 4;
// bytes a lane measures of its own match before the warp takes over
constexpr uint32_t kLaneExtend = 64;
#ifndef CHUCKY_SEARCH_STRENGTH
#define CHUCKY_SEARCH_STRENGTH 6
#endif
#ifndef CHUCKY_HISTORY_SEGS
#define CHUCKY_HISTORY_SEGS 1
#endif
// positions probed per lane step grow by one for every 2^strength literals
// since the last match (sparse probing of incompressible runs); the default
// strength (a batch may carry another, CodecBatch::strength)
constexpr int kSearchStrength = CHUCKY_SEARCH_STRENGTH;
// segments of the region before a warp's own that enter its table, and the
// stride of the positions entered
constexpr uint32_t kHistorySegs = CHUCKY_HISTORY_SEGS;
#ifndef CHUCKY_HISTORY_STRIDE
#define CHUCKY_HISTORY_STRIDE 2
#endif
constexpr uint32_t kHistoryStride = CHUCKY_HISTORY_STRIDE;
static_assert((2u << kHashLog) >= kSegBytes / 8,
              "a warp's table holds its literal bitmap");

struct Seq
{
  uint32_t lit;    // literals before the match
  uint32_t match;  // match length (>= 4)
  uint32_t offset; // distance back to the match source (>= 1)
};

struct SegInfo
{
  uint32_t nseq;     // sequences with a match
  uint32_t trailing; // literals after the last match of the segment
};

// ---- wide match window (the higher levels) ---------------------------------
//
// A region's own hash table only reaches back into the region.  At the
// higher levels a first pass (lz77_index_k) records, for every region, the
// last position of each hash of 4 bytes (a deterministic maximum);
// the parse then also probes the tables of up to `back` earlier regions,
// nearest first, verifies each candidate against the chunk in global
// memory and takes the first that beats the lane's local match (measured
// up to kLaneExtend - 1 bytes).
// (hash log per codec: 15 bits for LZ4, 14 for zstd; the zstd parse reaches
// further back, so smaller tables keep more of them in L2)
__host__ __device__ constexpr uint64_t wide_entries(int hlog) { return uint64_t(1) << hlog; }
// lanes whose local match is shorter than this probe the wide window
constexpr uint32_t kWideProbeBelow = 16;

struct WideWindow
{
  const uint8_t* chunk;   // the chunk's bytes (4-byte aligned; readable past the end)
  const uint16_t* tables; // the chunk's region tables [regions][1 << hlog]
  uint32_t region;        // the region being parsed
  uint32_t back;          // earlier regions probed
  uint32_t max_dist;      // farthest match source allowed (bytes back)
  int hlog;               // hash bits of the tables
};

__device__ __forceinline__ uint32_t hash4w(uint32_t v, int hlog)
{
  return (v * 2654435761u) >> (32 - hlog);
}

// Table entries: the region offset (14 bits) and, in the two spare bits, a
// tag -- the two hash bits below the table's -- so that most entries of
// other values are passed over without loading their bytes; 0xFFFF: none
// (offsets are at most kRegionBytes - 4).
static_assert(kRegionLog == 14, "region offsets fill 14 bits of an entry");
__device__ __forceinline__ uint32_t wide_tag(uint32_t v, int hlog)
{
  return ((v * 2654435761u) >> (30 - hlog)) & 3u;
}

// 4 bytes of `base` (4-byte aligned) at any byte position p
__device__ __forceinline__ uint32_t load4(const uint8_t* base, uint32_t p)
{
  const uint32_t* w = reinterpret_cast<const uint32_t*>(base + (p & ~3u));
  return __funnelshift_r(__ldg(w), __ldg(w + 1), (p & 3) * 8);
}

// 4 bytes at byte position `pos` of a word array.
__device__ __forceinline__ uint32_t word_at(const uint32_t* w, uint32_t pos)
{
  return __funnelshift_r(w[pos >> 2], w[(pos >> 2) + 1], (pos & 3) * 8);
}

__device__ __forceinline__ uint32_t hash4(uint32_t v)
{
  return (v * 2654435761u) >> (32 - kHashLog);
}

// Copy bytes [r0, r1) of a chunk at `base` (4-byte aligned; r0 a multiple
// of 16; readable 16 bytes past r1) into `words` (kRegionStageWords words of
// shared memory) with all `nthreads` threads of the CTA; ends with a CTA
// barrier.
__device__ __forceinline__ void lz77_stage_region(const uint8_t* base,
                                                  uint32_t r0,
                                                  uint32_t r1,
                                                  uint32_t* words,
                                                  unsigned tid,
                                                  unsigned nthreads)
{
  const uint8_t* src = base + r0;
  const uint32_t nvec = (r1 - r0 + 15) >> 4;
  if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
    const uint4* v = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(words);
#pragma unroll 4
    for (uint32_t i = tid; i < nvec; i += nthreads)
      d[i] = __ldg(v + i);
  } else {
    const uint32_t* v = reinterpret_cast<const uint32_t*>(src);
#pragma unroll 8
    for (uint32_t i = tid; i < 4 * nvec; i += nthreads)
      words[i] = __ldg(v + i);
  }
  if (tid < 4)
    words[4 * nvec + tid] = 0;
  __syncthreads();
}

// Length of the match of position q against cand (< q), up to kLaneExtend
// bytes, ending at or before `end` (one lane).
__device__ __forceinline__ uint32_t lane_match(const uint32_t* words,
                                               const uint8_t* bytes,
                                               uint32_t q,
                                               uint32_t cand,
                                               uint32_t end)
{
  uint32_t len = 4;
  while (len < kLaneExtend) {
    if (q + len + 4 > end) { // the last bytes before `end`, one by one
      while (q + len < end && bytes[q + len] == bytes[cand + len])
        ++len;
      break;
    }
    const uint32_t x = word_at(words, q + len) ^ word_at(words, cand + len);
    if (x) {
      len += uint32_t(__ffs(int(x)) - 1) >> 3;
      break;
    }
    len += 4;
  }
  return len;
}

// Match length of candidate c (chunk position) for position q (region
// position, its bytes in the staged region) whose first 4 bytes are known
// equal, up to `cap` bytes.
__device__ __forceinline__ uint32_t wide_extend(const WideWindow& W,
                                                const uint32_t* words,
                                                uint32_t q,
                                                uint32_t c,
                                                uint32_t cap)
{
  uint32_t m = 4;
  while (m + 4 <= cap) {
    const uint32_t d = word_at(words, q + m) ^ load4(W.chunk, c + m);
    if (d) {
      m += uint32_t(__ffs(int(d)) - 1) >> 3;
      break;
    }
    m += 4;
  }
  if (m + 4 > cap) { // the last bytes before the cap, one by one
    const uint8_t* bytes = reinterpret_cast<const uint8_t*>(words);
    while (m < cap && bytes[q + m] == W.chunk[c + m])
      ++m;
  }
  return m > cap ? cap : m;
}

// One lane's probe of the wide window for one position.
struct WideLane
{
  bool on;        // still searching
  uint32_t q, x;  // position (region-relative) and its 4 bytes
  uint32_t h, tag;
  uint32_t cap, need;
};

__device__ __forceinline__ WideLane wide_lane(const WideWindow& W,
                                              bool probe,
                                              uint32_t q,
                                              uint32_t x,
                                              uint32_t end,
                                              bool ok,
                                              uint32_t len)
{
  WideLane L;
  L.on = probe;
  L.q = q;
  L.x = x;
  L.h = hash4w(x, W.hlog);
  L.tag = wide_tag(x, W.hlog);
  L.cap = probe ? min(kLaneExtend - 1, end - q) : 0;
  L.need = ok ? len + 1 : 4;
  return L;
}

// Candidates of two positions of a lane (its a and b windows) in the wide
// window's earlier regions, nearest region first; for each, the first
// candidate that matches longer than its (cand, len) replaces them and
// ends its search.  Only entries with the value's tag are checked against
// the chunk (its bytes in global memory, the lane's from the staged region
// `words`).  The two searches are independent; their loads are issued side
// by side.  Where probing has thinned out (`step` > 1: a literal run) only
// the two nearest regions are probed.
__device__ __forceinline__ void wide_probe2(const WideWindow& W,
                                            const uint32_t* words,
                                            uint32_t r0,
                                            uint32_t step,
                                            WideLane A,
                                            bool& oka,
                                            uint32_t& ca,
                                            uint32_t& la,
                                            WideLane B,
                                            bool& okb,
                                            uint32_t& cb,
                                            uint32_t& lb)
{
  const uint64_t entries = wide_entries(W.hlog);
  const uint32_t nb = min(step > 1 ? min(W.back, 2u) : W.back, W.region);
  for (uint32_t k = 0; k < nb && (A.on || B.on); ++k) {
    const uint32_t rr = W.region - 1 - k;
    const uint16_t* tb = W.tables + uint64_t(rr) * entries;
    const uint16_t ta = A.on ? tb[A.h] : uint16_t(0xFFFF);
    const uint16_t tbb = B.on ? tb[B.h] : uint16_t(0xFFFF);
    const bool ga = ta != 0xFFFF && (uint32_t(ta) >> 14) == A.tag;
    const bool gb = tbb != 0xFFFF && (uint32_t(tbb) >> 14) == B.tag;
    const uint32_t cxa = rr * kRegionBytes + (ta & 0x3FFFu);
    const uint32_t cxb = rr * kRegionBytes + (tbb & 0x3FFFu);
    // the regions further back are further still
    const bool fa = ga && r0 + A.q - cxa > W.max_dist;
    const bool fb = gb && r0 + B.q - cxb > W.max_dist;
    if (fa)
      A.on = false;
    if (fb)
      B.on = false;
    const bool va = ga && !fa, vb = gb && !fb;
    const uint32_t xa = va ? load4(W.chunk, cxa) : ~A.x;
    const uint32_t xb = vb ? load4(W.chunk, cxb) : ~B.x;
    if (va && xa == A.x) {
      const uint32_t m = wide_extend(W, words, A.q, cxa, A.cap);
      if (m >= A.need) {
        oka = true;
        la = m;
        ca = cxa - r0; // before the region: wraps, offsets stay q - cand
        A.on = false;
      }
    }
    if (vb && xb == B.x) {
      const uint32_t m = wide_extend(W, words, B.q, cxb, B.cap);
      if (m >= B.need) {
        okb = true;
        lb = m;
        cb = cxb - r0;
        B.on = false;
      }
    }
  }
}

// Parse segment [s0, s1) of a chunk whose bytes from r0 (the region start,
// r0 <= s0) on are staged in `words`.  Matches may start at positions in
// [s0, start_limit), reach back to r0 and end at or before `match_end`.
// `table` holds 1 << kHashLog u16 entries private to this warp (16-byte
// aligned).
__device__ inline SegInfo lz77_parse_segment(const uint32_t* words,
                                             uint32_t r0,
                                             uint32_t s0,
                                             uint32_t s1,
                                             uint32_t start_limit,
                                             uint32_t match_end,
                                             uint16_t* table,
                                             Seq* out,
                                             uint32_t min_match = 4,
                                             const WideWindow* wide = nullptr,
                                             int strength = kSearchStrength)
{
  const int lane = threadIdx.x & 31;
  const uint8_t* bytes = reinterpret_cast<const uint8_t*>(words);
  // empty table (16-byte stores: the tables are 16-byte aligned rows)
  for (int i = lane; i < (1 << kHashLog) / 8; i += 32)
    reinterpret_cast<uint4*>(table)[i] =
      make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
  __syncwarp();
  // positions below are relative to r0
  const uint32_t first = s0 - r0;
  const uint32_t lim = start_limit > s0 ? start_limit - r0 : first;
  const uint32_t end = match_end - r0;
  // history: the region's positions before this segment
  const uint32_t hist0 =
    first > kHistorySegs * kSegBytes ? first - kHistorySegs * kSegBytes : 0;
  for (uint32_t w0 = hist0; w0 < first; w0 += 32 * kHistoryStride) {
    const uint32_t q = w0 + lane * kHistoryStride;
    const uint32_t h = hash4(word_at(words, q));
    __syncwarp();
    table[h] = uint16_t(q);
  }
  __syncwarp();
  uint32_t w0 = first, p = first, lit_start = first, nseq = 0;
  // Greedy parse of one window's hits (lanes at or after the parse point).
  // Every hit lane knows where its match ends, hence the first hit lane at
  // or after that end: the greedy choices are the chain of these links from
  // the first hit lane at or after p, walked with one shuffle per match,
  // and the chosen lanes then write their sequences side by side.  A match
  // measured to kLaneExtend bytes ends the chain; the warp extends it and
  // the parse continues after its true end.
  const unsigned below_me = (1u << lane) - 1;
  auto take = [&](unsigned hits, uint32_t base, uint32_t step, uint32_t cand,
                  uint32_t len) {
    const uint32_t mpos_l = base + lane * step;
    const uint32_t end_l = mpos_l + len;
    const unsigned longs = __ballot_sync(0xffffffffu, ((hits >> lane) & 1) && len >= kLaneExtend);
    // first lane at or after position x (no division while the probing is
    // dense: matches come often then)
    auto lane_from = [&](uint32_t x) {
      const uint32_t d = x > base ? x - base : 0;
      return step == 1 ? d : (d + step - 1) / step;
    };
    int nxt = 32; // next hit lane after this lane's match
    if ((hits >> lane) & 1) {
      const uint32_t f = lane_from(end_l);
      const unsigned nm = f >= 32 ? 0u : hits & (0xffffffffu << f);
      nxt = nm ? __ffs(int(nm)) - 1 : 32;
    }
    for (;;) {
      const uint32_t from = lane_from(p);
      if (from >= 32)
        break;
      const unsigned m = hits & (0xffffffffu << from);
      if (!m)
        break;
      unsigned sel = 0;
      int k = __ffs(int(m)) - 1, last = k;
      for (;;) {
        sel |= 1u << k;
        last = k;
        if ((longs >> k) & 1)
          break;
        const int nk = __shfl_sync(0xffffffffu, nxt, k);
        if (nk >= 32)
          break;
        k = nk;
      }
      // the literals before a chosen match start at the previous chosen
      // match's end (the parse point for the first)
      const unsigned prev = sel & below_me;
      const int pl = prev ? 31 - __clz(int(prev)) : 0;
      const uint32_t pend = __shfl_sync(0xffffffffu, end_l, pl);
      const uint32_t lit0 = prev ? pend : lit_start;
      const bool extend = (longs >> last) & 1;
      if (((sel >> lane) & 1) && !(extend && lane == last))
        out[nseq + __popc(prev)] = Seq{ mpos_l - lit0, len, mpos_l - cand };
      nseq += __popc(sel);
      if (!extend) {
        p = __shfl_sync(0xffffffffu, end_l, last);
        lit_start = p;
        break; // the chain ended: no hit starts at or after p
      }
      // long match: the warp extends it
      const uint32_t mpos = base + uint32_t(last) * step;
      const uint32_t src = __shfl_sync(0xffffffffu, cand, last);
      const uint32_t ls = __shfl_sync(0xffffffffu, lit0, last);
      uint32_t mlen = __shfl_sync(0xffffffffu, len, last);
      for (;;) {
        const uint32_t a = mpos + mlen + lane, b = src + mlen + lane;
        const bool same = a < end && bytes[a] == bytes[b];
        const unsigned eq = __ballot_sync(0xffffffffu, same);
        if (eq == 0xffffffffu) {
          mlen += 32;
          continue;
        }
        mlen += __ffs(int(~eq)) - 1;
        break;
      }
      if (lane == 0)
        out[nseq - 1] = Seq{ mpos - ls, mlen, mpos - src };
      p = mpos + mlen;
      lit_start = p;
    }
  };
  // Two windows (a, b) per iteration, probed side by side: b's probes do
  // not see a's positions in the table (b finds them only as runs or short
  // periods), in exchange for twice the independent work per step.
  while (w0 < lim) {
    const uint32_t step = 1 + ((w0 > lit_start ? w0 - lit_start : 0) >> strength);
    const uint32_t qa = w0 + lane * step, qb = qa + 32 * step;
    const bool va = qa < lim && qa + 4 <= end, vb = qb < lim && qb + 4 <= end;
    uint32_t xa = 0, xb = 0, ha = 0, hb = 0, ca = 0, cb = 0;
    bool oka = false, okb = false;
    if (va) {
      xa = word_at(words, qa);
      ha = hash4(xa);
    }
    if (vb) {
      xb = word_at(words, qb);
      hb = hash4(xb);
    }
    const uint16_t ta = va ? table[ha] : uint16_t(0xFFFF);
    const uint16_t tb = vb ? table[hb] : uint16_t(0xFFFF);
    // entries can be ahead of q: a window skipped into a long match leaves
    // later positions in the table
    if (ta != 0xFFFF && ta < qa) {
      ca = ta;
      oka = word_at(words, ca) == xa;
    }
    if (tb != 0xFFFF && tb < qb) {
      cb = tb;
      okb = word_at(words, cb) == xb;
    }
    // runs and short periods (1, 2, 4 positions back) within the windows
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const uint32_t d = 1u << i;
      const uint32_t pa = __shfl_up_sync(0xffffffffu, xa, d);
      const uint32_t pb0 = __shfl_up_sync(0xffffffffu, xb, d);
      const uint32_t pb1 = __shfl_sync(0xffffffffu, xa, (lane + 32 - d) & 31);
      const uint32_t pb = uint32_t(lane) >= d ? pb0 : pb1;
      if (va && !oka && uint32_t(lane) >= d && pa == xa) {
        ca = qa - d * step;
        oka = true;
      }
      // (when b's position is valid every earlier position is too)
      if (vb && !okb && pb == xb) {
        cb = qb - d * step;
        okb = true;
      }
    }
    uint32_t la = oka ? lane_match(words, bytes, qa, ca, end) : 0;
    uint32_t lb = okb ? lane_match(words, bytes, qb, cb, end) : 0;
    if (wide) { // earlier regions, for lanes without a good local match
      const bool pa = va && la < kWideProbeBelow, pb = vb && lb < kWideProbeBelow;
      if (pa || pb)
        wide_probe2(*wide, words, r0, step, wide_lane(*wide, pa, qa, xa, end, oka, la), oka,
                    ca, la, wide_lane(*wide, pb, qb, xb, end, okb, lb), okb, cb, lb);
    }
    __syncwarp();
    if (va)
      table[ha] = uint16_t(qa);
    __syncwarp();
    if (vb)
      table[hb] = uint16_t(qb);
    __syncwarp();
    const unsigned hits_a = __ballot_sync(0xffffffffu, oka && la >= min_match);
    const unsigned hits_b = __ballot_sync(0xffffffffu, okb && lb >= min_match);
    take(hits_a, w0, step, ca, la);
    take(hits_b, w0 + 32 * step, step, cb, lb);
    // next windows; skip those inside a long match
    w0 = p >= w0 + 128 * step ? p : w0 + 64 * step;
  }
  __syncwarp();
  return SegInfo{ nseq, (s1 - r0) - lit_start };
}

// Literal bytes of a parsed segment (those its matches do not cover), in
// order, compacted in place to the start of the segment's bytes in the
// staged region; returns their count.  Call after every warp of the CTA
// has finished parsing (the region is no longer read as history).
// `bitmap` is kSegBytes / 8 bytes of the warp's (free again) hash table.
__device__ inline uint32_t lz77_compact_literals(uint32_t* words,
                                                 uint32_t r0,
                                                 uint32_t s0,
                                                 uint32_t s1,
                                                 const Seq* sq,
                                                 uint32_t nseq,
                                                 uint32_t* bitmap)
{
  const unsigned lane = threadIdx.x & 31;
  const uint32_t n = s1 - s0;
  if (nseq == 0) // every byte is a literal, already in place
    return n;
  const uint32_t nwords = (n + 31) >> 5;
  // bit i of word j: position 32 j + i is a literal
  for (uint32_t j = lane; j < nwords; j += 32) {
    const uint32_t lo = 32 * j;
    bitmap[j] = n - lo >= 32 ? 0xFFFFFFFFu : (1u << (n - lo)) - 1;
  }
  __syncwarp();
  // clear the bits under every match
  uint32_t pos = 0;
  for (uint32_t base = 0; base < nseq; base += 32) {
    const uint32_t i = base + lane;
    uint32_t lt = 0, ml = 0;
    if (i < nseq) {
      const Seq q = sq[i];
      lt = q.lit;
      ml = q.match;
    }
    uint32_t ex = lt + ml;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, ex, o);
      if (lane >= o)
        ex += y;
    }
    const uint32_t tot = __shfl_sync(0xffffffffu, ex, 31);
    ex -= lt + ml;
    uint32_t a = pos + ex + lt; // match start, segment-relative
    const uint32_t e = a + ml;
    while (a < e) {
      const uint32_t j = a >> 5, b = a & 31;
      const uint32_t k = min(32u - b, e - a);
      const uint32_t mask = (k == 32 ? 0xFFFFFFFFu : ((1u << k) - 1)) << b;
      if (mask == 0xFFFFFFFFu)
        bitmap[j] = 0;
      else
        atomicAnd(bitmap + j, ~mask);
      a += k;
    }
    pos += tot;
  }
  __syncwarp();
  // compact 1 KiB at a time: every lane reads its 32 bytes into registers,
  // then writes their literal bytes at the final place (never after the
  // source, so later bytes are still intact).  Lanes start at different
  // bytes of their word (the place of each byte follows from the bitmap)
  // so that their stores fall in different banks.
  uint8_t* bytes = reinterpret_cast<uint8_t*>(words) + (s0 - r0);
  const int rot = int(lane & 7) * 4;
  uint32_t out = 0;
  for (uint32_t c = 0; c < nwords; c += 32) {
    const uint32_t j = c + lane;
    uint32_t m = 0;
    uint4 lo4 = make_uint4(0, 0, 0, 0), hi4 = make_uint4(0, 0, 0, 0);
    if (j < nwords) {
      m = bitmap[j];
      const uint4* src = reinterpret_cast<const uint4*>(bytes + 32 * j);
      lo4 = src[0];
      hi4 = src[1];
    }
    const uint32_t cnt = __popc(m);
    uint32_t ex = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, ex, o);
      if (lane >= o)
        ex += y;
    }
    const uint32_t tot = __shfl_sync(0xffffffffu, ex, 31);
    ex -= cnt;
    __syncwarp();
    const uint32_t d = out + ex;
    // all 32 bytes literal (the common case): whole aligned words, bytes
    // only at the unaligned ends
    uint32_t mr = m == 0xFFFFFFFFu ? 0u : __funnelshift_r(m, m, rot);
    if (m == 0xFFFFFFFFu) {
      const uint32_t w8[9] = { lo4.x, lo4.y, lo4.z, lo4.w, hi4.x, hi4.y, hi4.z, hi4.w, 0 };
      const uint32_t h = (4 - (d & 3)) & 3; // head bytes
#pragma unroll
      for (uint32_t j = 0; j < 3; ++j)
        if (j < h)
          bytes[d + j] = uint8_t(w8[0] >> (8 * j));
      uint32_t* dw = reinterpret_cast<uint32_t*>(bytes + d + h);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (i < 7 || h == 0)
          dw[i] = __funnelshift_r(w8[i], w8[i + 1], h * 8);
#pragma unroll
      for (uint32_t j = 1; j < 4; ++j)
        if (h > 0 && j >= h)
          bytes[d + 28 + j] = uint8_t(w8[7] >> (8 * j));
    }
    while (mr) {
      const int i = (__ffs(int(mr)) - 1 + rot) & 31;
      mr &= mr - 1;
      const uint32_t wd = i < 16 ? (i < 8 ? (i < 4 ? lo4.x : lo4.y) : (i < 12 ? lo4.z : lo4.w))
                                 : (i < 24 ? (i < 20 ? hi4.x : hi4.y) : (i < 28 ? hi4.z : hi4.w));
      bytes[d + __popc(m & ((1u << i) - 1))] = uint8_t(wd >> ((i & 3) * 8));
    }
    out += tot;
    __syncwarp();
  }
  return out;
}

// The wide window's first pass: one CTA per region, the last position of
// every hash of 4 bytes within the region (a maximum: the same table in
// any thread order), written as 16-bit entries (offset and tag, above).
// `in_at(c)` gives chunk c's bytes; `rpc` regions per chunk.  The region is
// staged and the table built in dynamic shared memory
// (wide_index_smem(hlog) bytes).
constexpr uint32_t kWideIndexThreads = 512;
inline size_t wide_index_smem(int hlog)
{
  return size_t(wide_entries(hlog) + kRegionStageWords) * sizeof(uint32_t);
}

template<typename Batch>
__global__ void __launch_bounds__(kWideIndexThreads)
lz77_index_k(Batch b, uint16_t* tables, uint32_t rpc, int hlog)
{
  CHUCKY_DYN_SHARED(uint32_t, sm); // table, then the staged region
  const uint32_t entries = uint32_t(wide_entries(hlog));
  uint32_t* tbl = sm;
  uint32_t* words = sm + entries;
  const uint64_t chunk = blockIdx.x / rpc;
  const uint32_t region = blockIdx.x % rpc;
  const uint8_t* base = b.in_at(chunk);
  const uint32_t r0 = region * kRegionBytes;
  const uint32_t r1 = min(b.chunk_bytes, r0 + kRegionBytes);
  uint4* t4 = reinterpret_cast<uint4*>(tbl);
  for (uint32_t i = threadIdx.x; i < entries / 4; i += blockDim.x)
    t4[i] = make_uint4(0, 0, 0, 0);
  lz77_stage_region(base, r0, r1, words, threadIdx.x, blockDim.x); // (ends with a barrier)
  // positions whose 4 bytes lie in the region: (offset + 1) << 2 | tag,
  // so the maximum is the last position
  for (uint32_t p = threadIdx.x; p + 4 <= r1 - r0; p += blockDim.x) {
    const uint32_t v = word_at(words, p);
    atomicMax(&tbl[hash4w(v, hlog)], ((p + 1) << 2) | wide_tag(v, hlog));
  }
  __syncthreads();
  // two entries per thread and step: 4-byte stores
  auto entry = [](uint32_t a) {
    return a ? ((a & 3u) << 14) | ((a >> 2) - 1) : 0xFFFFu;
  };
  uint32_t* out = reinterpret_cast<uint32_t*>(tables + (chunk * rpc + region) * entries);
  for (uint32_t i = threadIdx.x; i < entries / 2; i += blockDim.x)
    out[i] = entry(tbl[2 * i]) | (entry(tbl[2 * i + 1]) << 16);
}

// Launches lz77_index_k over every region of a batch (`tables`: 4-byte
// aligned, n_chunks * rpc * wide_entries(hlog) entries).
template<typename Batch>
inline cudaError_t lz77_launch_index(const Batch& b, uint16_t* tables, uint32_t rpc,
                                     int hlog, cudaStream_t st)
{
  const size_t smem = wide_index_smem(hlog);
  cudaError_t e = cudaFuncSetAttribute(lz77_index_k<Batch>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(smem));
  if (e != cudaSuccess)
    return e;
  CHUCKY_LAUNCH(lz77_index_k<Batch>, unsigned(b.n_chunks * rpc), kWideIndexThreads, smem,
                st, b, tables, rpc, hlog);
  return cudaGetLastError();
}

} // namespace chucky
