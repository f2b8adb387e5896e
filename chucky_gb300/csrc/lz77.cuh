// Warp-parallel greedy LZ77 match finder shared by the LZ4 and zstd encoders.
//
// A chunk is cut into segments of kSegBytes; one warp parses one segment
// with a private hash table (12-bit hash of 4 bytes -> last position, 16-bit
// positions relative to the segment) in shared memory.  Each step looks at
// the 32 positions p..p+31 at once: every lane hashes the 4 bytes at its
// position, probes the table and verifies the candidate (or, for runs and
// periods of 1, 2 or 4 bytes, the lane 1, 2 or 4 positions back in the same
// step); the lowest lane
// with a verified match wins (greedy, earliest match first), the warp
// extends it 32 bytes per step, and parsing resumes after the match.  All 32
// positions are inserted after the probe, so the table only ever holds
// earlier positions.  Matches stay inside the segment, so segments are
// independent and the parse is deterministic.
//
// Output per segment: sequences (literal length, match length, offset) in
// scratch, the sequence count and the trailing literal count.
#pragma once

#include <stdint.h>

namespace chucky {

constexpr int kSegLog = 14;
constexpr uint32_t kSegBytes = 1u << kSegLog; // 16 KiB
constexpr int kHashLog = 12;
constexpr uint32_t kMaxSeqPerSeg = kSegBytes / 4 + 1;

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

// 4 bytes at an arbitrary byte position of a 4-byte aligned buffer; the
// buffer must stay readable 4 bytes past `pos + 3`.
__device__ __forceinline__ uint32_t load_u32(const uint8_t* base, uint32_t pos)
{
  const uint32_t* w = reinterpret_cast<const uint32_t*>(base) + (pos >> 2);
  const uint32_t lo = __ldg(w), hi = __ldg(w + 1);
  return __funnelshift_r(lo, hi, (pos & 3) * 8);
}

__device__ __forceinline__ uint32_t hash4(uint32_t v)
{
  return (v * 2654435761u) >> (32 - kHashLog);
}

// Parse segment [s0, s1) of a chunk at `base` (4-byte aligned).  Matches
// may start before `start_limit` and end at or before `match_end`; bytes
// from `s0` on are visible to the matcher.  `table` holds 1 << kHashLog
// u16 entries private to this warp.
__device__ inline SegInfo lz77_parse_segment(const uint8_t* base,
                                             uint32_t s0,
                                             uint32_t s1,
                                             uint32_t start_limit,
                                             uint32_t match_end,
                                             uint16_t* table,
                                             Seq* out,
                                             uint32_t min_match = 4)
{
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < (1 << kHashLog); i += 32)
    table[i] = 0xFFFF;
  __syncwarp();
  // The bytes under the 32 probed positions come from a 256-byte window
  // held in registers (lane i: words i and 32+i), refilled with coalesced
  // 128-byte warp loads, so probing costs no memory latency.
  const uint32_t* wbase = reinterpret_cast<const uint32_t*>(base);
  uint32_t win = s0 & ~3u; // byte position of the window start
  uint32_t cur = __ldg(wbase + (win >> 2) + lane);
  uint32_t nxt = __ldg(wbase + (win >> 2) + 32 + lane);
  uint32_t p = s0, lit_start = s0, nseq = 0;
  while (p < start_limit) {
    if (p >= win + 128) { // slide (or jump) the window
      if (p < win + 256) {
        cur = nxt;
        win += 128;
        nxt = __ldg(wbase + (win >> 2) + 32 + lane);
      } else {
        win = p & ~3u;
        cur = __ldg(wbase + (win >> 2) + lane);
        nxt = __ldg(wbase + (win >> 2) + 32 + lane);
      }
    }
    const uint32_t q = p + lane;
    const bool valid = q < start_limit && q + 4 <= match_end;
    // words j and j+1 of the window hold bytes [q, q+4)
    const uint32_t j = (q - win) >> 2; // <= 63 - 1 since p < win + 128
    const uint32_t a0 = __shfl_sync(0xffffffffu, cur, j & 31);
    const uint32_t b0 = __shfl_sync(0xffffffffu, nxt, j & 31);
    const uint32_t a1 = __shfl_sync(0xffffffffu, cur, (j + 1) & 31);
    const uint32_t b1 = __shfl_sync(0xffffffffu, nxt, (j + 1) & 31);
    const uint32_t lo = j < 32 ? a0 : b0;
    const uint32_t hi = (j + 1) < 32 ? a1 : b1;
    uint32_t v = 0, h = 0, cand = 0xFFFFFFFFu;
    bool ok = false;
    if (valid) {
      v = __funnelshift_r(lo, hi, (q & 3) * 8);
      h = hash4(v);
      const uint16_t t = table[h];
      // entries can be ahead of q: positions probed in an earlier step
      // may lie past where the last match ended
      if (t != 0xFFFF && s0 + t < q) {
        cand = s0 + t;
        ok = load_u32(base, cand) == v;
      }
    }
    // runs and short periods (1, 2, 4 bytes) match positions of this same
    // step that are not in the table yet
    {
      const uint32_t v1 = __shfl_up_sync(0xffffffffu, v, 1);
      const uint32_t v2 = __shfl_up_sync(0xffffffffu, v, 2);
      const uint32_t v4 = __shfl_up_sync(0xffffffffu, v, 4);
      if (valid && !ok) {
        if (lane >= 1 && v1 == v) {
          cand = q - 1;
          ok = true;
        } else if (lane >= 2 && v2 == v) {
          cand = q - 2;
          ok = true;
        } else if (lane >= 4 && v4 == v) {
          cand = q - 4;
          ok = true;
        }
      }
    }
    __syncwarp();
    if (valid)
      table[h] = uint16_t(q - s0);
    __syncwarp();
    const unsigned hit = __ballot_sync(0xffffffffu, ok);
    if (!hit) {
      p += 32;
      continue;
    }
    const int k = __ffs(hit) - 1;
    const uint32_t mpos = __shfl_sync(0xffffffffu, q, k);
    const uint32_t src = __shfl_sync(0xffffffffu, cand, k);
    // extend 32 bytes per step
    uint32_t len = 4;
    for (;;) {
      const uint32_t a = mpos + len + lane, b = src + len + lane;
      const bool same = a < match_end && base[a] == base[b];
      const unsigned eq = __ballot_sync(0xffffffffu, same);
      if (eq == 0xffffffffu) {
        len += 32;
        continue;
      }
      len += __ffs(~eq) - 1;
      break;
    }
    if (len < min_match) { // too short to pay for a sequence: literals
      p = mpos + 1;
      continue;
    }
    if (lane == 0)
      out[nseq] = Seq{ mpos - lit_start, len, mpos - src };
    ++nseq;
    p = mpos + len;
    lit_start = p;
  }
  __syncwarp();
  return SegInfo{ nseq, s1 - lit_start };
}

} // namespace chucky
