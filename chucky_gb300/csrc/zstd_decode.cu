// zstd frame decoder: zstd frames (the CODEC_ZSTD chunk format) back to
// chunk bytes on the device, for on-device verification and readback of
// stores.  The reference decodes its chunks on the host with
// ZSTD_decompress (src/cpu/compress.c:85-93, tests/test_compress.c:30-165);
// this is the same contract on the GPU, written from the format's
// specification (RFC 8878) for any conforming frame, not only this
// library's: skippable frames, raw / RLE / compressed blocks, raw / RLE /
// Huffman (1 or 4 streams, direct or FSE-coded weights, treeless) literals,
// predefined / RLE / FSE / repeat sequence tables, repeat offsets, several
// frames one after another.  Frames with a dictionary are reported as
// unsupported; a content checksum is skipped, not verified.
//
// One CTA per chunk, its first thread decoding (the format is sequential
// within a block); the decoding tables live in shared memory.  Literals are
// Huffman-decoded on demand while the sequences execute (stream by stream,
// in order), so no literal buffer is needed.  Every read is checked against
// the chunk's compressed size and every write against chunk_bytes; a
// malformed frame sets its status and stops.
#include "chucky_gb300.h"
#include "kernels_codec.hpp"
#include "launch.cuh"
#include "zstd_format.cuh"

#include <cuda_runtime.h>

namespace chucky {

namespace {

enum : uint32_t
{
  kZOk = 0,
  kZTruncated = 1,   // the input ends inside a header, table or stream
  kZCorrupt = 2,     // invalid field, table, bitstream or offset
  kZOverflow = 3,    // it would write more than chunk_bytes
  kZShort = 4,       // it decodes to fewer than chunk_bytes
  kZUnsupported = 5, // a dictionary frame
};

constexpr uint32_t kBlockMax = 128u << 10;
constexpr int kDecHufBits = 11;

struct FseEntry
{
  uint16_t base; // next state base
  uint8_t sym;
  uint8_t nb;    // bits to read for the next state
};

struct FseTable
{
  FseEntry e[1 << 9];
  int al; // accuracy log; -1: none yet (repeat mode invalid)
};

struct DecShared
{
  uint16_t huf[1 << kDecHufBits]; // symbol | bits << 8
  int huf_bits;                   // -1: no table yet
  FseTable ll, ml, of;
  FseEntry w[1 << 6];             // Huffman weights
  int16_t norm[64];
  uint16_t next[64];
  uint8_t weight[256];
};

__device__ __forceinline__ int dec_highbit(uint32_t v) { return 31 - __clz(int(v)); }

// ---- bit readers ------------------------------------------------------------

// A backward bitstream (RFC 8878 4.1): the last byte's highest set bit marks
// the end; bits are read from just below it towards the first byte, each
// field most significant bit first.  Bits [0, pos) are still unread.
struct BitIn
{
  const uint8_t* b = nullptr;
  int64_t pos = 0;

  __device__ bool init(const uint8_t* p, uint64_t n)
  {
    if (n == 0 || p[n - 1] == 0)
      return false;
    b = p;
    pos = int64_t(n) * 8 - 8 + dec_highbit(p[n - 1]);
    return true;
  }
  // bits [start, start + nb) (0 <= start, nb <= 32) as an integer
  __device__ uint32_t get(int64_t start, int nb) const
  {
    if (nb == 0)
      return 0;
    const int64_t first = start >> 3, last = (start + nb - 1) >> 3;
    uint64_t v = 0;
    for (int64_t i = last; i >= first; --i)
      v = (v << 8) | b[i];
    v >>= (start & 7);
    return uint32_t(v & ((nb == 32) ? 0xFFFFFFFFull : ((1ull << nb) - 1)));
  }
  // the next nb bits (zeros for bits before the stream's start, which make
  // pos negative: the caller checks pos)
  __device__ uint32_t read(int nb)
  {
    pos -= nb;
    if (pos >= 0)
      return get(pos, nb);
    const int64_t have = pos + nb; // bits still there
    if (have <= 0)
      return 0;
    return get(0, int(have)) << (nb - int(have));
  }
  // the next nb bits without consuming them (zeros past the start)
  __device__ uint32_t peek(int nb) const
  {
    if (pos >= nb)
      return get(pos - nb, nb);
    if (pos <= 0)
      return 0;
    return get(0, int(pos)) << (nb - int(pos));
  }
};

// FSE table description (RFC 8878 4.1.1): a forward little-endian bitstream
// of normalized counts.  Returns the bytes it takes, or 0 when malformed.
__device__ uint32_t read_ncount(const uint8_t* p, uint64_t avail, int max_al, int max_sym,
                                int16_t* norm, int* nsym, int* al_out)
{
  uint64_t bit = 0;
  auto peek32 = [&](uint64_t at) -> uint32_t {
    uint64_t v = 0;
    const uint64_t byte = at >> 3;
    for (int k = 4; k >= 0; --k)
      v = (v << 8) | (byte + k < avail ? p[byte + k] : 0u);
    return uint32_t(v >> (at & 7));
  };
  if (avail == 0)
    return 0;
  const int al = int(peek32(0) & 15) + 5;
  bit = 4;
  if (al > max_al)
    return 0;
  int remaining = (1 << al) + 1;
  int threshold = 1 << al;
  int nb = al + 1;
  int s = 0;
  bool prev0 = false;
  while (remaining > 1 && s <= max_sym) {
    if (prev0) { // runs of zero counts: 2-bit repeat flags
      int n0 = 0;
      for (;;) {
        const uint32_t r = peek32(bit) & 3;
        bit += 2;
        n0 += int(r);
        if (r != 3)
          break;
        if (bit > avail * 8)
          return 0;
      }
      if (s + n0 > max_sym) // a count must follow the zeros
        return 0;
      for (int k = 0; k < n0; ++k)
        norm[s++] = 0;
    }
    const int mx = (2 * threshold - 1) - remaining;
    const uint32_t v = peek32(bit);
    int count;
    if (int(v & uint32_t(threshold - 1)) < mx) {
      count = int(v & uint32_t(threshold - 1));
      bit += uint64_t(nb - 1);
    } else {
      count = int(v & uint32_t(2 * threshold - 1));
      if (count >= threshold)
        count -= mx;
      bit += uint64_t(nb);
    }
    --count; // -1: a "less than one" probability
    remaining -= count < 0 ? -count : count;
    if (remaining < 1)
      return 0;
    norm[s++] = int16_t(count);
    prev0 = count == 0;
    while (remaining < threshold) {
      --nb;
      threshold >>= 1;
    }
    if (bit > avail * 8)
      return 0;
  }
  if (remaining != 1)
    return 0;
  *nsym = s;
  *al_out = al;
  return uint32_t((bit + 7) >> 3);
}

// Decoding table from normalized counts (RFC 8878 4.1.1).
__device__ bool build_fse(FseEntry* t, const int16_t* norm, int nsym, int al, uint16_t* next)
{
  const int size = 1 << al;
  if (nsym < 1 || nsym > 64)
    return false;
  int total = 0; // the counts must fill the table exactly
  for (int s = 0; s < nsym; ++s)
    total += norm[s] == -1 ? 1 : (norm[s] > 0 ? norm[s] : 0);
  if (total != size)
    return false;
  int high = size - 1;
  for (int s = 0; s < nsym; ++s) {
    if (norm[s] == -1) {
      t[high--].sym = uint8_t(s);
      next[s] = 1;
    } else {
      next[s] = uint16_t(norm[s] < 0 ? 0 : norm[s]);
    }
  }
  const int step = (size >> 1) + (size >> 3) + 3, mask = size - 1;
  int pos = 0;
  for (int s = 0; s < nsym; ++s)
    for (int i = 0; i < norm[s]; ++i) {
      t[pos].sym = uint8_t(s);
      do
        pos = (pos + step) & mask;
      while (pos > high);
    }
  if (pos != 0)
    return false;
  for (int u = 0; u < size; ++u) {
    const int s = t[u].sym;
    const uint32_t ns = next[s]++;
    if (ns == 0)
      return false;
    const int nb = al - dec_highbit(ns);
    t[u].nb = uint8_t(nb);
    t[u].base = uint16_t((ns << nb) - uint32_t(size));
  }
  return true;
}

// ---- literals ---------------------------------------------------------------

struct Lits
{
  int type = 0;        // 0 raw, 1 RLE, 2 Huffman
  const uint8_t* raw = nullptr;
  uint8_t rle = 0;
  uint32_t size = 0;   // regenerated bytes
  uint32_t done = 0;
  // Huffman streams, decoded in order
  const uint8_t* s[4] = {};
  uint64_t slen[4] = {};
  uint32_t scount[4] = {};
  int nstreams = 0, cur = -1;
  uint32_t cur_left = 0;
  BitIn bi;

  // the next literal byte; false when the section is malformed
  __device__ bool next(uint8_t& v, const DecShared& S)
  {
    if (done >= size)
      return false;
    if (type == 0) {
      v = raw[done++];
      return true;
    }
    if (type == 1) {
      ++done;
      v = rle;
      return true;
    }
    while (cur_left == 0) { // the next stream (the previous one consumed exactly)
      if (cur >= 0 && bi.pos != 0)
        return false;
      if (++cur >= nstreams || !bi.init(s[cur], slen[cur]))
        return false;
      cur_left = scount[cur];
    }
    const uint16_t e = S.huf[bi.peek(S.huf_bits)];
    bi.pos -= e >> 8;
    if (bi.pos < 0)
      return false;
    v = uint8_t(e);
    --cur_left;
    ++done;
    return true;
  }
  // every literal produced and, for Huffman literals, every stream consumed
  // exactly (streams after the current one may only be empty)
  __device__ bool finished()
  {
    if (done != size)
      return false;
    if (type != 2)
      return true;
    if (cur >= 0 && bi.pos != 0)
      return false;
    while (++cur < nstreams) {
      if (scount[cur] != 0 || !bi.init(s[cur], slen[cur]) || bi.pos != 0)
        return false;
    }
    return true;
  }
};

// Huffman tree description (RFC 8878 4.2.1) -> S.huf, S.huf_bits.  Returns
// the bytes it takes, 0 when malformed.
__device__ uint32_t read_huffman(const uint8_t* p, uint64_t avail, DecShared& S)
{
  if (avail < 1)
    return 0;
  const uint32_t hb = p[0];
  int nw = 0;
  uint32_t used;
  if (hb >= 128) { // direct: 4 bits per weight
    nw = int(hb) - 127;
    used = 1 + uint32_t(nw + 1) / 2;
    if (used > avail)
      return 0;
    for (int i = 0; i < nw; ++i)
      S.weight[i] = (i & 1) ? (p[1 + i / 2] & 15) : (p[1 + i / 2] >> 4);
  } else { // FSE-coded, two interleaved states
    used = 1 + hb;
    if (used > avail || hb == 0)
      return 0;
    int nsym = 0, al = 0;
    const uint32_t d = read_ncount(p + 1, hb, 6, 15, S.norm, &nsym, &al);
    if (!d || d >= hb)
      return 0;
    if (!build_fse(S.w, S.norm, nsym, al, S.next))
      return 0;
    BitIn bi;
    if (!bi.init(p + 1 + d, hb - d))
      return 0;
    uint32_t s1 = bi.read(al), s2 = bi.read(al);
    if (bi.pos < 0)
      return 0;
    for (;;) {
      if (nw >= 255)
        return 0;
      FseEntry e = S.w[s1];
      S.weight[nw++] = e.sym;
      s1 = e.base + bi.read(e.nb);
      if (bi.pos < 0) {
        S.weight[nw++] = S.w[s2].sym;
        break;
      }
      if (nw >= 255)
        return 0;
      e = S.w[s2];
      S.weight[nw++] = e.sym;
      s2 = e.base + bi.read(e.nb);
      if (bi.pos < 0) {
        if (nw >= 255)
          return 0;
        S.weight[nw++] = S.w[s1].sym;
        break;
      }
    }
  }
  // the last weight completes the sum of 2^(w-1) to a power of two
  uint32_t total = 0;
  for (int i = 0; i < nw; ++i) {
    if (S.weight[i] > kDecHufBits)
      return 0;
    if (S.weight[i])
      total += 1u << (S.weight[i] - 1);
  }
  if (total == 0 || nw > 255)
    return 0;
  const int bits = dec_highbit(total) + 1;
  if (bits > kDecHufBits)
    return 0;
  const uint32_t rest = (1u << bits) - total;
  if (rest & (rest - 1))
    return 0;
  S.weight[nw++] = uint8_t(dec_highbit(rest) + 1);
  uint32_t start[kDecHufBits + 2] = {};
  uint32_t cnt[kDecHufBits + 2] = {};
  for (int i = 0; i < nw; ++i)
    cnt[S.weight[i]]++;
  uint32_t acc = 0;
  for (int w = 1; w <= bits; ++w) {
    start[w] = acc;
    acc += cnt[w] << (w - 1);
  }
  if (acc != (1u << bits))
    return 0;
  for (int i = 0; i < nw; ++i) {
    const int w = S.weight[i];
    if (!w)
      continue;
    const uint16_t e = uint16_t(i | ((bits + 1 - w) << 8));
    for (uint32_t u = start[w]; u < start[w] + (1u << (w - 1)); ++u)
      S.huf[u] = e;
    start[w] += 1u << (w - 1);
  }
  S.huf_bits = bits;
  return used;
}

// ---- sequences --------------------------------------------------------------

// One of the three sequence tables, in mode 0..3; returns the bytes its
// description takes (0 for predefined / repeat), or -1 when malformed.
__device__ int64_t read_seq_table(int mode, const uint8_t* p, uint64_t avail, FseTable& T,
                                  const int16_t* predef, int predef_n, int predef_al,
                                  int max_al, int max_sym, DecShared& S)
{
  if (mode == 0) {
    for (int i = 0; i < predef_n; ++i)
      S.norm[i] = predef[i];
    if (!build_fse(T.e, S.norm, predef_n, predef_al, S.next))
      return -1;
    T.al = predef_al;
    return 0;
  }
  if (mode == 1) { // one symbol, no state bits
    if (avail < 1 || p[0] > max_sym)
      return -1;
    T.e[0].sym = p[0];
    T.e[0].nb = 0;
    T.e[0].base = 0;
    T.al = 0;
    return 1;
  }
  if (mode == 2) {
    int nsym = 0, al = 0;
    const uint32_t d = read_ncount(p, avail, max_al, max_sym, S.norm, &nsym, &al);
    if (!d || !build_fse(T.e, S.norm, nsym, al, S.next))
      return -1;
    T.al = al;
    return d;
  }
  return T.al >= 0 ? 0 : -1; // repeat the previous block's table
}

struct Frame
{
  uint8_t* out;
  uint64_t cap; // chunk_bytes
  uint64_t op;  // bytes written
  uint32_t rep[3];
};

__device__ uint32_t put_literals(Frame& F, Lits& L, uint32_t n, const DecShared& S)
{
  if (n > L.size - L.done)
    return kZCorrupt;
  if (F.op + n > F.cap)
    return kZOverflow;
  if (L.type == 0) {
    for (uint32_t i = 0; i < n; ++i)
      F.out[F.op + i] = L.raw[L.done + i];
    L.done += n;
    F.op += n;
    return kZOk;
  }
  for (uint32_t i = 0; i < n; ++i) {
    uint8_t v;
    if (!L.next(v, S))
      return kZCorrupt;
    F.out[F.op++] = v;
  }
  return kZOk;
}

// One compressed block of `n` bytes at p.
__device__ uint32_t decode_block(const uint8_t* p, uint64_t n, Frame& F, DecShared& S)
{
  // literals section header
  if (n < 1)
    return kZTruncated;
  const uint32_t b0 = p[0];
  const int ltype = int(b0 & 3), fmt = int((b0 >> 2) & 3);
  Lits L;
  uint64_t at = 0;
  if (ltype <= 1) { // raw or RLE
    uint32_t size;
    if (fmt == 0 || fmt == 2) {
      size = b0 >> 3;
      at = 1;
    } else if (fmt == 1) {
      if (n < 2)
        return kZTruncated;
      size = (b0 >> 4) + (uint32_t(p[1]) << 4);
      at = 2;
    } else {
      if (n < 3)
        return kZTruncated;
      size = (b0 >> 4) + (uint32_t(p[1]) << 4) + (uint32_t(p[2]) << 12);
      at = 3;
    }
    if (size > kBlockMax)
      return kZCorrupt;
    L.size = size;
    if (ltype == 0) {
      if (at + size > n)
        return kZTruncated;
      L.type = 0;
      L.raw = p + at;
      at += size;
    } else {
      if (at + 1 > n)
        return kZTruncated;
      L.type = 1;
      L.rle = p[at];
      at += 1;
    }
  } else { // Huffman-coded, with a tree (2) or the previous one (3)
    const int hsz = fmt <= 1 ? 3 : fmt + 2; // header bytes
    if (uint64_t(hsz) > n)
      return kZTruncated;
    uint64_t v = 0;
    for (int k = hsz - 1; k >= 0; --k)
      v = (v << 8) | p[k];
    const int field = hsz == 3 ? 10 : hsz == 4 ? 14 : 18;
    const uint32_t regen = uint32_t((v >> 4) & ((1ull << field) - 1));
    const uint32_t comp = uint32_t((v >> (4 + field)) & ((1ull << field) - 1));
    const int nstreams = fmt == 0 ? 1 : 4;
    at = uint64_t(hsz);
    if (regen > kBlockMax || at + comp > n)
      return kZCorrupt;
    const uint8_t* q = p + at;
    uint64_t qn = comp;
    if (ltype == 2) {
      const uint32_t t = read_huffman(q, qn, S);
      if (!t)
        return kZCorrupt;
      q += t;
      qn -= t;
    } else if (S.huf_bits < 0) {
      return kZCorrupt;
    }
    L.type = 2;
    L.size = regen;
    L.nstreams = nstreams;
    if (nstreams == 1) {
      L.s[0] = q;
      L.slen[0] = qn;
      L.scount[0] = regen;
    } else {
      if (qn < 6)
        return kZCorrupt;
      const uint64_t l1 = q[0] | (uint32_t(q[1]) << 8);
      const uint64_t l2 = q[2] | (uint32_t(q[3]) << 8);
      const uint64_t l3 = q[4] | (uint32_t(q[5]) << 8);
      if (6 + l1 + l2 + l3 > qn)
        return kZCorrupt;
      const uint32_t seg = (regen + 3) / 4;
      if (uint64_t(seg) * 3 > regen)
        return kZCorrupt;
      L.s[0] = q + 6;
      L.s[1] = L.s[0] + l1;
      L.s[2] = L.s[1] + l2;
      L.s[3] = L.s[2] + l3;
      L.slen[0] = l1;
      L.slen[1] = l2;
      L.slen[2] = l3;
      L.slen[3] = qn - 6 - l1 - l2 - l3;
      L.scount[0] = L.scount[1] = L.scount[2] = seg;
      L.scount[3] = regen - 3 * seg;
    }
    at += comp;
  }
  // sequences section header
  if (at >= n)
    return kZTruncated;
  uint32_t nseq = p[at];
  if (nseq == 0) {
    at += 1;
  } else if (nseq < 128) {
    at += 1;
  } else if (nseq < 255) {
    if (at + 2 > n)
      return kZTruncated;
    nseq = ((nseq - 128) << 8) + p[at + 1];
    at += 2;
  } else {
    if (at + 3 > n)
      return kZTruncated;
    nseq = p[at + 1] + (uint32_t(p[at + 2]) << 8) + 0x7F00;
    at += 3;
  }
  if (nseq == 0) {
    if (at != n)
      return kZCorrupt;
    const uint32_t r = put_literals(F, L, L.size - L.done, S);
    if (r != kZOk)
      return r;
    return L.finished() ? kZOk : kZCorrupt;
  }
  if (at >= n)
    return kZTruncated;
  const uint32_t modes = p[at++];
  if (modes & 3)
    return kZCorrupt;
  int64_t d = read_seq_table(int(modes >> 6), p + at, n - at, S.ll, kLLNormD, 36, 6, 9, 35, S);
  if (d < 0)
    return kZCorrupt;
  at += uint64_t(d);
  d = read_seq_table(int((modes >> 4) & 3), p + at, n - at, S.of, kOFNormD, 29, 5, 8, 31, S);
  if (d < 0)
    return kZCorrupt;
  at += uint64_t(d);
  d = read_seq_table(int((modes >> 2) & 3), p + at, n - at, S.ml, kMLNormD, 53, 6, 9, 52, S);
  if (d < 0)
    return kZCorrupt;
  at += uint64_t(d);
  BitIn bi;
  if (at >= n || !bi.init(p + at, n - at))
    return kZCorrupt;
  uint32_t sll = bi.read(S.ll.al), sof = bi.read(S.of.al), sml = bi.read(S.ml.al);
  if (bi.pos < 0)
    return kZCorrupt;
  for (uint32_t i = 0; i < nseq; ++i) {
    const FseEntry& eo = S.of.e[sof];
    const FseEntry& em = S.ml.e[sml];
    const FseEntry& el = S.ll.e[sll];
    const uint32_t ofc = eo.sym, mlc = em.sym, llc = el.sym;
    if (ofc > 31 || mlc > 52 || llc > 35)
      return kZCorrupt;
    const uint32_t ofv = (1u << ofc) + bi.read(int(ofc));
    const uint32_t ml = kMLBase[mlc] + bi.read(kMLBits[mlc]);
    const uint32_t ll = kLLBase[llc] + bi.read(kLLBits[llc]);
    if (i + 1 < nseq) {
      sll = el.base + bi.read(el.nb);
      sml = em.base + bi.read(em.nb);
      sof = eo.base + bi.read(eo.nb);
    }
    if (bi.pos < 0)
      return kZCorrupt;
    // offsets: repeat codes (RFC 8878 3.1.2.5)
    uint32_t off;
    if (ofv > 3) {
      off = ofv - 3;
      F.rep[2] = F.rep[1];
      F.rep[1] = F.rep[0];
      F.rep[0] = off;
    } else {
      const uint32_t idx = ofv - 1 + (ll == 0 ? 1 : 0);
      if (idx == 0) {
        off = F.rep[0];
      } else if (idx == 1) {
        off = F.rep[1];
        F.rep[1] = F.rep[0];
        F.rep[0] = off;
      } else {
        off = idx == 2 ? F.rep[2] : F.rep[0] - 1;
        F.rep[2] = F.rep[1];
        F.rep[1] = F.rep[0];
        F.rep[0] = off;
      }
    }
    const uint32_t r = put_literals(F, L, ll, S);
    if (r != kZOk)
      return r;
    if (off == 0 || off > F.op)
      return kZCorrupt;
    if (F.op + ml > F.cap)
      return kZOverflow;
    for (uint32_t k = 0; k < ml; ++k, ++F.op)
      F.out[F.op] = F.out[F.op - off];
  }
  if (bi.pos != 0)
    return kZCorrupt;
  const uint32_t r = put_literals(F, L, L.size - L.done, S);
  if (r != kZOk)
    return r;
  return L.finished() ? kZOk : kZCorrupt;
}

__global__ void __launch_bounds__(32) zstd_decode_k(const uint8_t* in,
                                                    const uint64_t* in_off,
                                                    const uint64_t* in_size,
                                                    uint8_t* out,
                                                    uint64_t out_stride,
                                                    uint64_t chunk_bytes,
                                                    uint32_t* status)
{
  __shared__ DecShared S;
  if (threadIdx.x != 0)
    return;
  const uint64_t c = blockIdx.x;
  const uint8_t* p = in + in_off[c];
  const uint64_t n = in_size[c];
  Frame F{ out + c * out_stride, chunk_bytes, 0, { 1, 4, 8 } };
  uint64_t at = 0;
  uint32_t st = kZOk;
  auto le = [&](uint64_t k, int bytes) {
    uint64_t v = 0;
    for (int i = bytes - 1; i >= 0; --i)
      v = (v << 8) | p[k + i];
    return v;
  };
  while (st == kZOk && at < n) {
    if (at + 4 > n) {
      st = kZTruncated;
      break;
    }
    const uint32_t magic = uint32_t(le(at, 4));
    if ((magic & 0xFFFFFFF0u) == 0x184D2A50u) { // skippable frame
      if (at + 8 > n) {
        st = kZTruncated;
        break;
      }
      const uint64_t sz = le(at + 4, 4);
      if (at + 8 + sz > n) {
        st = kZTruncated;
        break;
      }
      at += 8 + sz;
      continue;
    }
    if (magic != 0xFD2FB528u) {
      st = kZCorrupt;
      break;
    }
    at += 4;
    if (at >= n) {
      st = kZTruncated;
      break;
    }
    const uint32_t fhd = p[at++];
    const int fcs_flag = int(fhd >> 6), single = int((fhd >> 5) & 1);
    const int checksum = int((fhd >> 2) & 1), did_flag = int(fhd & 3);
    if (fhd & 8) {
      st = kZCorrupt;
      break;
    }
    const int did_bytes = did_flag == 3 ? 4 : did_flag;
    const int fcs_bytes = fcs_flag == 0 ? (single ? 1 : 0) : (1 << fcs_flag);
    const uint64_t hdr = uint64_t(single ? 0 : 1) + uint64_t(did_bytes) + uint64_t(fcs_bytes);
    if (at + hdr > n) {
      st = kZTruncated;
      break;
    }
    if (!single)
      at += 1; // window descriptor: the whole chunk is the window here
    if (did_bytes && le(at, did_bytes) != 0) {
      st = kZUnsupported;
      break;
    }
    at += uint64_t(did_bytes);
    uint64_t fcs = ~uint64_t(0);
    if (fcs_bytes) {
      fcs = le(at, fcs_bytes) + (fcs_bytes == 2 ? 256 : 0);
      at += uint64_t(fcs_bytes);
    }
    const uint64_t frame_start = F.op;
    S.huf_bits = -1;
    S.ll.al = S.ml.al = S.of.al = -1;
    F.rep[0] = 1;
    F.rep[1] = 4;
    F.rep[2] = 8;
    for (;;) { // blocks
      if (at + 3 > n) {
        st = kZTruncated;
        break;
      }
      const uint32_t bh = uint32_t(le(at, 3));
      at += 3;
      const int last = int(bh & 1), type = int((bh >> 1) & 3);
      const uint32_t bsize = bh >> 3;
      if (type == 3 || bsize > kBlockMax) {
        st = kZCorrupt;
        break;
      }
      if (type == 1) { // RLE: one byte, bsize times
        if (at + 1 > n) {
          st = kZTruncated;
          break;
        }
        if (F.op + bsize > F.cap) {
          st = kZOverflow;
          break;
        }
        for (uint32_t k = 0; k < bsize; ++k)
          F.out[F.op + k] = p[at];
        F.op += bsize;
        at += 1;
      } else {
        if (at + bsize > n) {
          st = kZTruncated;
          break;
        }
        if (type == 0) {
          if (F.op + bsize > F.cap) {
            st = kZOverflow;
            break;
          }
          for (uint32_t k = 0; k < bsize; ++k)
            F.out[F.op + k] = p[at + k];
          F.op += bsize;
        } else if ((st = decode_block(p + at, bsize, F, S)) != kZOk) {
          break;
        }
        at += bsize;
      }
      if (last)
        break;
    }
    if (st != kZOk)
      break;
    if (fcs != ~uint64_t(0) && F.op - frame_start != fcs) {
      st = kZCorrupt;
      break;
    }
    if (checksum) { // content checksum: skipped
      if (at + 4 > n) {
        st = kZTruncated;
        break;
      }
      at += 4;
    }
  }
  if (st == kZOk && F.op != chunk_bytes)
    st = kZShort;
  status[c] = st;
}

} // namespace

cudaError_t launch_zstd_decode(const uint8_t* in,
                               const uint64_t* in_off,
                               const uint64_t* in_size,
                               uint64_t n_chunks,
                               uint8_t* out,
                               uint64_t out_stride,
                               uint64_t chunk_bytes,
                               uint32_t* status,
                               cudaStream_t st)
{
  if (!n_chunks)
    return cudaSuccess;
  note_launches(1);
  CHUCKY_LAUNCH(zstd_decode_k, unsigned(n_chunks), 32, 0, st, in, in_off, in_size, out,
                out_stride, chunk_bytes, status);
  return cudaGetLastError();
}

} // namespace chucky

extern "C" int
chucky_zstd_decode_chunks(const void* d_in,
                          const uint64_t* d_in_offsets,
                          const uint64_t* d_in_sizes,
                          size_t n_chunks,
                          void* d_out,
                          size_t out_stride,
                          size_t chunk_bytes,
                          uint32_t* d_status,
                          void* cuda_stream)
{
  if (!n_chunks)
    return 0;
  if (!d_in || !d_in_offsets || !d_in_sizes || !d_out || !d_status ||
      out_stride < chunk_bytes || n_chunks > 0x7FFFFFFFu)
    return 1;
  const cudaError_t e = chucky::launch_zstd_decode(
    static_cast<const uint8_t*>(d_in), d_in_offsets, d_in_sizes, n_chunks,
    static_cast<uint8_t*>(d_out), out_stride, chunk_bytes, d_status,
    static_cast<cudaStream_t>(cuda_stream));
  return e == cudaSuccess ? 0 : 3;
}
