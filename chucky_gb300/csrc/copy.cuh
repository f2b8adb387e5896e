// Cooperative byte copy for arbitrary source and destination alignment.
//
// The destination is written with aligned 16-byte stores: each vector is
// assembled from five aligned 32-bit source words by funnel shifts, so only
// the (< 16 byte) head and tail go byte by byte.  `lane`/`lanes` describe the
// cooperating threads (a warp, a CTA, or a piece of a grid).  The source
// must stay readable 20 bytes past its end.
#pragma once

#include <stdint.h>

namespace chucky {

__device__ __forceinline__ void copy_bytes(uint8_t* dst,
                                           const uint8_t* src,
                                           uint64_t n,
                                           unsigned lane,
                                           unsigned lanes)
{
  const uint64_t lead = (16 - (reinterpret_cast<uintptr_t>(dst) & 15)) & 15;
  const uint64_t head = n < lead ? n : lead;
  for (uint64_t i = lane; i < head; i += lanes)
    dst[i] = src[i];
  const uint64_t nvec = (n - head) >> 4;
  const uint8_t* s = src + head;
  uint4* d = reinterpret_cast<uint4*>(dst + head);
  const uintptr_t sa = reinterpret_cast<uintptr_t>(s);
  const uint32_t* w = reinterpret_cast<const uint32_t*>(sa & ~uintptr_t(3));
  const unsigned sh = unsigned(sa & 3) * 8;
  // kBatch vectors per thread and step: all their loads are issued before
  // the first store (the compiler may not move a load above a store that
  // could alias it), so a thread waits on memory once per step
  constexpr int kBatch = 4;
  uint64_t v = lane;
  for (; v + (kBatch - 1) * uint64_t(lanes) < nvec; v += kBatch * uint64_t(lanes)) {
    uint32_t r[kBatch][5];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const uint32_t* p = w + 4 * (v + u * uint64_t(lanes));
#pragma unroll
      for (int k = 0; k < 5; ++k)
        r[u][k] = p[k];
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      uint4 o;
      o.x = __funnelshift_r(r[u][0], r[u][1], sh);
      o.y = __funnelshift_r(r[u][1], r[u][2], sh);
      o.z = __funnelshift_r(r[u][2], r[u][3], sh);
      o.w = __funnelshift_r(r[u][3], r[u][4], sh);
      d[v + u * uint64_t(lanes)] = o;
    }
  }
  for (; v < nvec; v += lanes) {
    const uint32_t* p = w + 4 * v;
    const uint32_t w0 = p[0], w1 = p[1], w2 = p[2], w3 = p[3], w4 = p[4];
    uint4 o;
    o.x = __funnelshift_r(w0, w1, sh);
    o.y = __funnelshift_r(w1, w2, sh);
    o.z = __funnelshift_r(w2, w3, sh);
    o.w = __funnelshift_r(w3, w4, sh);
    d[v] = o;
  }
  const uint64_t done = head + (nvec << 4);
  for (uint64_t i = done + lane; i < n; i += lanes)
    dst[i] = src[i];
}

} // namespace chucky
