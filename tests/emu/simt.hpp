// CPU SIMT emulation of the CUDA subset the encoder kernels use -- TEST
// INFRASTRUCTURE ONLY.
//
// One CTA runs at a time on blockDim.x host threads; __syncthreads is a
// barrier over the CTA, warp collectives (__shfl*_sync, __ballot_sync,
// __syncwarp) exchange through per-warp slots between two warp barriers.
// __shared__ variables become function statics (one CTA runs at a time).
// Built with AddressSanitizer and UBSan (tests/test_codec_emu.py), every
// out-of-bounds or misaligned access of a kernel aborts with a report;
// misaligned 32-bit atomics are checked here as well.  The emulation lets
// the encoders be tested and debugged on the CPU, against the stock
// decoders, without a GPU.
#pragma once

#include <atomic>
#include <barrier>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <math.h>
#include <thread>
#include <vector>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __shared__ static
#define __constant__ static const
#define __launch_bounds__(...)
#define __restrict__
#define __grid_constant__
#define __align__(n) __attribute__((aligned(n)))

typedef int cudaError_t;
typedef void* cudaStream_t;
enum
{
  cudaSuccess = 0,
  cudaErrorInvalidValue = 1,
  cudaErrorNotSupported = 801
};

struct uint4
{
  unsigned x, y, z, w;
};

inline uint4 make_uint4(unsigned x, unsigned y, unsigned z, unsigned w)
{
  return uint4{ x, y, z, w };
}

struct dim3
{
  unsigned x = 1, y = 1, z = 1;
};

namespace simt {

extern thread_local dim3 threadIdx_, blockIdx_;
extern dim3 blockDim_, gridDim_;

struct Cta
{
  std::barrier<>* all = nullptr;
  std::vector<std::barrier<>*> warp;
  std::vector<uint64_t> slot; // one 64-bit slot per thread
};
extern Cta* cta;

inline void warp_sync()
{
  cta->warp[threadIdx_.x / 32]->arrive_and_wait();
}

template<typename T>
inline T shfl_generic(T v, int src_lane)
{
  const unsigned me = threadIdx_.x, base = me & ~31u;
  uint64_t bits = 0;
  std::memcpy(&bits, &v, sizeof(T));
  warp_sync();
  cta->slot[me] = bits;
  warp_sync();
  const uint64_t got = (src_lane >= 0 && src_lane < 32) ? cta->slot[base + src_lane]
                                                         : bits;
  warp_sync();
  T out;
  std::memcpy(&out, &got, sizeof(T));
  return out;
}

void fail(const char* what);

} // namespace simt

#define threadIdx simt::threadIdx_
#define blockIdx simt::blockIdx_
#define blockDim simt::blockDim_
#define gridDim simt::gridDim_

inline void __syncthreads()
{
  simt::cta->all->arrive_and_wait();
}
inline void __syncwarp(unsigned = 0xffffffffu)
{
  simt::warp_sync();
}
template<typename T>
inline T __shfl_sync(unsigned, T v, int lane)
{
  return simt::shfl_generic(v, lane);
}
template<typename T>
inline T __shfl_up_sync(unsigned, T v, unsigned d)
{
  const int lane = int(threadIdx.x & 31);
  const int src = lane - int(d);
  T r = simt::shfl_generic(v, src < 0 ? lane : src);
  return r;
}
template<typename T>
inline T __shfl_xor_sync(unsigned, T v, int m)
{
  return simt::shfl_generic(v, int(threadIdx.x & 31) ^ m);
}
inline unsigned __ballot_sync(unsigned, int pred)
{
  const unsigned me = threadIdx.x, base = me & ~31u;
  simt::warp_sync();
  simt::cta->slot[me] = pred ? 1 : 0;
  simt::warp_sync();
  unsigned m = 0;
  for (int i = 0; i < 32; ++i)
    m |= unsigned(simt::cta->slot[base + i] & 1) << i;
  simt::warp_sync();
  return m;
}
inline int __all_sync(unsigned mask, int pred)
{
  return __ballot_sync(mask, pred) == 0xffffffffu;
}
inline unsigned __match_any_sync(unsigned, unsigned v)
{
  const unsigned me = threadIdx.x, base = me & ~31u;
  simt::warp_sync();
  simt::cta->slot[me] = v;
  simt::warp_sync();
  unsigned m = 0;
  for (int i = 0; i < 32; ++i)
    m |= unsigned(simt::cta->slot[base + i] == v) << i;
  simt::warp_sync();
  return m;
}
inline int __ffs(unsigned x)
{
  return x ? __builtin_ctz(x) + 1 : 0;
}
inline int __clz(unsigned x)
{
  return x ? __builtin_clz(x) : 32;
}
inline int __popc(unsigned x)
{
  return __builtin_popcount(x);
}
inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned s)
{
  const uint64_t v = (uint64_t(hi) << 32) | lo;
  return unsigned(v >> (s & 31));
}
inline uint64_t __umul64hi(uint64_t a, uint64_t b)
{
  return uint64_t((unsigned __int128)a * b >> 64);
}
template<typename T>
inline T __ldg(const T* p)
{
  return *p;
}
inline unsigned atomicAdd(unsigned* p, unsigned v)
{
  return std::atomic_ref<unsigned>(*p).fetch_add(v);
}
inline unsigned atomicOr(unsigned* p, unsigned v)
{
  if (reinterpret_cast<uintptr_t>(p) & 3)
    simt::fail("misaligned 32-bit atomicOr");
  return std::atomic_ref<unsigned>(*p).fetch_or(v);
}
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v)
{
  return std::atomic_ref<unsigned long long>(*p).fetch_add(v);
}
inline unsigned atomicMin(unsigned* p, unsigned v)
{
  std::atomic_ref<unsigned> a(*p);
  unsigned cur = a.load();
  while (v < cur && !a.compare_exchange_weak(cur, v)) {
  }
  return cur;
}
inline unsigned atomicMax(unsigned* p, unsigned v)
{
  std::atomic_ref<unsigned> a(*p);
  unsigned cur = a.load();
  while (cur < v && !a.compare_exchange_weak(cur, v)) {
  }
  return cur;
}
inline int atomicMax(int* p, int v)
{
  std::atomic_ref<int> a(*p);
  int cur = a.load();
  while (cur < v && !a.compare_exchange_weak(cur, v)) {
  }
  return cur;
}
inline unsigned atomicAnd(unsigned* p, unsigned v)
{
  if (reinterpret_cast<uintptr_t>(p) & 3)
    simt::fail("misaligned 32-bit atomicAnd");
  return std::atomic_ref<unsigned>(*p).fetch_and(v);
}
using std::max;
using std::min;

namespace simt {

// Run `body` for every CTA of the grid on block.x host threads.
void launch(unsigned grid, unsigned block, const std::function<void()>& body);

} // namespace simt

#define CHUCKY_DYN_SHARED(T, name) static T name[1 << 20]
#define CHUCKY_LAUNCH(kernel, grid, block, smem, stream, ...)                  \
  simt::launch(unsigned(grid), unsigned(block), [&] { kernel(__VA_ARGS__); })

inline cudaError_t cudaGetLastError()
{
  return cudaSuccess;
}

inline cudaError_t cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t = nullptr)
{
  std::memset(p, v, n);
  return cudaSuccess;
}

enum cudaFuncAttribute
{
  cudaFuncAttributeMaxDynamicSharedMemorySize = 8
};

template<typename F>
inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int)
{
  return cudaSuccess;
}
