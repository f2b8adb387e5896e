// Per-element LOD arithmetic shared by the Morton and tiled LOD kernels.
// Matches the reference bit for bit: widened sums for mean (u8/u16 -> u32,
// u32 -> u64, i8/i16 -> i32, i32 -> i64, f16 -> f32; 64-bit and float types
// not widened), insertion-sort median taking buf[n/2], second extreme with
// >= / <= ties (src/cpu/lod.cpp:16-127), dim-0 fold with the per-step
// overflow-safe shift for 8..32-bit integers and plain sums otherwise, and
// emit dividing float means by the count (src/cpu/lod.cpp:366-438,
// src/gpu/lod.cu:828-941).
#pragma once

#include "common.cuh"
#include "types.lod.h"

namespace chucky {

template<typename T>
__device__ __forceinline__ bool lt(T a, T b)
{
  return a < b;
}
template<>
__device__ __forceinline__ bool lt<__half>(__half a, __half b)
{
  return __half2float(a) < __half2float(b);
}

template<typename T>
__device__ __forceinline__ T from_acc(typename WideAcc<T>::type v)
{
  return T(v);
}
template<>
__device__ __forceinline__ __half from_acc<__half>(float v)
{
  return __float2half_rn(v);
}

template<typename T>
__device__ __forceinline__ typename WideAcc<T>::type to_acc(T v)
{
  return typename WideAcc<T>::type(v);
}
template<>
__device__ __forceinline__ float to_acc<__half>(__half v)
{
  return __half2float(v);
}

// Reduce src[0..n) in order.
template<typename T>
__device__ T reduce_window(const T* src, uint64_t n, int method)
{
  using A = typename WideAcc<T>::type;
  switch (method) {
    case lod_reduce_mean: {
      A sum = A(0);
      for (uint64_t j = 0; j < n; ++j)
        sum += to_acc<T>(src[j]);
      return from_acc<T>(sum / A(n));
    }
    case lod_reduce_min: {
      T v = src[0];
      for (uint64_t j = 1; j < n; ++j)
        if (lt(src[j], v))
          v = src[j];
      return v;
    }
    case lod_reduce_max: {
      T v = src[0];
      for (uint64_t j = 1; j < n; ++j)
        if (lt(v, src[j]))
          v = src[j];
      return v;
    }
    case lod_reduce_median: {
      T buf[16];
      const uint64_t m = n <= 16 ? n : 16;
      for (uint64_t j = 0; j < m; ++j)
        buf[j] = src[j];
      for (uint64_t i = 1; i < m; ++i) {
        const T key = buf[i];
        uint64_t k = i;
        while (k > 0 && lt(key, buf[k - 1])) {
          buf[k] = buf[k - 1];
          --k;
        }
        buf[k] = key;
      }
      return buf[m / 2];
    }
    case lod_reduce_max_suppressed: {
      T t1 = src[0], t2 = src[0];
      for (uint64_t j = 1; j < n; ++j) {
        const T v = src[j];
        if (!lt(v, t1)) { // v >= t1
          t2 = t1;
          t1 = v;
        } else if (lt(t2, v))
          t2 = v;
      }
      return t2;
    }
    case lod_reduce_min_suppressed: {
      T t1 = src[0], t2 = src[0];
      for (uint64_t j = 1; j < n; ++j) {
        const T v = src[j];
        if (!lt(t1, v)) { // v <= t1
          t2 = t1;
          t1 = v;
        } else if (lt(v, t2))
          t2 = v;
      }
      return t2;
    }
  }
  return src[0];
}

// reduce_window for a full window of N values held in registers: the same
// operations in the same order (sums in window order, the insertion sort
// of the median with its comparisons in the same sequence), with
// compile-time indices so that nothing goes through local memory.
template<typename T, int N>
__device__ __forceinline__ T reduce_full(T (&w)[N], int method)
{
  using A = typename WideAcc<T>::type;
  switch (method) {
    case lod_reduce_mean: {
      A sum = A(0);
#pragma unroll
      for (int j = 0; j < N; ++j)
        sum += to_acc<T>(w[j]);
      return from_acc<T>(sum / A(N));
    }
    case lod_reduce_min: {
      T v = w[0];
#pragma unroll
      for (int j = 1; j < N; ++j)
        if (lt(w[j], v))
          v = w[j];
      return v;
    }
    case lod_reduce_max: {
      T v = w[0];
#pragma unroll
      for (int j = 1; j < N; ++j)
        if (lt(v, w[j]))
          v = w[j];
      return v;
    }
    case lod_reduce_median: {
#pragma unroll
      for (int i = 1; i < N; ++i) {
        const T key = w[i];
        bool go = true; // still shifting larger elements up
#pragma unroll
        for (int k = i; k > 0; --k) {
          const bool sh = go && lt(key, w[k - 1]);
          const T nk = sh ? w[k - 1] : (go ? key : w[k]);
          go = sh;
          w[k] = nk;
        }
        if (go)
          w[0] = key;
      }
      return w[N / 2];
    }
    case lod_reduce_max_suppressed: {
      T t1 = w[0], t2 = w[0];
#pragma unroll
      for (int j = 1; j < N; ++j) {
        const T v = w[j];
        if (!lt(v, t1)) { // v >= t1
          t2 = t1;
          t1 = v;
        } else if (lt(t2, v))
          t2 = v;
      }
      return t2;
    }
    case lod_reduce_min_suppressed: {
      T t1 = w[0], t2 = w[0];
#pragma unroll
      for (int j = 1; j < N; ++j) {
        const T v = w[j];
        if (!lt(t1, v)) { // v <= t1
          t2 = t1;
          t1 = v;
        } else if (lt(v, t2))
          t2 = v;
      }
      return t2;
    }
  }
  return w[0];
}

// (a + b) >> s without overflow for 8..32-bit integers; a + b otherwise
// (the dim-0 mean divides at emit for floats; 64-bit ints just sum).
template<typename T>
__device__ __forceinline__ T add_shift(T a, T b, int s)
{
  if constexpr (IsFloat<T>::value || sizeof(T) >= 8) {
    return T(a + b);
  } else {
    const T mask = T((1u << s) - 1);
    return T((a >> s) + (b >> s) + (((a & mask) + (b & mask)) >> s));
  }
}
template<>
__device__ __forceinline__ __half add_shift<__half>(__half a, __half b, int)
{
  return __float2half_rn(__half2float(a) + __half2float(b));
}

template<typename T>
__device__ __forceinline__ T fold_one(T acc, T v, int level, int method)
{
  if (method == lod_reduce_mean)
    return add_shift<T>(acc, v, level);
  if (method == lod_reduce_min)
    return lt(v, acc) ? v : acc;
  if (method == lod_reduce_max)
    return lt(acc, v) ? v : acc;
  return acc;
}

template<typename T>
__device__ __forceinline__ T emit_one(T acc, uint32_t count, int method)
{
  if constexpr (IsFloat<T>::value) {
    if (method == lod_reduce_mean) {
      if constexpr (sizeof(T) == 2)
        return __float2half_rn(__fdiv_rn(__half2float(acc), float(count)));
      else
        return T(acc / T(count));
    }
  }
  return acc;
}

} // namespace chucky
