// Shared device helpers for the sm_103a kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace chucky {

// 64-bit division by a runtime constant: q = n / d via one 128-bit high
// multiply and a single correction step (m = floor((2^64-1)/d) makes the
// estimate low by at most one).
struct FastDiv
{
  uint64_t d = 1;
  uint64_t m = 0; // 0 encodes d == 1

  FastDiv() = default;
  explicit FastDiv(uint64_t div)
    : d(div)
    , m(div > 1 ? ~uint64_t(0) / div : 0)
  {
  }

  __device__ __forceinline__ uint64_t div(uint64_t n) const
  {
    if (m == 0)
      return n;
    uint64_t q = __umul64hi(n, m);
    uint64_t r = n - q * d;
    if (r >= d)
      ++q;
    return q;
  }
  __device__ __forceinline__ void divmod(uint64_t n,
                                         uint64_t& q,
                                         uint64_t& r) const
  {
    if (m == 0) {
      q = n;
      r = 0;
      return;
    }
    q = __umul64hi(n, m);
    r = n - q * d;
    if (r >= d) {
      ++q;
      r -= d;
    }
  }
};

template<typename T>
struct WideAcc
{
  using type = T;
};
template<>
struct WideAcc<uint8_t>
{
  using type = uint32_t;
};
template<>
struct WideAcc<uint16_t>
{
  using type = uint32_t;
};
template<>
struct WideAcc<uint32_t>
{
  using type = uint64_t;
};
template<>
struct WideAcc<int8_t>
{
  using type = int32_t;
};
template<>
struct WideAcc<int16_t>
{
  using type = int32_t;
};
template<>
struct WideAcc<int32_t>
{
  using type = int64_t;
};
template<>
struct WideAcc<__half>
{
  using type = float;
};

template<typename T>
struct IsFloat
{
  static constexpr bool value = false;
};
template<>
struct IsFloat<__half>
{
  static constexpr bool value = true;
};
template<>
struct IsFloat<float>
{
  static constexpr bool value = true;
};
template<>
struct IsFloat<double>
{
  static constexpr bool value = true;
};

} // namespace chucky

// Dispatch a templated call on the dtype enum (element type T).
#define CHUCKY_DISPATCH_DTYPE(dt, CALL)                                        \
  switch (dt) {                                                                \
    case dtype_u8: {                                                           \
      using T = uint8_t;                                                       \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_u16: {                                                          \
      using T = uint16_t;                                                      \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_u32: {                                                          \
      using T = uint32_t;                                                      \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_u64: {                                                          \
      using T = uint64_t;                                                      \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_i8: {                                                           \
      using T = int8_t;                                                        \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_i16: {                                                          \
      using T = int16_t;                                                       \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_i32: {                                                          \
      using T = int32_t;                                                       \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_i64: {                                                          \
      using T = int64_t;                                                       \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_f16: {                                                          \
      using T = __half;                                                        \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_f32: {                                                          \
      using T = float;                                                         \
      CALL;                                                                    \
    } break;                                                                   \
    case dtype_f64: {                                                          \
      using T = double;                                                        \
      CALL;                                                                    \
    } break;                                                                   \
    default:                                                                   \
      return cudaErrorInvalidValue;                                            \
  }
