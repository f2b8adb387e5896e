// (b) LOD pyramid, general path: Morton-ordered level buffers.
//
// Works for any number of LOD dims and levels.  Per epoch:
//   gather  : values[b*n0 + m] = linear[fixed[b] + lut[m]]
//             (src/cpu/lod.cpp:241-267, src/gpu/lod.cu:224-304)
//   reduce  : parent i of level l+1 = reduce(child window
//             [ends[i-1], ends[i]) of level l), sequential in window order
//             (src/cpu/lod.cpp:55-127, 269-296; src/gpu/lod.cu:414-528)
//   fold    : dim-0 accumulators of levels >= 1
//             (src/cpu/lod.cpp:366-414; src/gpu/lod.cu:904-941)
//   emit    : accumulators -> level values (src/cpu/lod.cpp:416-438)
//   scatter : level values -> chunk slot via per-level LUTs
//             (src/cpu/lod.cpp:298-359, src/gpu/lod.cu:347-364)
// Arithmetic per dtype matches the reference bit for bit: widened sums for
// mean (u8/u16 -> u32, u32 -> u64, i8/i16 -> i32, i32 -> i64, f16 -> f32),
// insertion-sort median (upper median), second-extreme with >= / <= ties.
#include "kernels.hpp"
#include "lod_ops.cuh"

namespace chucky {

namespace lod {

constexpr int kThreads = 256;

template<typename T>
__global__ void __launch_bounds__(kThreads)
gather_k(const T* __restrict__ linear,
         T* __restrict__ values,
         const uint32_t* __restrict__ lut,
         const uint64_t* __restrict__ fixed,
         uint64_t n0,
         uint64_t total)
{
  for (uint64_t g = blockIdx.x * uint64_t(kThreads) + threadIdx.x; g < total;
       g += uint64_t(gridDim.x) * kThreads) {
    const uint64_t b = g / n0, m = g - b * n0;
    values[g] = linear[fixed[b] + lut[m]];
  }
}

template<typename T>
__global__ void __launch_bounds__(kThreads)
reduce_k(T* __restrict__ values,
         const uint64_t* __restrict__ ends,
         uint64_t src_beg,
         uint64_t dst_beg,
         uint64_t src_n,
         uint64_t dst_n,
         uint64_t total,
         int method)
{
  for (uint64_t g = blockIdx.x * uint64_t(kThreads) + threadIdx.x; g < total;
       g += uint64_t(gridDim.x) * kThreads) {
    const uint64_t b = g / dst_n, i = g - b * dst_n;
    const uint64_t lo = i ? ends[i - 1] : 0, hi = ends[i];
    values[dst_beg + b * dst_n + i] =
      reduce_window<T>(values + src_beg + b * src_n + lo, hi - lo, method);
  }
}

template<typename T>
__global__ void __launch_bounds__(kThreads)
fold_k(T* __restrict__ accum,
       const T* __restrict__ x,
       uint64_t n,
       uint32_t count,
       int level,
       int method)
{
  for (uint64_t g = blockIdx.x * uint64_t(kThreads) + threadIdx.x; g < n;
       g += uint64_t(gridDim.x) * kThreads)
    accum[g] = count == 0 ? x[g] : fold_one<T>(accum[g], x[g], level, method);
}

template<typename T>
__global__ void __launch_bounds__(kThreads)
emit_k(T* __restrict__ dst,
       const T* __restrict__ accum,
       uint64_t n,
       uint32_t count,
       int method)
{
  for (uint64_t g = blockIdx.x * uint64_t(kThreads) + threadIdx.x; g < n;
       g += uint64_t(gridDim.x) * kThreads)
    dst[g] = emit_one<T>(accum[g], count, method);
}

template<typename T>
__global__ void __launch_bounds__(kThreads)
to_chunks_k(const T* __restrict__ values,
            T* __restrict__ slot,
            const uint32_t* __restrict__ lut,
            const uint64_t* __restrict__ fixed,
            uint64_t n,
            uint64_t total)
{
  for (uint64_t g = blockIdx.x * uint64_t(kThreads) + threadIdx.x; g < total;
       g += uint64_t(gridDim.x) * kThreads) {
    const uint64_t b = g / n, i = g - b * n;
    slot[fixed[b] + lut[i]] = values[g];
  }
}

inline int grid_for(uint64_t work)
{
  const uint64_t blocks = (work + kThreads - 1) / kThreads;
  const uint64_t cap = uint64_t(device_sm_count()) * 16;
  return int(blocks < cap ? (blocks ? blocks : 1) : cap);
}

} // namespace lod

using namespace lod;

cudaError_t launch_lod_gather(const LodMortonArgs& a,
                              const uint8_t* linear,
                              uint8_t* values,
                              cudaStream_t st)
{
  const uint64_t n0 = a.lod_nelem[0], total = a.fixed_count * n0;
  CHUCKY_DISPATCH_DTYPE(a.dtype,
                        (gather_k<T><<<grid_for(total), kThreads, 0, st>>>(
                          reinterpret_cast<const T*>(linear),
                          reinterpret_cast<T*>(values),
                          a.d_gather_lut,
                          a.d_gather_fixed,
                          n0,
                          total)));
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_lod_reduce(const LodMortonArgs& a,
                              uint8_t* values,
                              cudaStream_t st)
{
  for (int l = 0; l + 1 < a.nlod; ++l) {
    const uint64_t total = a.fixed_count * a.lod_nelem[l + 1];
    CHUCKY_DISPATCH_DTYPE(a.dtype,
                          (reduce_k<T><<<grid_for(total), kThreads, 0, st>>>(
                            reinterpret_cast<T*>(values),
                            a.d_ends + a.ends_beg[l + 1],
                            a.level_beg[l],
                            a.level_beg[l + 1],
                            a.lod_nelem[l],
                            a.lod_nelem[l + 1],
                            total,
                            a.reduce_method)));
    note_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_lod_fold(const LodMortonArgs& a,
                            int level,
                            uint32_t count,
                            const uint8_t* values,
                            uint8_t* accum,
                            cudaStream_t st)
{
  const uint64_t n = a.fixed_count * a.lod_nelem[level];
  CHUCKY_DISPATCH_DTYPE(
    a.dtype,
    (fold_k<T><<<grid_for(n), kThreads, 0, st>>>(
      reinterpret_cast<T*>(accum) + a.accum_beg[level],
      reinterpret_cast<const T*>(values) + a.level_beg[level],
      n,
      count,
      level,
      a.append_method)));
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_lod_emit(const LodMortonArgs& a,
                            int level,
                            uint32_t count,
                            const uint8_t* accum,
                            uint8_t* values,
                            cudaStream_t st)
{
  const uint64_t n = a.fixed_count * a.lod_nelem[level];
  CHUCKY_DISPATCH_DTYPE(
    a.dtype,
    (emit_k<T><<<grid_for(n), kThreads, 0, st>>>(
      reinterpret_cast<T*>(values) + a.level_beg[level],
      reinterpret_cast<const T*>(accum) + a.accum_beg[level],
      n,
      count,
      a.append_method)));
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_lod_to_chunks(const LodMortonArgs& a,
                                 int level,
                                 const uint8_t* values,
                                 uint8_t* slot,
                                 cudaStream_t st)
{
  const uint64_t n = a.lod_nelem[level], total = a.fixed_count * n;
  CHUCKY_DISPATCH_DTYPE(
    a.dtype,
    (to_chunks_k<T><<<grid_for(total), kThreads, 0, st>>>(
      reinterpret_cast<const T*>(values) + a.level_beg[level],
      reinterpret_cast<T*>(slot),
      a.d_chunk_lut[level],
      a.d_chunk_fixed[level],
      n,
      total)));
  note_launches(1);
  return cudaGetLastError();
}

} // namespace chucky
