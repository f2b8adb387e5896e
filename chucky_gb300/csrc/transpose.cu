// (a) Scatter a row-major epoch into chunk-contiguous tiles.
//
// Element e of an epoch goes to ravel(e) over the lifted shape
// (c0, k0, c1, k1, ...) with the lifted strides of the level layout, exactly
// as src/gpu/transpose.cu:85-137 and src/cpu/transpose.cpp:10-105 of the
// reference.  The innermost lifted pair (count, chunk) spans one input row
// of `width` elements, so dst(e) = row_off[e / width] + col_off[e % width]:
// the two small tables replace the per-element unravel.  When the chunk
// extent of the innermost dim is a multiple of 16 bytes and that dim is
// innermost in storage, every 16-byte input vector lands in one contiguous,
// aligned run of its chunk row: one 16-byte load and one 16-byte store per
// thread, fully coalesced on both sides.
#include "kernels.hpp"

namespace chucky {

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
transpose_vec16_k(TransposeArgs a, uint64_t nvec)
{
  const uint32_t per = 16u / a.bpe;
  for (uint64_t v = blockIdx.x * uint64_t(kThreads) + threadIdx.x; v < nvec;
       v += uint64_t(gridDim.x) * kThreads) {
    const uint64_t e = v * per;
    uint64_t row, x;
    a.width.divmod(e, row, x);
    const uint64_t o = __ldg(a.row_off + row) + __ldg(a.col_off + x);
    const uint4 val = __ldg(reinterpret_cast<const uint4*>(a.src) + v);
    *reinterpret_cast<uint4*>(a.dst + o * a.bpe) = val;
  }
}

template<typename T>
__global__ void __launch_bounds__(kThreads)
transpose_scalar_k(TransposeArgs a, uint64_t first)
{
  const T* src = reinterpret_cast<const T*>(a.src);
  T* dst = reinterpret_cast<T*>(a.dst);
  for (uint64_t e = first + blockIdx.x * uint64_t(kThreads) + threadIdx.x;
       e < a.n;
       e += uint64_t(gridDim.x) * kThreads) {
    uint64_t row, x;
    a.width.divmod(e, row, x);
    dst[__ldg(a.row_off + row) + __ldg(a.col_off + x)] = src[e];
  }
}

int grid_for(uint64_t work)
{
  // persistent-style grid: a multiple of the SM count, capped by the work
  const uint64_t blocks = (work + kThreads - 1) / kThreads;
  const uint64_t cap = uint64_t(device_sm_count()) * 8;
  return int(blocks < cap ? (blocks ? blocks : 1) : cap);
}

} // namespace

cudaError_t launch_transpose(const TransposeArgs& a, cudaStream_t st)
{
  if (a.n == 0)
    return cudaSuccess;
  uint64_t first = 0;
  if (a.vector_ok) {
    const uint64_t per = 16u / a.bpe;
    const uint64_t nvec = a.n / per;
    if (nvec) {
      transpose_vec16_k<<<grid_for(nvec), kThreads, 0, st>>>(a, nvec);
      note_launches(1);
      first = nvec * per;
    }
  }
  if (first < a.n) {
    const int g = grid_for(a.n - first);
    note_launches(1);
    switch (a.bpe) {
      case 1:
        transpose_scalar_k<uint8_t><<<g, kThreads, 0, st>>>(a, first);
        break;
      case 2:
        transpose_scalar_k<uint16_t><<<g, kThreads, 0, st>>>(a, first);
        break;
      case 4:
        transpose_scalar_k<uint32_t><<<g, kThreads, 0, st>>>(a, first);
        break;
      case 8:
        transpose_scalar_k<uint64_t><<<g, kThreads, 0, st>>>(a, first);
        break;
      default:
        return cudaErrorInvalidValue;
    }
  }
  return cudaGetLastError();
}

} // namespace chucky
