// LZ4 block decoder: raw LZ4 blocks (the CODEC_LZ4_NON_STANDARD chunk
// format) back to chunk bytes on the device, for on-device verification and
// readback of stores.  The reference decodes its chunks on the host with
// LZ4_decompress_safe and the known chunk size (src/cpu/compress.c:85,
// tests/test_compress_cpu.c:75-190); this is the same contract on the GPU.
//
// A warp per block.  Every lane parses the same token stream (the byte
// loads broadcast within the warp), so the parse state needs no shuffles;
// literals are copied with the lanes side by side, and a match of offset d
// writes out[op + j] = out[op - d + j mod d] for j in [0, length), which
// reads only bytes already final before op, so any offset, overlapping
// ones included, is one pass.  Every read is checked against the block's
// size and every write against the chunk size; a malformed block sets its
// status and stops, nothing is read or written out of bounds.
#include "chucky_gb300.h"
#include "kernels_codec.hpp"
#include "launch.cuh"

#include <cuda_runtime.h>

namespace chucky {

namespace {

constexpr int kDecodeWarps = 4;

enum : uint32_t
{
  kDecodeOk = 0,
  kDecodeTruncated = 1, // the block ends inside a token, length or literals
  kDecodeBadOffset = 2, // a match offset of 0 or before the chunk start
  kDecodeOverrun = 3,   // the output would exceed the chunk size
  kDecodeShort = 4,     // the block ends before the chunk is complete
};

__global__ void __launch_bounds__(32 * kDecodeWarps)
lz4_decode_k(const uint8_t* in,
             const uint64_t* in_off,
             const uint64_t* in_size,
             uint64_t n_chunks,
             uint8_t* out,
             uint64_t out_stride,
             uint64_t chunk_bytes,
             uint32_t* status)
{
  const int lane = threadIdx.x & 31;
  const uint64_t c = uint64_t(blockIdx.x) * kDecodeWarps + (threadIdx.x >> 5);
  if (c >= n_chunks)
    return; // the whole warp
  const uint8_t* src = in + in_off[c];
  const uint64_t n = in_size[c];
  uint8_t* dst = out + c * out_stride;
  uint64_t ip = 0, op = 0;
  uint32_t st = kDecodeOk;
  while (true) {
    if (ip >= n) {
      st = kDecodeTruncated;
      break;
    }
    const uint32_t token = src[ip++];
    uint64_t lit = token >> 4;
    if (lit == 15) {
      uint32_t b = 255;
      while (b == 255) {
        if (ip >= n) {
          st = kDecodeTruncated;
          break;
        }
        b = src[ip++];
        lit += b;
      }
      if (st)
        break;
    }
    if (lit > n - ip) {
      st = kDecodeTruncated;
      break;
    }
    if (lit > chunk_bytes - op) {
      st = kDecodeOverrun;
      break;
    }
    for (uint64_t j = lane; j < lit; j += 32)
      dst[op + j] = src[ip + j];
    ip += lit;
    op += lit;
    if (ip == n) // the last sequence has literals only
      break;
    if (n - ip < 2) {
      st = kDecodeTruncated;
      break;
    }
    const uint64_t off = uint64_t(src[ip]) | uint64_t(src[ip + 1]) << 8;
    ip += 2;
    if (off == 0 || off > op) {
      st = kDecodeBadOffset;
      break;
    }
    uint64_t ml = (token & 15) + 4;
    if ((token & 15) == 15) {
      uint32_t b = 255;
      while (b == 255) {
        if (ip >= n) {
          st = kDecodeTruncated;
          break;
        }
        b = src[ip++];
        ml += b;
      }
      if (st)
        break;
    }
    if (ml > chunk_bytes - op) {
      st = kDecodeOverrun;
      break;
    }
    // the literals just written by other lanes are read below
    __syncwarp();
    const uint8_t* m = dst + op - off;
    for (uint64_t j = lane; j < ml; j += 32)
      dst[op + j] = m[j < off ? j : j % off];
    __syncwarp();
    op += ml;
  }
  if (st == kDecodeOk && op != chunk_bytes)
    st = kDecodeShort;
  if (lane == 0)
    status[c] = st;
}

} // namespace

cudaError_t launch_lz4_decode(const uint8_t* in,
                              const uint64_t* in_off,
                              const uint64_t* in_size,
                              uint64_t n_chunks,
                              uint8_t* out,
                              uint64_t out_stride,
                              uint64_t chunk_bytes,
                              uint32_t* status,
                              cudaStream_t st)
{
  const uint64_t grid = (n_chunks + kDecodeWarps - 1) / kDecodeWarps;
  CHUCKY_LAUNCH(lz4_decode_k, unsigned(grid), 32 * kDecodeWarps, 0, st, in, in_off,
                in_size, n_chunks, out, out_stride, chunk_bytes, status);
  note_launches(1);
  return cudaGetLastError();
}

} // namespace chucky

extern "C" int chucky_lz4_decode_chunks(const void* d_in,
                                        const uint64_t* d_in_offsets,
                                        const uint64_t* d_in_sizes,
                                        size_t n_chunks,
                                        void* d_out,
                                        size_t out_stride,
                                        size_t chunk_bytes,
                                        uint32_t* d_status,
                                        void* cuda_stream)
{
  if (n_chunks == 0)
    return 0;
  if (!d_in || !d_in_offsets || !d_in_sizes || !d_out || !d_status ||
      out_stride < chunk_bytes)
    return 1;
  const cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  if (n_chunks > (uint64_t(1) << 32))
    return 1;
  return chucky::launch_lz4_decode(static_cast<const uint8_t*>(d_in), d_in_offsets,
                                   d_in_sizes, n_chunks, static_cast<uint8_t*>(d_out),
                                   out_stride, chunk_bytes, d_status, st) == cudaSuccess
           ? 0
           : 3;
}
