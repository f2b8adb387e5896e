// (c) Batched chunk encoders behind the stream: dispatch on the codec id.
// Input: every chunk of the batch in the chunk pool (chunk_bytes each at the
// pool's chunk stride); output: compressed slots + sizes on the device.
#include "kernels_codec.hpp"
#include "stream_internal.hpp"

#include <cstdio>

namespace chucky {

int Stream::codec_init()
{
  const uint64_t n = uint64_t(P.K) * P.total_chunks;
  size_t bytes = 0;
  switch (cfg.codec.id) {
    case CODEC_NONE:
      return 0;
    case CODEC_LZ4_NON_STANDARD:
      bytes = lz4_scratch_bytes(n, uint32_t(P.chunk_bytes));
      break;
    case CODEC_ZSTD:
      bytes = zstd_scratch_bytes(n, uint32_t(P.chunk_bytes));
      break;
    default:
      return 1;
  }
  if (P.chunk_bytes >= (uint64_t(1) << 32))
    return 1;
  for (int i = 0; i < 2; ++i)
    if (cudaMallocHost(&h_chunk_ids[i], n * 4) != cudaSuccess ||
        cudaMalloc(&d_chunk_ids[i], n * 4) != cudaSuccess)
      return 1;
  return cudaMalloc(&codec_state, bytes) == cudaSuccess ? 0 : 1;
}

int Stream::codec_compress(uint64_t nchunks,
                           const uint32_t* d_ids,
                           uint8_t* out,
                           uint64_t* sizes)
{
  CodecBatch b{};
  b.in = d_pool;
  b.in_stride = layout.chunk_stride * P.bpe;
  b.chunk_bytes = uint32_t(P.chunk_bytes);
  b.n_chunks = nchunks;
  b.out = out;
  b.out_stride = comp_stride;
  b.out_sizes = sizes;
  b.level = cfg.codec.level;
  b.chunk_ids = d_ids;
  cudaError_t e = cudaErrorInvalidValue;
  if (cfg.codec.id == CODEC_LZ4_NON_STANDARD)
    e = launch_lz4(b, codec_state, s_comp);
  else if (cfg.codec.id == CODEC_ZSTD)
    e = launch_zstd(b, codec_state, s_comp);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "chucky_gb300: %s encoder launch failed: %s\n",
                 cfg.codec.id == CODEC_ZSTD ? "zstd" : "lz4",
                 cudaGetErrorString(e));
    return 1;
  }
  return 0;
}

void Stream::codec_release()
{
  cudaFree(codec_state);
  codec_state = nullptr;
  for (int i = 0; i < 2; ++i) {
    cudaFreeHost(h_chunk_ids[i]);
    cudaFree(d_chunk_ids[i]);
    h_chunk_ids[i] = nullptr;
    d_chunk_ids[i] = nullptr;
  }
}

} // namespace chucky
