// (c) Batched chunk encoders behind the stream: dispatch on the codec id.
// Input: every chunk of the batch in the chunk pool (chunk_bytes each at the
// pool's chunk stride); output: compressed slots + sizes on the device.
#include "kernels_codec.hpp"
#include "stream_internal.hpp"

#include <algorithm>
#include <cstdio>

namespace chucky {

int Stream::codec_init()
{
  const uint64_t n = uint64_t(P.K) * P.total_chunks;
  if (cfg.codec.id == CODEC_NONE)
    return 0;
  if (cfg.codec.id != CODEC_LZ4_NON_STANDARD && cfg.codec.id != CODEC_ZSTD)
    return 1;
  tune_key = TuneKey{};
  tune_key.codec = cfg.codec.id;
  tune_key.level = cfg.codec.level;
  tune_key.dtype = int(cfg.dtype);
  tune_key.rank = cfg.rank;
  for (int d = 0; d < cfg.rank && d < 16; ++d)
    tune_key.chunk[d] = cfg.dimensions[d].chunk_size;
  // The encoders' scratch grows with their input; batches larger than
  // kWaveBytes are encoded in waves that reuse one scratch area.
  constexpr uint64_t kWaveBytes = 256ull << 20;
  wave_chunks = std::max<uint64_t>(1, kWaveBytes / std::max<uint64_t>(1, P.chunk_bytes));
  if (wave_chunks > n)
    wave_chunks = n;
  const size_t bytes = cfg.codec.id == CODEC_ZSTD
                         ? zstd_scratch_bytes(wave_chunks, uint32_t(P.chunk_bytes), cfg.codec.level)
                         : lz4_scratch_bytes(wave_chunks, uint32_t(P.chunk_bytes), cfg.codec.level);
  if (P.chunk_bytes >= (uint64_t(1) << 32))
    return 1;
  for (int i = 0; i < 2; ++i)
    if (cudaHostAlloc(&h_chunk_ids[i], n * 4, cudaHostAllocMapped) != cudaSuccess ||
        cudaMalloc(&d_chunk_ids[i], n * 4) != cudaSuccess)
      return 1;
  if (engine) { // the engine owns the scratch
    for (int i = 0; i < 2; ++i)
      if (cudaEventCreateWithFlags(&ev_engine_done[i], cudaEventDisableTiming) !=
          cudaSuccess)
        return 1;
    return 0;
  }
  for (int i = 0; i < 2; ++i)
    if (cudaMalloc(&codec_state[i], bytes) != cudaSuccess)
      return 1;
  return 0;
}

int Stream::codec_compress(const uint8_t* pool,
                           uint64_t nchunks,
                           const uint32_t* d_ids,
                           const ChunkRuns* runs,
                           uint8_t* out,
                           uint64_t* sizes,
                           void* scratch,
                           cudaStream_t st)
{
  cudaError_t e = cudaSuccess;
  for (uint64_t first = 0; first < nchunks && e == cudaSuccess;
       first += wave_chunks) {
    CodecBatch b{};
    const uint64_t n = std::min<uint64_t>(wave_chunks, nchunks - first);
    b.in_stride = layout.chunk_stride * P.bpe;
    b.chunk_bytes = uint32_t(P.chunk_bytes);
    b.n_chunks = n;
    b.out_stride = comp_stride;
    b.level = cfg.codec.level;
    b.strength = tune.strength;
    b.min_match = tune.min_match;
    if (d_ids) { // chunk slots listed explicitly
      b.in = pool;
      b.out = out;
      b.out_sizes = sizes;
      b.chunk_ids = d_ids + first;
    } else if (runs) { // chunk slots as runs
      b.in = pool;
      b.out = out;
      b.out_sizes = sizes;
      b.n_runs = runs->n;
      b.id_base = first;
      for (uint32_t r = 0; r <= runs->n; ++r)
        b.run_first[r] = runs->first[r];
      for (uint32_t r = 0; r < runs->n; ++r)
        b.run_slot[r] = runs->slot[r];
    } else { // slots first .. first + n - 1
      b.in = pool + first * b.in_stride;
      b.out = out + first * comp_stride;
      b.out_sizes = sizes + first;
    }
    e = cfg.codec.id == CODEC_ZSTD ? launch_zstd(b, scratch, st)
                                   : launch_lz4(b, scratch, st);
  }
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
  for (int i = 0; i < 2; ++i) {
    cudaFree(codec_state[i]);
    codec_state[i] = nullptr;
    if (ev_engine_done[i])
      cudaEventDestroy(ev_engine_done[i]);
    ev_engine_done[i] = nullptr;
  }
  for (int i = 0; i < 2; ++i) {
    cudaFreeHost(h_chunk_ids[i]);
    cudaFree(d_chunk_ids[i]);
    h_chunk_ids[i] = nullptr;
    d_chunk_ids[i] = nullptr;
  }
}

} // namespace chucky

// ---- batched chunk encoding as a library call -------------------------------
// (the batch-level counterpart of the reference's codec_compress,
// src/gpu/compress.cu:284-369, which calls nvcomp)

extern "C" size_t
chucky_encode_bound(int codec_id, size_t chunk_bytes)
{
  if (codec_id != CODEC_LZ4_NON_STANDARD && codec_id != CODEC_ZSTD)
    return 0;
  return size_t(chucky::codec_bound(codec_id, chunk_bytes));
}

extern "C" size_t
chucky_encode_scratch_bytes(int codec_id, int level, size_t chunk_bytes, size_t n_chunks)
{
  if (!chunk_bytes || chunk_bytes >= (size_t(1) << 32))
    return 0;
  if (codec_id == CODEC_ZSTD)
    return chucky::zstd_scratch_bytes(n_chunks, uint32_t(chunk_bytes), level);
  if (codec_id == CODEC_LZ4_NON_STANDARD)
    return chucky::lz4_scratch_bytes(n_chunks, uint32_t(chunk_bytes), level);
  return 0;
}

extern "C" int
chucky_encode_chunks(int codec_id,
                     int level,
                     const void* d_chunks,
                     size_t chunk_bytes,
                     size_t in_stride,
                     size_t n_chunks,
                     void* d_out,
                     size_t out_stride,
                     uint64_t* d_sizes,
                     void* d_scratch,
                     size_t scratch_bytes,
                     void* cuda_stream)
{
  if (!n_chunks)
    return 0;
  if ((codec_id != CODEC_LZ4_NON_STANDARD && codec_id != CODEC_ZSTD) || !d_chunks ||
      !d_out || !d_sizes || !d_scratch || !chunk_bytes ||
      chunk_bytes >= (size_t(1) << 32) || in_stride < chunk_bytes ||
      (reinterpret_cast<uintptr_t>(d_chunks) & 3) || (in_stride & 3) ||
      out_stride < chucky::codec_bound(codec_id, chunk_bytes) ||
      scratch_bytes < chucky_encode_scratch_bytes(codec_id, level, chunk_bytes, n_chunks)) {
    std::fprintf(stderr, "chucky_gb300: chucky_encode_chunks: invalid arguments\n");
    return 1;
  }
  chucky::CodecBatch b{};
  b.in = static_cast<const uint8_t*>(d_chunks);
  b.in_stride = in_stride;
  b.chunk_bytes = uint32_t(chunk_bytes);
  b.n_chunks = n_chunks;
  b.out = static_cast<uint8_t*>(d_out);
  b.out_stride = out_stride;
  b.out_sizes = d_sizes;
  b.level = level;
  const cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  const cudaError_t e = codec_id == CODEC_ZSTD ? chucky::launch_zstd(b, d_scratch, st)
                                               : chucky::launch_lz4(b, d_scratch, st);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "chucky_gb300: chucky_encode_chunks: %s\n",
                 cudaGetErrorString(e));
    return 3;
  }
  return 0;
}
