// LZ4 chunk encoder that allocates nothing: the encoder's scratch is a
// fixed-size array in this module's device memory instead of a cudaMalloc'd
// area owned by a stream.
//
// The stream encodes chunks with launch_lz4 over scratch it allocates at
// create (codec.cu); this entry point runs the same three kernels (find,
// plan, emit) over caller-provided device input and output, with
// `g_lz4_scratch` as scratch.  The array exists once per device (it is
// allocated when the CUDA runtime loads this module into the device's
// context); its address is looked up once per device, on the first call made
// with that device current, and cached.
//
// Every call rewrites all of the scratch it later reads (per-segment
// sequences and metadata), so nothing in the array has to start at zero.
// Calls on one CUDA stream run one after another and are safe; calls whose
// kernels can overlap (different CUDA streams, different host threads)
// share the array and race.
#include "kernels_codec.hpp"
#include "plan.hpp"

#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <mutex>

namespace {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_lz4_scratch[kStaticScratchBytes];

std::mutex g_setup_mutex;
std::atomic<void*> g_scratch_ptr[kMaxDevices];

void* scratch_for_current_device()
{
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return nullptr;
  void* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (p)
    return p;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  p = g_scratch_ptr[dev].load(std::memory_order_relaxed);
  if (p)
    return p;
  if (cudaGetSymbolAddress(&p, g_lz4_scratch) != cudaSuccess || !p) {
    std::fprintf(stderr,
                 "chucky_gb300: static LZ4 scratch lookup failed on device %d: %s\n",
                 dev, cudaGetErrorString(cudaGetLastError()));
    return nullptr;
  }
  g_scratch_ptr[dev].store(p, std::memory_order_release);
  return p;
}

} // namespace

extern "C" size_t
chucky_lz4_static_scratch_bytes(void)
{
  return kStaticScratchBytes;
}

extern "C" int
chucky_lz4_encode_chunks_static(const void* d_chunks,
                                size_t chunk_bytes,
                                size_t in_stride,
                                size_t n_chunks,
                                void* d_out,
                                size_t out_stride,
                                uint64_t* d_sizes,
                                void* cuda_stream)
{
  if (!n_chunks)
    return 0;
  if (!d_chunks || !d_out || !d_sizes || !chunk_bytes ||
      chunk_bytes >= (size_t(1) << 32) || in_stride < chunk_bytes ||
      (reinterpret_cast<uintptr_t>(d_chunks) & 3) || (in_stride & 3)) {
    std::fprintf(stderr, "chucky_gb300: lz4 static encode: invalid arguments\n");
    return 1;
  }
  if (out_stride < chucky::codec_bound(CODEC_LZ4_NON_STANDARD, chunk_bytes)) {
    std::fprintf(stderr,
                 "chucky_gb300: lz4 static encode: out_stride %zu below the "
                 "bound %llu for %zu-byte chunks\n",
                 out_stride,
                 (unsigned long long)chucky::codec_bound(CODEC_LZ4_NON_STANDARD,
                                                         chunk_bytes),
                 chunk_bytes);
    return 1;
  }
  const size_t need = chucky::lz4_scratch_bytes(n_chunks, uint32_t(chunk_bytes));
  if (need > kStaticScratchBytes) {
    std::fprintf(stderr,
                 "chucky_gb300: lz4 static encode: %zu chunks of %zu bytes need "
                 "%zu bytes of scratch, above the fixed %zu\n",
                 n_chunks, chunk_bytes, need, kStaticScratchBytes);
    return 2;
  }
  void* scratch = scratch_for_current_device();
  if (!scratch)
    return 3;
  chucky::CodecBatch b{};
  b.in = static_cast<const uint8_t*>(d_chunks);
  b.in_stride = in_stride;
  b.chunk_bytes = uint32_t(chunk_bytes);
  b.n_chunks = n_chunks;
  b.out = static_cast<uint8_t*>(d_out);
  b.out_stride = out_stride;
  b.out_sizes = d_sizes;
  b.level = 1;
  const cudaError_t e =
    chucky::launch_lz4(b, scratch, static_cast<cudaStream_t>(cuda_stream));
  if (e != cudaSuccess) {
    std::fprintf(stderr, "chucky_gb300: lz4 static encode launch failed: %s\n",
                 cudaGetErrorString(e));
    return 3;
  }
  return 0;
}
