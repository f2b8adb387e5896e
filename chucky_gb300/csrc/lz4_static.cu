// LZ4 chunk encoder that allocates nothing: the encoder's scratch is a
// fixed-size array in this module's device memory instead of a cudaMalloc'd
// area owned by a stream.
//
// The stream encodes chunks with launch_lz4 over scratch it allocates at
// create (codec.cu); this entry point runs the same three kernels (find,
// plan, emit) over caller-provided device input and output, with
// `g_lz4_scratch` as scratch.  The array exists once per CUDA context (it is
// allocated when the CUDA runtime loads this module into the context, and
// the primary context of each device is the usual one); its address is looked
// up with cudaGetSymbolAddress on the first call made in a context and cached
// together with that context's ID (cuCtxGetId: unique for the life of the
// process, never reused).  A call made in another context -- another device,
// a context a driver-API caller created and made current, or the new primary
// context after cudaDeviceReset -- looks the address up again, so a stale
// address from a destroyed context is never used.
//
// Every call rewrites all of the scratch it later reads (per-segment
// sequences and metadata), so nothing in the array has to start at zero.
// Calls on one CUDA stream run one after another and are safe; calls whose
// kernels can overlap (different CUDA streams, different host threads)
// share the array and race.
#include "kernels_codec.hpp"
#include "plan.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;
constexpr int kMaxCachedContexts = 64;

__device__ __align__(256) unsigned char g_lz4_scratch[kStaticScratchBytes];

// cuCtxGetCurrent and cuCtxGetId, fetched through the runtime so that the
// library does not link libcuda itself (CUresult is an int-sized enum,
// CUcontext a pointer).
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);

struct CachedScratch
{
  unsigned long long ctx_id;
  void* ptr;
};

std::mutex g_setup_mutex;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_driver_looked_up = false;
CachedScratch g_cache[kMaxCachedContexts];
int g_cache_used = 0;

void* driver_entry(const char* name)
{
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion(name, &fn, 12000, cudaEnableDefault, &q) !=
        cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError(); // clear a failed lookup
    return nullptr;
  }
  return fn;
}

// The ID of the calling thread's current context, or 0 when there is none
// or the driver cannot tell (IDs start at 1).
unsigned long long current_context_id()
{
  if (!g_driver_looked_up) {
    g_driver_looked_up = true;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(driver_entry("cuCtxGetCurrent"));
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(driver_entry("cuCtxGetId"));
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!g_ctx_get_current || !g_ctx_get_id || g_ctx_get_current(&ctx) != 0 || !ctx ||
      g_ctx_get_id(ctx, &id) != 0)
    return 0;
  return id;
}

void* scratch_for_current_context()
{
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return nullptr;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  unsigned long long id = current_context_id();
  for (int i = 0; id && i < g_cache_used; ++i)
    if (g_cache[i].ctx_id == id)
      return g_cache[i].ptr;
  // also makes the device's primary context current when the thread had no
  // context yet
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_lz4_scratch);
  if (e != cudaSuccess || !p) {
    std::fprintf(stderr,
                 "chucky_gb300: static LZ4 scratch lookup failed on device %d: %s\n",
                 dev, cudaGetErrorString(e));
    return nullptr;
  }
  if (!id)
    id = current_context_id();
  if (!id) {
    std::fprintf(stderr,
                 "chucky_gb300: static LZ4 scratch: the current CUDA context of "
                 "device %d has no ID\n",
                 dev);
    return nullptr;
  }
  // the table keeps the most recent contexts (an evicted one that comes
  // back is looked up again)
  if (g_cache_used == kMaxCachedContexts) {
    for (int i = 1; i < kMaxCachedContexts; ++i)
      g_cache[i - 1] = g_cache[i];
    --g_cache_used;
  }
  g_cache[g_cache_used++] = CachedScratch{ id, p };
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
  const size_t need = chucky::lz4_scratch_bytes(n_chunks, uint32_t(chunk_bytes), 1);
  if (need > kStaticScratchBytes) {
    std::fprintf(stderr,
                 "chucky_gb300: lz4 static encode: %zu chunks of %zu bytes need "
                 "%zu bytes of scratch, above the fixed %zu\n",
                 n_chunks, chunk_bytes, need, kStaticScratchBytes);
    return 2;
  }
  void* scratch = scratch_for_current_context();
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
