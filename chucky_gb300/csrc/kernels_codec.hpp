// Batched chunk encoders (LZ4 block, zstd frame).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace chucky {

// Number of kernels this library has launched (process-wide).
void note_launches(unsigned n);

// Streaming multiprocessors of the current device.
int device_sm_count();

// Raw LZ4 blocks back to chunk bytes (a warp per block, bounds-checked):
// block i is in_size[i] bytes at in + in_off[i] and decodes to chunk_bytes
// bytes at out + i * out_stride; status[i] 0 when it did exactly that.
cudaError_t launch_lz4_decode(const uint8_t* in,
                              const uint64_t* in_off,
                              const uint64_t* in_size,
                              uint64_t n_chunks,
                              uint8_t* out,
                              uint64_t out_stride,
                              uint64_t chunk_bytes,
                              uint32_t* status,
                              cudaStream_t st);

// Addresses of one chunk of a batch gathered from several streams.
struct ChunkRef
{
  const uint8_t* in; // chunk_bytes of input (4-byte aligned)
  uint8_t* out;      // compressed slot (>= the codec bound)
  uint64_t* size;    // compressed size (written)
};

// zstd frames back to chunk bytes (a CTA per frame, bounds-checked): frame
// i is in_size[i] bytes at in + in_off[i] and decodes to chunk_bytes bytes
// at out + i * out_stride; status[i] 0 when it did exactly that.
cudaError_t launch_zstd_decode(const uint8_t* in,
                               const uint64_t* in_off,
                               const uint64_t* in_size,
                               uint64_t n_chunks,
                               uint8_t* out,
                               uint64_t out_stride,
                               uint64_t chunk_bytes,
                               uint32_t* status,
                               cudaStream_t st);

struct CodecBatch
{
  const uint8_t* in;    // first chunk (4-byte aligned)
  uint64_t in_stride;   // bytes between chunks
  uint32_t chunk_bytes; // codec input per chunk
  uint64_t n_chunks;     // chunks to encode (entries of chunk_ids if set)
  uint8_t* out;         // compressed slots
  uint64_t out_stride;  // bytes between slots (>= bound)
  uint64_t* out_sizes;  // [n_chunks] compressed sizes (written)
  uint32_t segs_per_chunk;
  int level;
  // parse parameters (0: the level's defaults), e.g. chosen by the
  // autotuner: search strength (positions probed per lane step grow by one
  // for every 2^strength literals since the last match) and the shortest
  // match taken (LZ4 >= 4; zstd levels without the wide window)
  int strength;
  int min_match;
  const uint32_t* chunk_ids; // optional: encode only these chunk slots
  // Otherwise, optionally, the slots as runs of consecutive slots (a batch
  // whose levels are not all active): entry id_base + i lies in run r when
  // run_first[r] <= id_base + i < run_first[r + 1] and is slot
  // run_slot[r] + (id_base + i - run_first[r]).  Passed by value, so no
  // table has to reach the device first.
  static constexpr int kMaxRuns = 16;
  uint32_t n_runs;
  uint64_t id_base;
  uint32_t run_first[kMaxRuns + 1];
  uint32_t run_slot[kMaxRuns];

  // Optional, overriding all of the above addressing: chunk i of the batch
  // is refs[i] (a device array), so one launch can encode the chunks of
  // several streams' pools (all of chunk_bytes bytes).
  const ChunkRef* refs;

  __host__ __device__ const uint8_t* in_at(uint64_t i) const
  {
    return refs ? refs[i].in : in + id(i) * in_stride;
  }
  __host__ __device__ uint8_t* out_at(uint64_t i) const
  {
    return refs ? refs[i].out : out + id(i) * out_stride;
  }
  __host__ __device__ uint64_t* size_at(uint64_t i) const
  {
    return refs ? refs[i].size : out_sizes + id(i);
  }

  // slot of the i-th chunk of the batch
  __host__ __device__ uint64_t id(uint64_t i) const
  {
    if (chunk_ids)
      return chunk_ids[i];
    if (!n_runs)
      return i;
    const uint64_t g = id_base + i;
    uint32_t r = 0;
    while (r + 1 < n_runs && g >= run_first[r + 1])
      ++r;
    return run_slot[r] + (g - run_first[r]);
  }
};

// The runs of consecutive chunk slots of a batch (see CodecBatch).
struct ChunkRuns
{
  uint32_t n;
  uint32_t first[CodecBatch::kMaxRuns + 1];
  uint32_t slot[CodecBatch::kMaxRuns];
};

// Scratch of one launch set.  The level selects the parse: LZ4 levels >= 2
// and zstd levels >= 3 also search the wide window (earlier regions of the
// chunk) and need room for its region tables.
size_t lz4_scratch_bytes(uint64_t n_chunks, uint32_t chunk_bytes, int level);
cudaError_t launch_lz4(CodecBatch b, void* scratch, cudaStream_t st);

size_t zstd_scratch_bytes(uint64_t n_chunks, uint32_t chunk_bytes, int level);
cudaError_t launch_zstd(CodecBatch b, void* scratch, cudaStream_t st);

} // namespace chucky
