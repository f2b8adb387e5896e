/* Extensions of this library beyond the reference's C API.
 *
 * None of these entry points has a counterpart in the reference; they exist
 * for callers that run many arrays through one stream object (serving) and
 * for benchmarking. */
#pragma once

#include "stream.gpu.h"
#include "writer.h"

#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  /* Start a new array on a stream that has been flushed (or never
   * appended to), keeping every device allocation: cursor, shard state and
   * dim-0 accumulators return to their initial state.  `sink` replaces the
   * stream's sink when not NULL.  Returns 0 on success, non-zero when the
   * stream still has unflushed data. */
  int tile_stream_gpu_restart(struct tile_stream_gpu* s,
                              struct shard_sink* sink);

  /* Append device memory in stream order with the caller's CUDA stream
   * `cuda_stream` (a cudaStream_t, not NULL): the copies out of `data` wait
   * for the work queued on `cuda_stream` so far (so a kernel of the caller
   * may still be producing the frame), and work the caller queues on
   * `cuda_stream` afterwards waits for those copies (so the caller may
   * reuse its buffer in stream order).  The host does not wait for either.
   * Otherwise as writer_append (result codes, `rest`, bounded capacity).
   * `data` must be device or managed memory; host memory is rejected with
   * writer_error_fail.  The reference has no counterpart; its devlog lists
   * this hand-off as a TODO (docs/devlog.md:9).  Plain writer_append
   * accepts device pointers too, but waits for its copies before it
   * returns. */
  struct writer_result tile_stream_gpu_append_device(struct tile_stream_gpu* s,
                                                     struct slice data,
                                                     void* cuda_stream);

  /* Append-to-delivered latency of every epoch delivered so far, in ms:
   * from the append call that completed the epoch's input to the end of
   * the sink writes of the batch holding it.  Writes up to `cap` values to
   * `out_ms` (may be NULL) and returns the total count. */
  size_t tile_stream_gpu_latencies(const struct tile_stream_gpu* s,
                                   double* out_ms,
                                   size_t cap);
  void tile_stream_gpu_clear_latencies(struct tile_stream_gpu* s);

  /* Latency bound for streams fed in small appends (no reference
   * counterpart: the reference delivers a batch when its K epochs are in,
   * src/stream/config.c:31-45).  With `ms` > 0, an append that finds the
   * oldest finished epoch of the batch being filled older than `ms`
   * starts that batch with the epochs it has (a partial batch, as a flush
   * does), and every append delivers the batches the GPU has finished
   * instead of leaving them to the next batch.  The shard bytes do not
   * change (chunks and their order within shards are the same) except
   * where the shard alignment pads each batch's group of chunks.  0 (the
   * default) turns it off.  Returns 0, or 1 for a negative `ms`. */
  int tile_stream_gpu_set_batch_deadline(struct tile_stream_gpu* s, double ms);

  /* A shard sink that discards every byte and counts them (the metering
   * sink of a throughput benchmark). */
  struct shard_sink* chucky_discard_sink_create(void);
  void chucky_discard_sink_destroy(struct shard_sink* s);
  uint64_t chucky_discard_sink_bytes(const struct shard_sink* s);

  /* Number of CUDA kernels this library has launched in this process. */
  uint64_t chucky_launch_count(void);

  /* crc32c (Castagnoli) of a buffer, as used by shard indexes. */
  uint32_t chucky_crc32c(const void* data, size_t len);

  /* LZ4 chunk encoder that allocates no memory (no reference counterpart).
   *
   * For callers that must not allocate once running: an acquisition loop
   * cannot afford cudaFree's device-wide synchronisation or an
   * out-of-memory failure in the middle of a run.  The encoder's scratch is
   * a fixed array of chucky_lz4_static_scratch_bytes() (32 MiB) in device
   * memory, one per CUDA context (held until the context ends), set up by
   * the first call made in that context (make that first call before any
   * stream capture and before anything that must not see setup work).  The
   * array's address is remembered per context ID, so calls after a
   * cudaDeviceReset, on another device, or in a context a driver-API caller
   * made current look it up again.  Requests needing more scratch than the
   * array holds -- about 10 MiB of input per call -- are rejected, however
   * large `n_chunks` is.
   *
   * Encodes `n_chunks` chunks of `chunk_bytes` each, chunk i at
   * d_chunks + i * in_stride (device memory, 4-byte aligned, `in_stride` a
   * multiple of 4; the 256 bytes after the last chunk must be readable),
   * into raw LZ4 blocks at d_out + i * out_stride (`out_stride` at least
   * chunk_bytes + chunk_bytes / 255 + 16) and their sizes at d_sizes[i],
   * asynchronously on `cuda_stream` (a cudaStream_t; NULL for the default
   * stream).  The output is byte-identical to what a tile_stream_gpu with
   * CODEC_LZ4_NON_STANDARD writes for the same chunk bytes.
   *
   * All calls in a context share its one scratch array: calls ordered on
   * one CUDA stream are safe, calls that may overlap (other streams, other
   * threads) race.  No part of the array needs to start at zero.
   *
   * Returns 0 on success, 1 for invalid arguments, 2 when the request
   * exceeds the fixed scratch, 3 for a CUDA error. */
  size_t chucky_lz4_static_scratch_bytes(void);
  int chucky_lz4_encode_chunks_static(const void* d_chunks,
                                      size_t chunk_bytes,
                                      size_t in_stride,
                                      size_t n_chunks,
                                      void* d_out,
                                      size_t out_stride,
                                      uint64_t* d_sizes,
                                      void* cuda_stream);

  /* Batched chunk encoding on the device, the stream's own encoders as a
   * library call (the batch counterpart of the reference's codec_compress,
   * src/gpu/compress.cu:284-369, which calls nvcomp).
   *
   * chucky_encode_bound: worst-case encoded size of one chunk (0 for a
   * codec other than CODEC_LZ4_NON_STANDARD / CODEC_ZSTD).
   * chucky_encode_scratch_bytes: device scratch chucky_encode_chunks needs
   * (the level matters: LZ4 levels >= 2 and zstd levels >= 3 search a
   * wider window, with region tables of about the input's size).
   * chucky_encode_chunks: encodes `n_chunks` chunks of `chunk_bytes`, chunk
   * i at d_chunks + i * in_stride (device memory, 4-byte aligned, the 256
   * bytes after the last chunk readable), into raw LZ4 blocks or zstd
   * frames at d_out + i * out_stride (out_stride >= the bound), sizes at
   * d_sizes[i], asynchronously on `cuda_stream` (a cudaStream_t; NULL for
   * the default stream), using `d_scratch` (not shared with a call that may
   * overlap).  The output equals what a tile_stream_gpu with that codec
   * writes for the same chunk bytes.  Returns 0, 1 for invalid arguments,
   * 3 for a CUDA error. */
  size_t chucky_encode_bound(int codec_id, size_t chunk_bytes);
  size_t chucky_encode_scratch_bytes(int codec_id, int level, size_t chunk_bytes,
                                     size_t n_chunks);
  int chucky_encode_chunks(int codec_id,
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
                           void* cuda_stream);

  /* Decode raw LZ4 blocks (CODEC_LZ4_NON_STANDARD chunks) on the device,
   * for on-device verification and readback; no counterpart in the
   * reference, which decodes with LZ4_decompress_safe on the host
   * (src/cpu/compress.c:85).
   *
   * Block i is d_in_sizes[i] bytes at d_in + d_in_offsets[i] and decodes
   * to exactly `chunk_bytes` bytes at d_out + i * out_stride.  All
   * pointers are device memory.  d_status[i] is set to 0 when block i
   * decoded to exactly chunk_bytes bytes, 1 when it ends inside a
   * sequence, 2 for a match offset of 0 or before the chunk start, 3 when
   * it would write past chunk_bytes, 4 when it ends short of chunk_bytes;
   * a malformed block is never read or written out of bounds.  Runs
   * asynchronously on `cuda_stream` (a cudaStream_t; NULL for the default
   * stream).  Returns 0 when launched, 1 for invalid arguments, 3 for a
   * CUDA error. */
  int chucky_lz4_decode_chunks(const void* d_in,
                               const uint64_t* d_in_offsets,
                               const uint64_t* d_in_sizes,
                               size_t n_chunks,
                               void* d_out,
                               size_t out_stride,
                               size_t chunk_bytes,
                               uint32_t* d_status,
                               void* cuda_stream);

  /* Decode zstd frames (CODEC_ZSTD chunks) on the device, for on-device
   * verification and readback; no counterpart in the reference, which
   * decodes with ZSTD_decompress on the host (src/cpu/compress.c:85-93).
   * Any conforming frame (RFC 8878) decodes, not only this library's:
   * skippable frames, several frames in a row, raw / RLE / compressed
   * blocks, every literals and sequences mode; frames that need a
   * dictionary are refused; a content checksum is skipped, not verified.
   *
   * Chunk i is d_in_sizes[i] bytes at d_in + d_in_offsets[i] and decodes to
   * exactly `chunk_bytes` bytes at d_out + i * out_stride.  All pointers are
   * device memory.  d_status[i] is set to 0 when chunk i decoded to exactly
   * chunk_bytes bytes, 1 when its input ends early, 2 for an invalid field,
   * table, bitstream or offset, 3 when it would write past chunk_bytes, 4
   * when it decodes to fewer bytes, 5 for a dictionary frame; a malformed
   * frame is never read or written out of bounds.  Runs asynchronously on
   * `cuda_stream` (a cudaStream_t; NULL for the default stream); a CTA per
   * chunk, no scratch.  Returns 0 when launched, 1 for invalid arguments, 3
   * for a CUDA error. */
  int chucky_zstd_decode_chunks(const void* d_in,
                                const uint64_t* d_in_offsets,
                                const uint64_t* d_in_sizes,
                                size_t n_chunks,
                                void* d_out,
                                size_t out_stride,
                                size_t chunk_bytes,
                                uint32_t* d_status,
                                void* cuda_stream);

  /* Encoder autotuner (no reference counterpart): the match finder's search
   * strength and shortest match are picked per (codec, level, dtype, chunk
   * shape) by timing candidates on a sample of the first batch's chunks:
   * among those that compress at most 1 % worse than the defaults, encode
   * time weighed
   * against the device-to-host cost of the compressed bytes; the choice is
   * kept for the process.  Off unless enabled here, by
   * CHUCKY_AUTOTUNE=1 in the environment, or by a server created with
   * `autotune` set (chucky_serve.h).  Streams created while it is on tune
   * at their first batch (the host waits for the trials, tens of ms, once
   * per key).
   * chucky_autotune_entries: the table (up to `cap` entries to `out`, which
   * may be NULL); returns the entry count.
   * chucky_autotune_pick: the choice among n measured candidates (index),
   * given encode seconds and compressed bytes for `in_bytes` of input and
   * the copy-out rate in GB/s: of the candidates whose output is at most
   * 1 % above `preferred`'s (the smallest output's when `preferred` < 0),
   * the one of least max(encode, copy-out) + 1/4 min(encode, copy-out); a
   * candidate within 1 % of that cost loses to `preferred`. */
  struct chucky_autotune_entry
  {
    int codec, level, dtype, rank;
    uint64_t chunk_shape[16];
    uint64_t chunk_bytes;
    int strength;   /* 0: the level's default */
    int min_match;  /* 0: the level's default */
    double encode_gbs, ratio; /* of the chosen candidate on the sample */
    uint32_t candidates;      /* 0: tuning failed, defaults kept */
  };
  void chucky_autotune_set_enabled(int on);
  int chucky_autotune_enabled(void);
  size_t chucky_autotune_entries(struct chucky_autotune_entry* out, size_t cap);
  void chucky_autotune_clear(void);
  int chucky_autotune_pick(const double* enc_s,
                           const double* out_bytes,
                           int n,
                           double in_bytes,
                           double d2h_gbs,
                           int preferred);

#ifdef __cplusplus
}
#endif
