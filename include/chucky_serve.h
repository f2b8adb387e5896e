/* Served form: many concurrent ingest streams on one GPU, admitted against
 * an HBM budget, with their encoder work batched across streams.
 *
 * No counterpart in the reference, whose GPU multi-array stream is an open
 * TODO (docs/devlog.md:6); its CPU analogue is the multi-array stream
 * (src/multiarray/stream.c:552-728), which shares one pool among arrays of
 * one writer.  Here a server keeps GPU streams (tile_stream_gpu) resident
 * on the device and hands them to requests:
 *
 *   * admission: a request is admitted once fewer than `max_streams`
 *     requests are open and its stream fits the HBM budget (the sum of the
 *     device-memory estimates of the resident streams).  A finished
 *     request's stream stays resident, idle, and is restarted for the next
 *     request with the same configuration (no allocation); idle streams of
 *     other configurations are released when room is needed;
 *   * continuous batching: with `batch_encoders`, the server's streams do
 *     not encode on their own.  Each batch (every chunk of its epochs, all
 *     pyramid levels) goes to one shared encoder engine, which encodes the
 *     ready batches of all open requests that share a codec and chunk size
 *     in common launches -- work that arrives while earlier launches run on
 *     the GPU joins the next ones;
 *   * each request's shards are byte-identical to those of the same input
 *     through a tile_stream_gpu of its own (the encoders work per chunk).
 *
 * Threading: one thread per open request drives it (writer_append /
 * writer_flush on chucky_request_writer); different requests may be driven
 * from different threads at the same time.  The server's own calls are
 * thread-safe. */
#pragma once

#include "types.stream.h"
#include "writer.h"

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  struct chucky_server_config
  {
    size_t hbm_budget_bytes; /* admission budget of the resident streams */
    int max_streams;         /* requests open at once (>= 1) */
    int batch_encoders;      /* 1: shared encoder engine across streams */
    size_t encoder_wave_bytes; /* engine launch size (0: 256 MiB of input) */
    int encoder_lanes;         /* engine CUDA streams, rounds overlap (0: 2) */
    int autotune;              /* 1: turn on the encoder autotuner
                                  (chucky_autotune_set_enabled, process-wide) */
    double batch_deadline_ms;  /* > 0: every request's stream starts a
                                  partial batch once its oldest epoch has
                                  waited this long
                                  (tile_stream_gpu_set_batch_deadline) */
  };

  struct chucky_server;
  struct chucky_request;

  struct chucky_server* chucky_server_create(
    const struct chucky_server_config* config);

  /* All requests must be closed first. */
  void chucky_server_destroy(struct chucky_server* s);

  /* Admit a request: a resident stream for `config` writing to `sink`.
   * Waits up to `timeout_ms` (< 0: without limit) for a free slot and room
   * in the budget.  NULL when the configuration is invalid, can never fit
   * the budget, or the wait timed out.  `config->dimensions` must outlive
   * the request. */
  struct chucky_request* chucky_server_open(struct chucky_server* s,
                                            const struct tile_stream_configuration* config,
                                            struct shard_sink* sink,
                                            int timeout_ms);

  /* Server start-up: create idle resident streams for `configs[0..n)` (one
   * each; repeat a configuration to keep several), in order, while they fit
   * the budget.  Requests with those configurations then start without
   * allocating.  `sink` is a placeholder sink (each request brings its
   * own).  Returns the number of streams created. */
  size_t chucky_server_prewarm(struct chucky_server* s,
                               const struct tile_stream_configuration* const* configs,
                               size_t n,
                               struct shard_sink* sink);

  /* The request's writer (append / flush as for tile_stream_gpu). */
  struct writer* chucky_request_writer(struct chucky_request* r);

  /* End a request (after its flush, or to abandon it): its stream returns
   * to the idle pool (or is released when it was not flushed).  Its
   * append-to-delivered latencies join the server's statistics.  Returns 0,
   * or 1 when the request was not flushed. */
  int chucky_request_close(struct chucky_request* r);

  struct chucky_server_stats
  {
    uint64_t requests;        /* closed */
    uint64_t input_bytes;     /* appended by closed requests */
    uint64_t epochs;          /* latency samples */
    double p50_ms, p99_ms, max_ms; /* append-to-delivered, per epoch */
    uint64_t streams_created, streams_reused, streams_evicted;
    uint64_t peak_resident_bytes;
    uint64_t peak_open;
    /* shared encoder engine */
    uint64_t engine_rounds, engine_jobs, engine_launch_sets;
    uint64_t engine_max_jobs_per_round;
  };

  void chucky_server_get_stats(struct chucky_server* s,
                               struct chucky_server_stats* out);
  void chucky_server_reset_stats(struct chucky_server* s);

  /* Request-loop driver: runs `n` requests against the server, one host
   * thread per admitted request, as a front end would.  Request i arrives
   * at arrival_s[i] seconds after the start (sorted or not), waits for
   * admission, appends its `bytes` from `data` in pieces of `append_bytes`
   * with exponentially distributed gaps of mean `mean_gap_s` (0: back to
   * back), flushes and closes.  Returns 0 when every request succeeded;
   * `wall_s` receives the time from the start to the last close. */
  struct chucky_replay_request
  {
    const struct tile_stream_configuration* config;
    struct shard_sink* sink;
    const void* data;
    size_t bytes;
    size_t append_bytes;
    double arrival_s;
    double mean_gap_s;
    uint64_t seed;
  };

  int chucky_server_replay(struct chucky_server* s,
                           const struct chucky_replay_request* requests,
                           size_t n,
                           double* wall_s);

#ifdef __cplusplus
}
#endif
