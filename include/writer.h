/* Writer / shard-sink interfaces.  Struct layouts and vtables match
 * src/writer.h:8-74 of the reference; the helpers replace
 * src/writer.h:76-98 (implemented in writer.c of the reference). */
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  struct io_event
  {
    uint64_t seq;
  };

  struct slice
  {
    const void* beg;
    const void* end;
  };

  enum writer_error_code
  {
    writer_error_ok = 0,
    writer_error_fail = 1,
    writer_error_finished = 2, /* capacity reached or flush already called */
  };

  struct writer_result
  {
    int error;         /* writer_error_code */
    struct slice rest; /* input not consumed */
  };

  /* Returned by the library; append/flush drive the stream. */
  struct writer
  {
    struct writer_result (*append)(struct writer* self, struct slice data);
    struct writer_result (*flush)(struct writer* self);
  };

  /* Provided by the caller: one open shard file. */
  struct shard_writer
  {
    int (*write)(struct shard_writer* self,
                 uint64_t offset,
                 const void* beg,
                 const void* end);
    /* Zero-copy variant (may be NULL): the buffer stays valid until the
     * sink's fence for this level retires. */
    int (*write_direct)(struct shard_writer* self,
                        uint64_t offset,
                        const void* beg,
                        const void* end);
    int (*finalize)(struct shard_writer* self);
  };

  /* Provided by the caller: opens shards and (optionally) tracks IO. */
  struct shard_sink
  {
    struct shard_writer* (*open)(struct shard_sink* self,
                                 uint8_t level,
                                 uint64_t shard_index);
    int (*update_append)(struct shard_sink* self,
                         uint8_t level,
                         uint8_t n_append,
                         const uint64_t* append_sizes); /* may be NULL */
    struct io_event (*record_fence)(struct shard_sink* self,
                                    uint8_t level); /* may be NULL */
    void (*wait_fence)(struct shard_sink* self,
                       uint8_t level,
                       struct io_event ev); /* may be NULL */
  };

  struct writer_result writer_ok(void);
  struct writer_result writer_error(void);
  struct writer_result writer_error_at(const void* beg, const void* end);
  struct writer_result writer_finished_at(const void* beg, const void* end);

  /* w->append(w, data). */
  struct writer_result writer_append(struct writer* w, struct slice data);

  /* w->flush(w); terminal. */
  struct writer_result writer_flush(struct writer* w);

  /* Append, backing off 1..64 ms while no input is consumed; gives up after
   * 10 stalls in a row (src/writer.c:19-45). */
  struct writer_result writer_append_wait(struct writer* w, struct slice data);

#ifdef __cplusplus
}
#endif
