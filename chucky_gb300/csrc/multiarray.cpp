// Multi-array writer over one GPU stream per array (the GPU counterpart of
// the reference's CPU multi-array stream, src/multiarray/stream.c:552-830).
//
// The reference shares one chunk pool between its arrays, so it flushes the
// departing array's batch and clears the pool when the caller switches
// arrays.  Here every array keeps its own resident stream; switching only
// checks the reference's rule (the departing array must stand at an epoch
// boundary) and each array's shards are byte-identical to those of the
// array ingested on its own.
#include "multiarray.gpu.h"

#include <new>
#include <vector>

namespace {

struct MultiArray
{
  multiarray_writer writer; // first member: the vtable the caller holds
  std::vector<tile_stream_gpu*> streams;
  std::vector<uint64_t> epoch_elements;
  int active = -1;
};

MultiArray* from_writer(multiarray_writer* w)
{
  return reinterpret_cast<MultiArray*>(w);
}

multiarray_writer_result result(int error, const void* beg, const void* end)
{
  return multiarray_writer_result{ error, slice{ beg, end } };
}

multiarray_writer_result update_impl(multiarray_writer* self,
                                     int array_index,
                                     slice data)
{
  MultiArray* m = from_writer(self);
  if (array_index < 0 || array_index >= int(m->streams.size()))
    return result(multiarray_writer_fail, data.beg, data.end);
  if (array_index != m->active && m->active >= 0) {
    // src/multiarray/stream.c:552-571: switch only at an epoch boundary
    const int a = m->active;
    if (tile_stream_gpu_cursor(m->streams[a]) % m->epoch_elements[a] != 0)
      return result(multiarray_writer_not_flushable, data.beg, data.end);
  }
  m->active = array_index;
  writer* w = tile_stream_gpu_writer(m->streams[array_index]);
  const writer_result r = writer_append(w, data);
  switch (r.error) {
    case writer_error_ok:
      return result(multiarray_writer_ok, r.rest.beg, r.rest.end);
    case writer_error_finished:
      return result(multiarray_writer_finished, r.rest.beg, r.rest.end);
    default:
      return result(multiarray_writer_fail, r.rest.beg, r.rest.end);
  }
}

multiarray_writer_result flush_impl(multiarray_writer* self)
{
  MultiArray* m = from_writer(self);
  int error = multiarray_writer_ok;
  for (tile_stream_gpu* s : m->streams) {
    const writer_result r = writer_flush(tile_stream_gpu_writer(s));
    if (r.error == writer_error_fail && error == multiarray_writer_ok)
      error = multiarray_writer_fail;
  }
  return result(error, nullptr, nullptr);
}

void add(stream_metric& a, const stream_metric& b)
{
  a.ms += b.ms;
  a.best_ms = b.best_ms < a.best_ms ? b.best_ms : a.best_ms;
  a.input_bytes += b.input_bytes;
  a.output_bytes += b.output_bytes;
  a.count += b.count;
  if (!a.name)
    a.name = b.name;
}

} // namespace

extern "C" multiarray_tile_stream_gpu*
multiarray_tile_stream_gpu_create(int n_arrays,
                                  const tile_stream_configuration configs[],
                                  shard_sink* sinks[],
                                  int enable_metrics)
{
  (void)enable_metrics;
  if (n_arrays <= 0 || !configs || !sinks)
    return nullptr;
  MultiArray* m = new (std::nothrow) MultiArray{};
  if (!m)
    return nullptr;
  m->writer.update = update_impl;
  m->writer.flush = flush_impl;
  for (int i = 0; i < n_arrays; ++i) {
    tile_stream_gpu* s = tile_stream_gpu_create(&configs[i], sinks[i]);
    if (!s) {
      multiarray_tile_stream_gpu_destroy(
        reinterpret_cast<multiarray_tile_stream_gpu*>(m));
      return nullptr;
    }
    m->streams.push_back(s);
    m->epoch_elements.push_back(tile_stream_gpu_layout(s)->epoch_elements);
  }
  return reinterpret_cast<multiarray_tile_stream_gpu*>(m);
}

extern "C" void
multiarray_tile_stream_gpu_destroy(multiarray_tile_stream_gpu* ms)
{
  MultiArray* m = reinterpret_cast<MultiArray*>(ms);
  if (!m)
    return;
  for (tile_stream_gpu* s : m->streams)
    tile_stream_gpu_destroy(s);
  delete m;
}

extern "C" multiarray_writer*
multiarray_tile_stream_gpu_writer(multiarray_tile_stream_gpu* ms)
{
  return ms ? &reinterpret_cast<MultiArray*>(ms)->writer : nullptr;
}

extern "C" stream_metrics
multiarray_tile_stream_gpu_get_metrics(const multiarray_tile_stream_gpu* ms)
{
  stream_metrics out{};
  const MultiArray* m = reinterpret_cast<const MultiArray*>(ms);
  if (!m || m->streams.empty())
    return out;
  out = tile_stream_gpu_get_metrics(m->streams[0]);
  for (size_t i = 1; i < m->streams.size(); ++i) {
    const stream_metrics b = tile_stream_gpu_get_metrics(m->streams[i]);
    add(out.memcpy, b.memcpy);
    add(out.h2d, b.h2d);
    add(out.lod_gather, b.lod_gather);
    add(out.lod_reduce, b.lod_reduce);
    add(out.lod_append_fold, b.lod_append_fold);
    add(out.lod_morton_chunk, b.lod_morton_chunk);
    add(out.scatter, b.scatter);
    add(out.compress, b.compress);
    add(out.aggregate, b.aggregate);
    add(out.d2h, b.d2h);
    add(out.sink, b.sink);
  }
  return out;
}
