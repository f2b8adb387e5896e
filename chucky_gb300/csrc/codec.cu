// (c) Batched chunk encoders behind the stream: dispatch on the codec id.
#include "stream_internal.hpp"

namespace chucky {

int Stream::codec_init()
{
  return cfg.codec.id == CODEC_NONE ? 0 : 1; // encoders land in lz4.cu/zstd.cu
}

int Stream::codec_compress(uint64_t nchunks)
{
  (void)nchunks;
  return 1;
}

void Stream::codec_release() {}

} // namespace chucky
