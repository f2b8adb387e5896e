/* Chunk codecs.  Enumerators and struct layout match src/types.codec.h:10-34
 * of the reference. */
#pragma once

#include <stdint.h>

#ifdef __cplusplus
extern "C"
{
#endif

  enum compression_codec
  {
    CODEC_NONE,
    CODEC_LZ4_NON_STANDARD, /* raw LZ4 block per chunk (no frame) */
    CODEC_ZSTD,             /* one standard zstd frame per chunk */
    CODEC_BLOSC_LZ4,
    CODEC_BLOSC_ZSTD,
  };

  enum codec_shuffle
  {
    CODEC_SHUFFLE_NONE = 0,
    CODEC_SHUFFLE_BYTE = 1,
    CODEC_SHUFFLE_BIT = 2,
  };

  struct codec_config
  {
    enum compression_codec id;
    uint8_t level;              /* LZ4: 1..12 (0 rejected); zstd: any */
    enum codec_shuffle shuffle; /* blosc only */
  };

  /* Replaces src/types.codec.c:3-8. */
  int codec_is_blosc(enum compression_codec c);

  /* Replaces src/types.codec.c:10-14: NONE, LZ4 and ZSTD run on the GPU. */
  int codec_is_gpu_supported(enum compression_codec c);

#ifdef __cplusplus
}
#endif
