// Tables of the zstd format (RFC 8878) shared by the encoder (zstd.cu) and
// the decoder (zstd_decode.cu).
#pragma once

#include <stdint.h>

namespace chucky {

// Predefined distributions (RFC 8878 3.1.1.3.2.2), one list each, as host
// arrays (the encoder builds its predefined tables on the host) and device
// constants (the decoder builds them in its kernel).
#define CHUCKY_ZSTD_LL_NORM                                                     \
  4, 3, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 3, \
    2, 1, 1, 1, 1, 1, -1, -1, -1, -1
#define CHUCKY_ZSTD_ML_NORM                                                     \
  1, 4, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, \
    1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1,  \
    -1, -1, -1
#define CHUCKY_ZSTD_OF_NORM                                                     \
  1, 1, 1, 1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1,   \
    -1, -1, -1, -1

namespace {

static const int16_t kLLNormH[36] = { CHUCKY_ZSTD_LL_NORM };
static const int16_t kMLNormH[53] = { CHUCKY_ZSTD_ML_NORM };
static const int16_t kOFNormH[29] = { CHUCKY_ZSTD_OF_NORM };
__constant__ int16_t kLLNormD[36] = { CHUCKY_ZSTD_LL_NORM };
__constant__ int16_t kMLNormD[53] = { CHUCKY_ZSTD_ML_NORM };
__constant__ int16_t kOFNormD[29] = { CHUCKY_ZSTD_OF_NORM };

// Literal-length and match-length codes: base values and extra bits
// (RFC 8878 3.1.1.3.2.1.1).
__constant__ uint32_t kLLBase[36] = { 0,  1,  2,   3,   4,   5,    6,    7,
                                      8,  9,  10,  11,  12,  13,   14,   15,
                                      16, 18, 20,  22,  24,  28,   32,   40,
                                      48, 64, 128, 256, 512, 1024, 2048, 4096,
                                      8192, 16384, 32768, 65536 };
__constant__ uint8_t kLLBits[36] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 3, 3,
                                     4, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16 };
__constant__ uint32_t kMLBase[53] = {
  3,  4,  5,  6,  7,  8,  9,  10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20,
  21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 33, 34, 35, 37, 39, 41,
  43, 47, 51, 59, 67, 83, 99, 131, 259, 515, 1027, 2051, 4099, 8195, 16387,
  32771, 65539
};
__constant__ uint8_t kMLBits[53] = { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 3, 3, 4, 4,
                                     5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16 };

} // namespace

} // namespace chucky
