/* Prototype-only declarations of the public libzstd entry points that the
 * reference CPU backend calls (libzstd 1.5.x ABI).  Used only to compile the
 * reference sources into oracle/_ref against the system libzstd.so.1. */
#pragma once
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
size_t ZSTD_compress(void* dst, size_t dstCapacity, const void* src,
                     size_t srcSize, int compressionLevel);
size_t ZSTD_decompress(void* dst, size_t dstCapacity, const void* src,
                       size_t compressedSize);
size_t ZSTD_compressBound(size_t srcSize);
unsigned ZSTD_isError(size_t code);
const char* ZSTD_getErrorName(size_t code);
#ifdef __cplusplus
}
#endif
