/* Prototype-only declarations of the public liblz4 entry points that the
 * reference CPU backend calls (liblz4 1.9.x ABI).  Used only to compile the
 * reference sources into oracle/_ref against the system liblz4.so.1. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
int LZ4_compress_HC(const char* src, char* dst, int srcSize, int dstCapacity,
                    int compressionLevel);
int LZ4_compressBound(int inputSize);
int LZ4_decompress_safe(const char* src, char* dst, int compressedSize,
                        int dstCapacity);
#ifdef __cplusplus
}
#endif
