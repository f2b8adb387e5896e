/* Element types of a stream.  Enumerator order and byte widths match
 * src/dtype.h:10-23 (enum) and :25-45 (dtype_bpe) of the reference. */
#pragma once

#include <stddef.h>

#ifdef __cplusplus
extern "C"
{
#endif

  enum dtype
  {
    dtype_u8,
    dtype_u16,
    dtype_u32,
    dtype_u64,
    dtype_i8,
    dtype_i16,
    dtype_i32,
    dtype_i64,
    dtype_f16,
    dtype_f32,
    dtype_f64,
  };

  /* Bytes per element; 0 for an unknown enumerator. */
  static inline size_t dtype_bpe(enum dtype dt)
  {
    switch (dt) {
      case dtype_u8:
      case dtype_i8:
        return 1;
      case dtype_u16:
      case dtype_i16:
      case dtype_f16:
        return 2;
      case dtype_u32:
      case dtype_i32:
      case dtype_f32:
        return 4;
      case dtype_u64:
      case dtype_i64:
      case dtype_f64:
        return 8;
    }
    return 0;
  }

  /* Zarr v3 "data_type" name. */
  static inline const char* dtype_zarr_string(enum dtype dt)
  {
    static const char* const names[] = { "uint8",  "uint16", "uint32",
                                         "uint64", "int8",   "int16",
                                         "int32",  "int64",  "float16",
                                         "float32", "float64" };
    if ((unsigned)dt <= (unsigned)dtype_f64)
      return names[dt];
    return "unknown";
  }

#ifdef __cplusplus
}
#endif
