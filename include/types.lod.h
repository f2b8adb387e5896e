/* Level-of-detail reduce methods.  Enumerator order matches
 * src/types.lod.h:10-18 of the reference. */
#pragma once

#include "dtype.h"

#ifdef __cplusplus
extern "C"
{
#endif

  enum lod_reduce_method
  {
    lod_reduce_mean,
    lod_reduce_min,
    lod_reduce_max,
    lod_reduce_median,
    lod_reduce_max_suppressed, /* second highest of the window */
    lod_reduce_min_suppressed, /* second lowest of the window */
  };

  /* Dim-0 accumulators are kept in the element type itself (no widening),
   * as in src/types.lod.h:23-28. */
  static inline size_t dtype_accum_bpe(enum dtype dt,
                                       enum lod_reduce_method method)
  {
    (void)method;
    return dtype_bpe(dt);
  }

#ifdef __cplusplus
}
#endif
