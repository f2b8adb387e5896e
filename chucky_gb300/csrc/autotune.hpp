// Encoder autotuner: parse parameters picked per (codec, level, dtype, chunk
// shape) by timing candidates on the GPU.
//
// The reference has no counterpart (its encoders are nvcomp's, or the CPU
// libraries').  The parameters tuned are the match finder's search strength
// (how fast probing thins out in literal runs) and its shortest match
// (CodecBatch::strength, ::min_match): they trade encoder time against
// compressed bytes, and which trade pays depends on the data and on what
// the compressed bytes cost downstream (the copy to the host).  A key seen
// for the first time is tuned on a sample of the chunks of its first batch:
// every candidate encodes the sample (into the tuner's own buffers) and is
// timed with CUDA events.  The candidates whose output is at most 1 % above
// the defaults' are eligible (the tuner buys speed or ratio, never speed
// with ratio), and of those the one with the lowest cost per input byte
// wins, cost =
// max(encode, copy-out) + 1/4 min(encode, copy-out), the copy-out at the
// device-to-host rate measured once per device (the two run on different
// engines and mostly overlap).  The choice is kept for the process, so
// every stream of a key encodes the same way.
//
// Tuning is off unless enabled (chucky_autotune_set_enabled, the
// environment variable CHUCKY_AUTOTUNE=1, or a server created with
// autotuning): without it a stream's output is byte-identical run to run
// and to the library's batch encoders at their defaults.
#pragma once

#include "kernels_codec.hpp"

#include <cuda_runtime.h>
#include <stdint.h>

namespace chucky {

struct TuneKey
{
  int codec = 0, level = 0, dtype = 0, rank = 0;
  uint64_t chunk[16] = {}; // chunk extents, outermost first
  bool operator<(const TuneKey& o) const;
};

struct TuneParams
{
  int strength = 0;  // 0: the level's default
  int min_match = 0; // 0: the level's default
};

bool autotune_enabled();
void autotune_set_enabled(bool on);

// The parameters for `key`.  A new key (with tuning enabled) is tuned on
// `n` sample chunks of `chunk_bytes` (device memory, each readable 256 bytes
// past its end), after the work `ready` marks (an event, or null); the host
// waits for the trials.  With tuning disabled, or when the trials fail,
// returns the defaults (and a failed key is not retried).
TuneParams autotune(const TuneKey& key,
                    uint32_t chunk_bytes,
                    const uint8_t* const* sample,
                    uint32_t n,
                    cudaEvent_t ready);

// Index of the eligible candidate of least cost (see above) among n, given
// each one's encode seconds and compressed bytes for `in_bytes` of input; a
// candidate within 1 % of the best cost loses to `preferred` (the
// defaults) when that is eligible.
int autotune_pick(const double* enc_s,
                  const double* out_bytes,
                  int n,
                  double in_bytes,
                  double d2h_gbs,
                  int preferred);

} // namespace chucky
