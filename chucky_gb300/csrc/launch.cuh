// Kernel launch spelled as a macro so that the encoder sources can also be
// compiled by the CPU SIMT emulation used in tests (tests/emu).
#pragma once

#ifndef CHUCKY_LAUNCH
#define CHUCKY_LAUNCH(kernel, grid, block, smem, stream, ...)                  \
  kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__)
#endif

// Dynamically sized shared memory array of a kernel.
#ifndef CHUCKY_DYN_SHARED
#define CHUCKY_DYN_SHARED(T, name) extern __shared__ __align__(16) T name[]
#endif
