// Stand-in for <cuda_runtime.h> when the encoder sources are compiled for
// the CPU SIMT emulation (tests/emu/simt.hpp).  Test infrastructure only.
#pragma once
#include "../simt.hpp"
