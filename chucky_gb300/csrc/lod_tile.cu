// (b) LOD pyramid, tiled single-pass path (1 to 3 LOD dims).
//
// A CTA owns one power-of-two tile of the LOD dims of one fixed-dims slice
// (64x64 for 2-D, 16^3 for 3-D, 1024 for 1-D) and produces every level
// inside that tile from one staged read of L0:
//   1. L0 tile: coalesced loads from the row-major epoch buffer into shared
//      memory, then stored to the L0 chunk tiles of the pool slot;
//   2. level l+1 = reduce of the in-bounds 2^D children of each parent, in
//      Z order of the child offset (dim 0 fastest) -- exactly the Morton
//      window [ends[i-1], ends[i]) of the reference, so sums accumulate in
//      the reference's order (src/cpu/lod.cpp:55-127, 269-296;
//      src/lod/lod_plan.c:105-125);
//   3. each level is either stored to its chunk tiles, or (dim-0
//      downsampling) folded into a dense accumulator and emitted when the
//      level's period completes (src/cpu/lod.cpp:366-438).
// The Morton buffers, gather LUT and per-level scatter LUTs of the general
// path are not needed: chunk positions are computed from coordinates.
#include "kernels.hpp"
#include "lod_ops.cuh"

namespace chucky {

namespace {

constexpr int kTileThreads = 256;

template<int D>
struct TileGeom;
template<>
struct TileGeom<1>
{
  static constexpr int log = 10; // 1024
};
template<>
struct TileGeom<2>
{
  static constexpr int log = 6; // 64 x 64
};
template<>
struct TileGeom<3>
{
  static constexpr int log = 4; // 16^3
};

// parents of levels 1..TL inside one L0 tile: the accumulator values a
// CTA stages for its dim-0 folds
template<int D>
__host__ __device__ constexpr int stage_elems()
{
  int n = 0;
  for (int l = 1; l <= TileGeom<D>::log; ++l)
    n += 1 << (D * (TileGeom<D>::log - l));
  return n;
}

// chunk-pool offset (elements) of LOD coords x at level l (fixed part added
// by the caller)
template<int D>
__device__ __forceinline__ uint64_t chunk_pos(const LodTileArgs& a,
                                              int l,
                                              const uint32_t* x)
{
  uint64_t o = 0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const uint32_t cs = a.cs[k];
    o += uint64_t(x[k] / cs) * a.lv[l].S[k] + uint64_t(x[k] % cs) * a.lv[l].s[k];
  }
  return o;
}

template<typename T, int D>
__global__ void __launch_bounds__(kTileThreads)
lod_tile_k(LodTileArgs a)
{
  constexpr int TL = TileGeom<D>::log;
  constexpr int TE = 1 << TL;             // tile edge at L0
  constexpr int TN = 1 << (D * TL);       // tile elements at L0
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* cur = reinterpret_cast<T*>(smem_raw);    // level l values (TN)
  T* nxt = cur + TN;                          // level 1 values (TN >> D); the
                                              // two regions swap per level
  constexpr int TS = stage_elems<D>();
  T* const stage = nxt + (TN >> D); // folded levels' accumulators (TS)

  const uint64_t b = blockIdx.y; // fixed-dims slice
  uint32_t tcoord[3] = { 0, 0, 0 };
  {
    uint64_t t = blockIdx.x;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      tcoord[k] = uint32_t(t % a.tiles[k]);
      t /= a.tiles[k];
    }
  }
  const T* lin = reinterpret_cast<const T*>(a.linear) + a.gather_fixed[b];
  T* slot = reinterpret_cast<T*>(a.slot);

  // ---- accumulators of the levels folded this epoch (dim-0 downsampling),
  // loaded up front with L0: the CTA waits on global memory once instead of
  // once per level.  Entry j of the stage is parent j - base(l) of level l
  // (levels in order, parents row-major in the tile, last dim fastest).
  constexpr int kPre = (TS + kTileThreads - 1) / kTileThreads;
  T pre[kPre];
  uint32_t pre_ok = 0;
#pragma unroll
  for (int s = 0; s < kPre; ++s) {
    const int j = s * kTileThreads + int(threadIdx.x);
    if (j >= TS)
      continue;
    int l = 1, base = 0;
    while (j - base >= (1 << (D * (TL - l)))) {
      base += 1 << (D * (TL - l));
      ++l;
    }
    if (l >= a.nlod || !((a.fold_mask >> l) & 1) || a.count[l] == 0)
      continue;
    const int plog = TL - l;
    int r = j - base;
    uint32_t pc[3];
#pragma unroll
    for (int k = D - 1; k >= 0; --k) {
      pc[k] = uint32_t(r & ((1 << plog) - 1));
      r >>= plog;
    }
    uint64_t ai = 0;
    bool in = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const uint32_t gx = ((tcoord[k] * uint32_t(TE)) >> l) + pc[k];
      in &= gx < a.lv[l].shape[k];
      ai = ai * a.lv[l].shape[k] + gx;
    }
    if (!in)
      continue;
    pre[s] = reinterpret_cast<const T*>(a.accum)[a.lv[l].accum_off +
                                                 b * a.lv[l].nelem + ai];
    pre_ok |= 1u << s;
  }

  // ---- L0: load (innermost LOD dim fastest -> coalesced rows) ----
  uint32_t ext[3]; // extent of this tile at the current level (<= edge)
  uint32_t org[3]; // tile origin at the current level
#pragma unroll
  for (int k = 0; k < D; ++k) {
    org[k] = tcoord[k] * TE;
    const uint64_t rem = a.lv[0].shape[k] - org[k];
    ext[k] = uint32_t(rem < uint64_t(TE) ? rem : uint64_t(TE));
  }
  const uint64_t fixed0 = a.lv[0].chunk_fixed ? a.lv[0].chunk_fixed[b] : 0;
  // Fast path (2-D, whole tile inside one chunk, rows contiguous in the
  // input and in the chunk, 16-byte aligned): rows move as 16-byte vectors.
  bool fast = D == 2 && sizeof(T) <= 16;
  uint64_t in0 = 0, out0 = fixed0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    fast &= ext[k] == uint32_t(TE) && a.cs[k] % TE == 0;
    in0 += uint64_t(org[k]) * a.in_stride[k];
    out0 += uint64_t(org[k] / a.cs[k]) * a.lv[0].S[k] +
            uint64_t(org[k] % a.cs[k]) * a.lv[0].s[k];
  }
  if (D == 2) {
    constexpr uint64_t kVecElems = 16 / sizeof(T);
    fast &= a.in_stride[D - 1] == 1 && a.lv[0].s[D - 1] == 1 &&
            (a.gather_fixed[b] + in0) % kVecElems == 0 &&
            uint64_t(a.in_stride[0]) % kVecElems == 0 && out0 % kVecElems == 0 &&
            a.lv[0].s[0] % kVecElems == 0 &&
            (reinterpret_cast<uintptr_t>(lin) & 15) == 0 &&
            (reinterpret_cast<uintptr_t>(slot) & 15) == 0;
  }
  // Every thread issues all its L0 loads before its first store (the
  // stores could alias the input as far as the compiler knows, so it would
  // not hoist the loads itself).
  if constexpr (D == 2) {
    if (fast) {
      constexpr int kVec = 16 / int(sizeof(T)); // elements per vector
      constexpr int kVpr = TE / kVec;           // vectors per row
      constexpr int kIt = TE * kVpr / kTileThreads;
      constexpr int kG = kIt < 4 ? kIt : 4; // vectors in flight per thread
#pragma unroll 1
      for (int g = 0; g < kIt; g += kG) {
        uint4 v[kG];
#pragma unroll
        for (int s = 0; s < kG; ++s) {
          const int i = (g + s) * kTileThreads + int(threadIdx.x);
          const int row = i / kVpr, col = i % kVpr;
          v[s] = *reinterpret_cast<const uint4*>(
            lin + in0 + uint64_t(row) * a.in_stride[0] + uint64_t(col) * kVec);
        }
#pragma unroll
        for (int s = 0; s < kG; ++s) {
          const int i = (g + s) * kTileThreads + int(threadIdx.x);
          const int row = i / kVpr, col = i % kVpr;
          *reinterpret_cast<uint4*>(cur + row * TE + col * kVec) = v[s];
          *reinterpret_cast<uint4*>(slot + out0 + uint64_t(row) * a.lv[0].s[0] +
                                    uint64_t(col) * kVec) = v[s];
        }
      }
    }
  }
  if (!fast) {
    constexpr int kIt = TN / kTileThreads;
    constexpr int kG = 4; // elements in flight per thread
#pragma unroll 1
    for (int g = 0; g < kIt; g += kG) {
      T v[kG];
      uint32_t ok = 0;
#pragma unroll
      for (int s = 0; s < kG; ++s) {
        const int i = (g + s) * kTileThreads + int(threadIdx.x);
        uint32_t in = 1;
        uint64_t off = 0;
        int r = i;
#pragma unroll
        for (int k = D - 1; k >= 0; --k) { // row-major in the tile, last LOD dim fastest
          in &= (r & (TE - 1)) < int(ext[k]);
          off += uint64_t(org[k] + (r & (TE - 1))) * a.in_stride[k];
          r >>= TL;
        }
        if (in) {
          v[s] = lin[off];
          ok |= 1u << s;
        }
      }
#pragma unroll
      for (int s = 0; s < kG; ++s) {
        if (!((ok >> s) & 1))
          continue;
        const int i = (g + s) * kTileThreads + int(threadIdx.x);
        uint32_t x[3];
        int r = i;
#pragma unroll
        for (int k = D - 1; k >= 0; --k) {
          x[k] = org[k] + (r & (TE - 1));
          r >>= TL;
        }
        cur[i] = v[s];
        slot[fixed0 + chunk_pos<D>(a, 0, x)] = v[s];
      }
    }
  }
#pragma unroll
  for (int s = 0; s < kPre; ++s)
    if ((pre_ok >> s) & 1)
      stage[s * kTileThreads + int(threadIdx.x)] = pre[s];
  __syncthreads();

  // ---- levels 1.. ----
  int edge = TE, elog = TL, sbase = 0;
  for (int l = 1; l < a.nlod && l <= TL; ++l) {
    const int pe = edge >> 1; // parent tile edge
    const int plog = elog - 1;
    int pn = 1;
#pragma unroll
    for (int k = 0; k < D; ++k)
      pn *= pe;
    uint32_t cext[3], porg[3], pext[3];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      cext[k] = ext[k];
      porg[k] = org[k] >> 1;
      const uint64_t shp = a.lv[l].shape[k];
      const uint64_t rem = shp > porg[k] ? shp - porg[k] : 0;
      pext[k] = uint32_t(rem < uint64_t(pe) ? rem : uint64_t(pe));
    }
    const bool fold = (a.fold_mask >> l) & 1;
    const bool emit = (a.emit_mask >> l) & 1;
    const uint64_t fixedl = a.lv[l].chunk_fixed ? a.lv[l].chunk_fixed[b] : 0;
    // 32-bit index arithmetic where it fits: offsets within the parent
    // tile's chunk, and a slice's accumulator index (the slice's base
    // pointer once per level)
    uint32_t s32[3], shp32[3];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      s32[k] = uint32_t(a.lv[l].s[k]);
      shp32[k] = uint32_t(a.lv[l].shape[k]);
    }
    const bool ai32 = a.lv[l].nelem <= 0xFFFFFFFFull;
    T* const accb = fold ? reinterpret_cast<T*>(a.accum) + a.lv[l].accum_off +
                             b * a.lv[l].nelem
                         : nullptr;
    // the parent tile lies inside one chunk along every dim: chunk offsets
    // are a tile base plus within-chunk strides (no per-element division)
    bool inchunk = true;
    uint64_t tbase = fixedl;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      inchunk &= a.cs[k] % uint32_t(pe) == 0;
      tbase += uint64_t(porg[k] / a.cs[k]) * a.lv[l].S[k] +
               uint64_t(porg[k] % a.cs[k]) * a.lv[l].s[k];
    }
    const bool off32 = inchunk && a.lv[l].off32;
    for (int i = threadIdx.x; i < pn; i += kTileThreads) {
      uint32_t p[3], in = 1;
      int r = i;
#pragma unroll
      for (int k = D - 1; k >= 0; --k) {
        const int lp = r & (pe - 1);
        p[k] = uint32_t(lp);
        in &= uint32_t(lp) < pext[k];
        r >>= plog;
      }
      if (!in)
        continue;
      // children in Z order of the offset (dim 0 = least significant bit)
      bool full = true;
#pragma unroll
      for (int k = 0; k < D; ++k)
        full &= 2 * p[k] + 1 < cext[k];
      T v;
      if (full) { // every child in bounds: the window stays in registers
        T w[1 << D];
#pragma unroll
        for (int z = 0; z < (1 << D); ++z) {
          int ci = 0;
#pragma unroll
          for (int k = 0; k < D; ++k)
            ci = (ci << elog) + int(2 * p[k] + ((z >> k) & 1));
          w[z] = cur[ci];
        }
        v = reduce_full<T, (1 << D)>(w, a.method);
      } else {
        T win[8];
        int n = 0;
#pragma unroll
        for (int z = 0; z < (1 << D); ++z) {
          int ci = 0;
          bool ok = true;
#pragma unroll
          for (int k = 0; k < D; ++k) {
            const uint32_t c = 2 * p[k] + ((z >> k) & 1);
            ok &= c < cext[k];
            ci = (ci << elog) + int(c);
          }
          if (ok)
            win[n++] = cur[ci];
        }
        v = reduce_window<T>(win, uint64_t(n), a.method);
      }
      int pi = 0;
#pragma unroll
      for (int k = 0; k < D; ++k)
        pi = (pi << plog) + int(p[k]);
      nxt[pi] = v;
      uint32_t gx[3];
#pragma unroll
      for (int k = 0; k < D; ++k)
        gx[k] = porg[k] + p[k];
      uint64_t pos;
      if (off32) {
        uint32_t o = 0;
#pragma unroll
        for (int k = 0; k < D; ++k)
          o += p[k] * s32[k];
        pos = tbase + o;
      } else if (inchunk) {
        pos = tbase;
#pragma unroll
        for (int k = 0; k < D; ++k)
          pos += uint64_t(p[k]) * a.lv[l].s[k];
      } else {
        pos = fixedl + chunk_pos<D>(a, l, gx);
      }
      if (fold) {
        // dense accumulator [fixed][row-major level coords]; its value
        // before this epoch is in the stage
        T* acc;
        if (ai32) {
          uint32_t ai = 0;
#pragma unroll
          for (int k = 0; k < D; ++k)
            ai = ai * shp32[k] + gx[k];
          acc = accb + ai;
        } else {
          uint64_t ai = 0;
#pragma unroll
          for (int k = 0; k < D; ++k)
            ai = ai * a.lv[l].shape[k] + gx[k];
          acc = accb + ai;
        }
        const uint32_t cnt = a.count[l];
        const T av =
          cnt == 0 ? v : fold_one<T>(stage[sbase + i], v, l, a.append_method);
        *acc = av;
        if (emit)
          slot[pos] = emit_one<T>(av, cnt + 1, a.append_method);
      } else if (emit) {
        slot[pos] = v;
      }
    }
    __syncthreads();
    // next level reads nxt: swap
    T* t = cur;
    cur = nxt;
    nxt = t;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      org[k] = porg[k];
      ext[k] = pext[k];
    }
    edge = pe;
    elog = plog;
    sbase += pn;
    __syncthreads();
  }
}

// Emit every element of a dense accumulator level to its chunk positions
// (the dim-0 drain at flush, src/cpu/pipeline.c:414-473).
template<typename T, int D>
__global__ void lod_drain_k(LodTileArgs a, int l, uint32_t count)
{
  const uint64_t n = a.lv[l].nelem * a.fixed_count;
  for (uint64_t g = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; g < n;
       g += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t b = g / a.lv[l].nelem;
    uint64_t r = g - b * a.lv[l].nelem;
    uint32_t x[3];
#pragma unroll
    for (int k = D - 1; k >= 0; --k) {
      x[k] = uint32_t(r % a.lv[l].shape[k]);
      r /= a.lv[l].shape[k];
    }
    const T* acc = reinterpret_cast<const T*>(a.accum) + a.lv[l].accum_off;
    T* slot = reinterpret_cast<T*>(a.slot);
    slot[a.lv[l].chunk_fixed[b] + chunk_pos<D>(a, l, x)] =
      emit_one<T>(acc[g], count, a.append_method);
  }
}

template<typename T, int D>
cudaError_t launch_tile_typed(const LodTileArgs& a, cudaStream_t st)
{
  constexpr int TL = TileGeom<D>::log;
  uint64_t tiles = 1;
  for (int k = 0; k < D; ++k)
    tiles *= a.tiles[k];
  const dim3 grid(unsigned(tiles), unsigned(a.fixed_count));
  const size_t tn = size_t(1) << (D * TL);
  const size_t smem = sizeof(T) * (tn + (tn >> D) + size_t(stage_elems<D>()));
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(lod_tile_k<T, D>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  lod_tile_k<T, D><<<grid, kTileThreads, smem, st>>>(a);
  note_launches(1);
  return cudaGetLastError();
}

template<typename T, int D>
cudaError_t launch_drain_typed(const LodTileArgs& a, int l, uint32_t count,
                               cudaStream_t st)
{
  const uint64_t n = a.lv[l].nelem * a.fixed_count;
  const uint64_t blocks = (n + 255) / 256;
  const uint64_t cap = uint64_t(device_sm_count()) * 16;
  const unsigned grid = unsigned(blocks < cap ? (blocks ? blocks : 1) : cap);
  lod_drain_k<T, D><<<grid, 256, 0, st>>>(a, l, count);
  note_launches(1);
  return cudaGetLastError();
}

template<int D>
cudaError_t launch_tile_d(const LodTileArgs& a, cudaStream_t st)
{
  CHUCKY_DISPATCH_DTYPE(a.dtype, return (launch_tile_typed<T, D>)(a, st));
  return cudaErrorInvalidValue;
}

template<int D>
cudaError_t launch_drain_d(const LodTileArgs& a, int l, uint32_t count,
                           cudaStream_t st)
{
  CHUCKY_DISPATCH_DTYPE(a.dtype,
                        return (launch_drain_typed<T, D>)(a, l, count, st));
  return cudaErrorInvalidValue;
}

} // namespace

int lod_tile_levels(int lod_ndim)
{
  switch (lod_ndim) {
    case 1:
      return TileGeom<1>::log;
    case 2:
      return TileGeom<2>::log;
    case 3:
      return TileGeom<3>::log;
    default:
      return 0;
  }
}

uint32_t lod_tile_edge(int lod_ndim)
{
  const int l = lod_tile_levels(lod_ndim);
  return l ? (1u << l) : 0;
}

cudaError_t launch_lod_tile(const LodTileArgs& a, cudaStream_t st)
{
  switch (a.lod_ndim) {
    case 1:
      return launch_tile_d<1>(a, st);
    case 2:
      return launch_tile_d<2>(a, st);
    case 3:
      return launch_tile_d<3>(a, st);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_lod_drain(const LodTileArgs& a,
                             int level,
                             uint32_t count,
                             cudaStream_t st)
{
  switch (a.lod_ndim) {
    case 1:
      return launch_drain_d<1>(a, level, count, st);
    case 2:
      return launch_drain_d<2>(a, level, count, st);
    case 3:
      return launch_drain_d<3>(a, level, count, st);
    default:
      return cudaErrorInvalidValue;
  }
}

} // namespace chucky
