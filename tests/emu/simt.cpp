// CPU SIMT emulation runtime -- TEST INFRASTRUCTURE ONLY (see simt.hpp).
#include "simt.hpp"

#include <memory>

namespace simt {

thread_local dim3 threadIdx_, blockIdx_;
dim3 blockDim_, gridDim_;
Cta* cta = nullptr;

void fail(const char* what)
{
  std::fprintf(stderr, "simt: %s (block %u thread %u)\n", what, blockIdx_.x,
               threadIdx_.x);
  std::abort();
}

void launch(unsigned grid, unsigned block, const std::function<void()>& body)
{
  if (block == 0 || block % 32 != 0)
    fail("block size must be a multiple of 32");
  blockDim_ = dim3{ block, 1, 1 };
  gridDim_ = dim3{ grid, 1, 1 };
  Cta c;
  std::barrier<> all(block);
  std::vector<std::unique_ptr<std::barrier<>>> warps;
  for (unsigned w = 0; w < block / 32; ++w) {
    warps.emplace_back(new std::barrier<>(32));
    c.warp.push_back(warps.back().get());
  }
  c.all = &all;
  c.slot.assign(block, 0);
  cta = &c;
  // one worker per thread; all CTAs run one after another
  std::barrier<> cta_done(block);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < block; ++t)
    th.emplace_back([&, t] {
      threadIdx_ = dim3{ t, 1, 1 };
      for (unsigned b = 0; b < grid; ++b) {
        blockIdx_ = dim3{ b, 1, 1 };
        body();
        // threads that returned early still take part in later barriers of
        // the CTA: the kernels under test only return whole warps early and
        // never __syncthreads after such a return
        cta_done.arrive_and_wait();
      }
    });
  for (auto& x : th)
    x.join();
  cta = nullptr;
}

} // namespace simt
