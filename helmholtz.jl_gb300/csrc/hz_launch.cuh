// Internal launch helpers shared by the kernel translation units.
#pragma once

#include <cstdio>
#include <stdexcept>

#include "hz_kernels.cuh"

namespace hz {

static inline void check_launch(const char* name) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[256];
    snprintf(buf, sizeof(buf), "kernel %s launch failed: %s", name, cudaGetErrorString(e));
    throw std::runtime_error(buf);
  }
}

// bytes: the launch's algorithmic DRAM bytes (each input read once, each
// output written once), the numerator of its roofline fraction.
#define HZ_LAUNCH(ctx, name, bytes, kern, grid, block, smem, ...) \
  do {                                                          \
    static thread_local int _id = -1;                           \
    const char* _nm = (name);                                   \
    if (_id < 0 || (size_t)_id >= (ctx).names.size() ||         \
        (ctx).names[_id] != _nm)                                \
      _id = (ctx).name_id(_nm);                                 \
    cudaEvent_t _a = nullptr;                                   \
    (ctx).before(_id, &_a);                                     \
    kern<<<grid, block, smem, (ctx).stream>>>(__VA_ARGS__);     \
    check_launch(_nm);                                          \
    (ctx).after(_id, _a, (double)(bytes));                      \
  } while (0)

static constexpr int kSMs = 152;

// Column chunking: enough CTAs in flight for 152 SMs while each CTA reuses
// its per-node coefficients across as many right-hand sides as possible.
static inline int chunks_for(long long nblk_x, int ncols, int target = 8 * kSMs) {
  long long ch = (target + nblk_x - 1) / nblk_x;
  if (ch < 1) ch = 1;
  if (ch > ncols) ch = ncols;
  return (int)ch;
}

}  // namespace hz
