// 3x3 convolution of the 2D learned-correction network on the 5th-generation
// tensor cores (tcgen05.mma, accumulator in tensor memory).
//
// Implicit GEMM: D[node][co] = sum_t sum_ci in[node + off_t][ci] * w[co][t][ci],
// M = 128 nodes per tile (8 along x by 16 along y), N = Cout (16..256, a
// multiple of 16), K = 9 taps x Cin (Cin a multiple of 16).
//
// Shared memory holds the operands in the canonical K-major layout without
// swizzle: a "core matrix" is 8 rows of 16 bytes (8 BF16 channels) stored
// contiguously; the leading-dimension byte offset (LBO) steps between core
// matrices along K and the stride-dimension byte offset (SBO) along M (or N).
//   A: the input halo tile of a CTA, 10 x 18 nodes, one "plane" per 8-channel
//      group: plane p holds channels 8p..8p+7 of all 180 halo nodes, node
//      (hx, hy) at row hy * 10 + hx.  The 8 nodes of a tile line are 8
//      consecutive rows, so a core matrix is one tile line and consecutive lines
//      are SBO = 10 rows = 160 bytes apart; the two 8-channel halves of a
//      16-channel K step are LBO = one plane = 2880 bytes apart.  Tap (dx, dy)
//      only moves the start address, by ((dy + 1) * 10 + dx + 1) rows, so the
//      nine taps read one staged tile.  Halo nodes outside the grid are staged
//      as zeros: the zero padding of the convolution.
//   B: all the layer's weights, staged once per CTA: for tap t and 16-channel
//      K step c, two planes (8-channel halves) of Cout rows; SBO = 8 rows =
//      128 bytes (the next 8 output channels), LBO = one plane.
// One thread issues the 9 x Cin/16 MMAs of a tile (M=128, N=Cout, K=16 each,
// BF16 x BF16 -> FP32) and commits them to an mbarrier; the four warps then
// read their 32 accumulator rows (tensor-memory lanes) with tcgen05.ld and
// apply ReLU / the mask and store.  CTAs are persistent over the tiles so the
// weights are staged once.  Every wait is bounded: on a timeout the kernel sets
// *err, skips the rest of its tiles and still frees its tensor memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <stdexcept>
#include <string>

#include "hz_launch.cuh"
#include "hz_learn.h"

namespace hz {

using bf16 = __nv_bfloat16;

namespace {

constexpr int kTcTX = 8, kTcTY = 16;                 // tile: 8 x 16 nodes = M 128
constexpr int kTcHX = kTcTX + 2, kTcHY = kTcTY + 2;  // halo tile
constexpr int kTcRows = kTcHX * kTcHY;               // 180 halo nodes
constexpr int kTcPlane = kTcRows * 16;               // bytes of one 8-channel plane of the halo tile
constexpr int kTcM = 128;
constexpr int kTcHeader = 128;                       // mbarrier + tensor-memory address
constexpr long long kTcSpinLimit = 1LL << 22;        // bounded mbarrier waits
// Shared memory after the operands, so that a reading of the descriptors'
// byte offsets other than the one this kernel assumes (LBO along K, SBO along
// M / N) would still stay inside the allocation: the halo tile comes first,
// then the weights, then this guard band.
constexpr size_t kTcGuard = 40 * 1024;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, LBO and SBO (all >> 4), the
// descriptor version of this architecture (bits 46-47 = 1), no swizzle.
__device__ __forceinline__ unsigned long long sdesc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// BF16 (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// true once the phase with this parity has completed; false after the spin limit
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (long long it = 0; it < kTcSpinLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(unsigned d_tmem, unsigned long long adesc, unsigned long long bdesc,
                                       unsigned idesc, unsigned accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive 32-bit columns of this thread's tensor-memory lane
__device__ __forceinline__ void tc_ld16(unsigned taddr, float (&v)[16]) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

}  // namespace

__global__ void __launch_bounds__(128, 1) k_conv_tc(int nx, int ny, int B, int Cin, int Cout,
                                                    const bf16* __restrict__ in, int ldi, int i_off,
                                                    const bf16* __restrict__ w, bf16* __restrict__ out,
                                                    float* __restrict__ out32, int ldo, int o_off, int relu,
                                                    const bf16* __restrict__ mask, int ldm, int m_off, int mask_lo,
                                                    unsigned tmem_cols, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  unsigned long long* bar_p = reinterpret_cast<unsigned long long*>(tc_smem);
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(tc_smem + 8);
  const int NC = Cin / 16;                       // 16-channel K steps
  const int wplane = Cout * 16;                  // bytes of one weight plane
  unsigned char* sA = tc_smem + kTcHeader;       // 2 * NC halo planes
  unsigned char* sB = sA + 2 * NC * kTcPlane;    // 9 * NC * 2 weight planes
  const unsigned bar = smem_u32(bar_p);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long N = (long long)nx * ny;
  const int tiles_x = (nx + kTcTX - 1) / kTcTX, tiles_y = (ny + kTcTY - 1) / kTcTY;
  const long long tiles = (long long)tiles_x * tiles_y * B;

  if (tid == 0) mbar_init(bar, 1);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // weights: plane ((t * NC + c) * 2 + h), row co = w[co][t][16 c + 8 h .. +8)
  const int wunits = 9 * NC * 2 * Cout;
  for (int u = tid; u < wunits; u += blockDim.x) {
    const int h = u % 2, c = (u / 2) % NC, co = (u / (2 * NC)) % Cout, t = u / (2 * NC * Cout);
    const uint4 v = *reinterpret_cast<const uint4*>(w + ((long long)co * 9 + t) * Cin + 16 * c + 8 * h);
    *reinterpret_cast<uint4*>(sB + ((t * NC + c) * 2 + h) * wplane + co * 16) = v;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;
  const unsigned idesc = idesc_bf16(kTcM, Cout);
  const unsigned aBase = smem_u32(sA), bBase = smem_u32(sB);
  const int aunits = 2 * NC * kTcRows;
  unsigned phase = 0;
  bool ok = true;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const int b = (int)(tile / ((long long)tiles_x * tiles_y));
    const int tr = (int)(tile % ((long long)tiles_x * tiles_y));
    const int x0 = (tr % tiles_x) * kTcTX, y0 = (tr / tiles_x) * kTcTY;
    const bf16* inb = in + (long long)b * N * ldi + i_off;
    // halo tile: unit u = (row r, plane p), planes fastest so a warp reads whole node rows
    for (int u = tid; u < aunits; u += blockDim.x) {
      const int p = u % (2 * NC), r = u / (2 * NC);
      const int x = x0 + r % kTcHX - 1, y = y0 + r / kTcHX - 1;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (x >= 0 && x < nx && y >= 0 && y < ny)
        v = *reinterpret_cast<const uint4*>(inb + ((long long)y * nx + x) * ldi + 8 * p);
      *reinterpret_cast<uint4*>(sA + p * kTcPlane + r * 16) = v;
    }
    fence_async_smem();  // the staged tile is read by the tensor cores (async proxy)
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      for (int t = 0; t < 9; ++t) {
        const int dx = t % 3, dy = t / 3;  // offsets + 1
        for (int c = 0; c < NC; ++c) {
          const unsigned a = aBase + (2 * c) * kTcPlane + (dy * kTcHX + dx) * 16;
          const unsigned bb = bBase + ((t * NC + c) * 2) * wplane;
          tc_mma(tmem, sdesc(a, kTcPlane, kTcHX * 16), sdesc(bb, wplane, 128), idesc, (t | c) != 0);
        }
      }
      tc_commit(bar);
    }
    __syncwarp();
    // every thread waits; the block agrees on the outcome before anyone leaves the loop
    const bool done = mbar_wait(bar, phase);
    if (!__syncthreads_and(done)) {
      ok = false;
      if (tid == 0) {
        atomicExch(err, 1);
        mbar_wait(bar, phase);  // one more bounded wait for MMAs still in flight before the memory is freed
      }
      break;
    }
    phase ^= 1u;
    tc_fence_after();
    // epilogue: this thread's accumulator row is tile row warp * 32 + lane
    const int row = warp * 32 + lane;
    const int x = x0 + row % kTcTX, y = y0 + row / kTcTX;
    const bool in_grid = x < nx && y < ny;
    const long long orow = (long long)b * N + (long long)y * nx + x;
    for (int cb = 0; cb < Cout; cb += 16) {
      float v[16];
      tc_ld16(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)cb, v);
      if (!in_grid) continue;
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int co = cb + k;
        float s = v[k];
        if (relu) s = fmaxf(s, 0.f);
        if (mask && co >= mask_lo && !(__bfloat162float(mask[orow * ldm + m_off + co]) > 0.f)) s = 0.f;
        if (out32)
          out32[orow * ldo + o_off + co] = s;
        else
          out[orow * ldo + o_off + co] = __float2bfloat16_rn(s);
      }
    }
    tc_fence_before();
    __syncthreads();  // accumulator read and halo tile consumed before the next tile reuses them
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols) : "memory");
}

static size_t conv_tc_operands(int Cin, int Cout) {
  return (size_t)kTcHeader + (size_t)9 * (Cin / 16) * 2 * Cout * 16 + (size_t)2 * (Cin / 16) * kTcPlane;
}

static constexpr size_t kTcSmemMax = 227 * 1024;

size_t conv_tc_smem(int Cin, int Cout) {
  return std::min(kTcSmemMax, conv_tc_operands(Cin, Cout) + kTcGuard);
}

bool conv_tc_supported(int Cin, int Cout) {
  return Cin % 16 == 0 && Cin >= 16 && Cout % 16 == 0 && Cout >= 16 && Cout <= 256 &&
         conv_tc_operands(Cin, Cout) <= kTcSmemMax;
}

void conv_tc_launch(Ctx& ctx, const char* name, int nx, int ny, int B, int Cin, const bf16* in, int ldi, int i_off,
                    int Cout, const bf16* w, bf16* out, float* out32, int ldo, int o_off, int relu, const bf16* mask,
                    int ldm, int m_off, int mask_lo, int* err) {
  if (!conv_tc_supported(Cin, Cout)) throw std::runtime_error("conv_tc: unsupported channel counts");
  if ((ldi % 8) || (i_off % 8)) throw std::runtime_error("conv_tc: channel layout not aligned");
  const size_t smem = conv_tc_smem(Cin, Cout);
  static size_t set_bytes[kMaxDevices] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("conv_tc: device ordinal out of range");
  if (set_bytes[dev] < smem) {
    const cudaError_t e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw std::runtime_error(std::string("conv_tc: shared memory attribute: ") + cudaGetErrorString(e));
    }
    set_bytes[dev] = smem;
  }
  unsigned cols = 32;
  while ((int)cols < Cout) cols <<= 1;
  const long long N = (long long)nx * ny;
  const long long tiles = (long long)((nx + kTcTX - 1) / kTcTX) * ((ny + kTcTY - 1) / kTcTY) * B;
  const int grid = (int)std::max<long long>(1, std::min<long long>(tiles, kSMs));
  const double bytes = (double)B * N * (Cin * 2.0 + Cout * (out32 ? 4.0 : 2.0)) + 9.0 * Cin * Cout * 2.0;
  ctx.add_flops(name, 2.0 * 9.0 * Cin * Cout * (double)N * B);
  HZ_LAUNCH(ctx, name, bytes, k_conv_tc, grid, 128, smem, nx, ny, B, Cin, Cout, in, ldi, i_off, w, out, out32, ldo,
            o_off, relu, mask, ldm, m_off, mask_lo, cols, err);
}

}  // namespace hz
