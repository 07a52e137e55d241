// 3x3 (2D) and 3x3x3 (3D) convolutions of the learned-correction networks on the
// 5th-generation tensor cores (tcgen05.mma, accumulator in tensor memory),
// operands staged by the tensor memory accelerator (cp.async.bulk.tensor).
//
// Implicit GEMM: D[node][co] = sum_t sum_ci in[node + off_t][ci] * w[co][t][ci],
// M = 128 nodes per tile (8 along x by 16 along y of one z-plane), N = Cout
// (16..256, a multiple of 16; the first Cst <= Cout channels are stored), K =
// taps x Cin (9 or 27 taps, Cin a multiple of 16).
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
//      nine taps read one staged tile.  In 3D the halo tile holds three such
//      z-planes (z - 1, z, z + 1) one after the other and tap dz moves the
//      start address by whole z-planes.
//   B: all the layer's weights, staged once per CTA: for tap t and 8-channel
//      group p, one plane of Cout rows (row co = w[co][t][8p .. 8p + 8));
//      SBO = 8 rows = 128 bytes (the next 8 output channels), LBO = one plane.
// The weights reach shared memory as one image in exactly the layout of B
// (k_tc_wimage writes it once per weight update, or per backward convolution
// for the flipped weights), copied by the TMA unit's bulk engine
// (cp.async.bulk, 1-D, 32 KiB per copy).  A z-plane of the halo tile is one TMA
// tensor load: the activation tensor [B][N][ldi] is described to the TMA unit
// as the 5-D tensor (8 channels, x, y, plane, z + nz * batch) with the plane
// dimension (stride 16 bytes) ordered after y, so that one box of
// (8, 10, 18, Cin / 8, 1) lands plane after plane exactly as A above; halo nodes
// outside the grid are filled with zeros by the TMA unit, which is the zero
// padding of the convolution (a z-plane outside the grid is loaded from
// coordinate -1: all zeros).
//
// Warp-specialised persistent CTAs: a producer thread keeps up to four halo
// buffers in flight, an MMA thread issues the taps x Cin / 16 MMAs of a tile into
// one of two tensor-memory accumulators as soon as its halo has landed and the
// accumulator is free, and four epilogue warps read the other accumulator out
// (tcgen05.ld, ReLU / mask, BF16 or FP32 stores); the roles hand buffers to one
// another through mbarriers only, so the loads, MMAs and epilogues of
// consecutive tiles overlap.  Every wait is bounded: on a timeout the kernel
// sets *err and a shared abort flag, the roles leave their loops, wait (again
// bounded) for their copies and MMAs in flight, and the tensor memory is freed.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
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
constexpr int kTcHeader = 128;                       // mbarriers + tensor-memory address
constexpr int kTcAlign = 128;                        // TMA destinations start on 128-byte boundaries
constexpr long long kTcSpinLimit = 1LL << 22;        // bounded mbarrier waits
constexpr size_t kTcSmemMax = 227 * 1024;

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

// arrive on the barrier and add the bytes the copies of this phase will deliver
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// 1-D bulk copy global -> shared on the TMA unit: 16-byte aligned, size a multiple of 16
__device__ __forceinline__ void bulk_load(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(src)), "r"(bytes), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tma_load_5d(unsigned dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            int c4, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

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

__device__ __forceinline__ unsigned pack_bf16x2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const unsigned*>(&h);
}

// a tile: 8 x 16 nodes of plane zb = b * nz + z (z = 0 and zb = b on a 2D grid)
struct TileCoord {
  int zb, x0, y0;
};

__device__ __forceinline__ TileCoord tile_coord(long long tile, int tiles_x, int tiles_y) {
  const long long per = (long long)tiles_x * tiles_y;
  const int tr = (int)(tile % per);
  return {(int)(tile / per), (tr % tiles_x) * kTcTX, (tr / tiles_x) * kTcTY};
}

}  // namespace

// One row of the weight image per thread: row (t * Cin / 8 + p) * Cout + co holds
// W[co][t][8p .. 8p + 8) of the convolution's weights W [Cout][taps][Cin], where
//   flip = 0: W[co][t][ci] = co < wcout ? w[co][t][ci] : 0 for w [wcout][taps][Cin];
//   flip = 1: W[co][t][ci] = ci < wcout ? w[ci][taps - 1 - t][co] : 0 for w [wcout][taps][wcin]
//             (wcin = Cout): the transposed, flipped weights of the data gradient.
__global__ void k_tc_wimage(int taps, int Cin, int Cout, const bf16* __restrict__ w, int flip, int wcin, int wcout,
                            bf16* __restrict__ img) {
  const int NP = Cin / 8;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= taps * NP * Cout) return;
  const int co = idx % Cout, p = (idx / Cout) % NP, t = idx / (Cout * NP);
  alignas(16) bf16 v[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int ci = 8 * p + e;
    if (!flip)
      v[e] = co < wcout ? w[((long long)co * taps + t) * Cin + ci] : __float2bfloat16_rn(0.f);
    else
      v[e] = ci < wcout ? w[((long long)ci * taps + (taps - 1 - t)) * wcin + co] : __float2bfloat16_rn(0.f);
  }
  reinterpret_cast<uint4*>(img)[idx] = *reinterpret_cast<const uint4*>(v);
}

// Shared memory (from a 128-byte aligned base): header (mbarriers and the
// tensor-memory address), weights (taps * Cin / 8 planes of Cout * 16 bytes),
// then nbuf halo buffers of nzp z-planes (1 in 2D, 3 in 3D) of Cin / 8 planes
// each.  taps = 9 (2D) or 27 (3D, tap t = 9 (dz + 1) + 3 (dy + 1) + dx + 1); a
// 3D halo loads its three z-planes as three TMA boxes, a plane outside the grid
// from coordinate -1 (all zero fill).  Cst <= Cout output channels are stored
// (Cout is the MMA's N, a multiple of 16; Cst a multiple of 8).
// Warp roles (192 threads): warps 0-3 epilogue (warp w reads tensor-memory lanes
// 32 w .. 32 w + 31, tile rows of the same numbers), warp 4 lane 0 TMA
// producer, warp 5 lane 0 MMA issuer.  Barriers:
//   wbar        weights landed (TMA bytes)
//   full[s]     halo buffer s landed (TMA bytes)         producer -> MMA
//   empty[s]    halo buffer s read by its MMAs (commit)  MMA -> producer
//   accf[a]     accumulator a complete (commit)          MMA -> epilogue
//   acce[a]     accumulator a read out (4 warp arrivals) epilogue -> MMA
// The k-th use of a stage waits its "full" barrier with parity k & 1 and, from
// the second use on, its "empty" barrier with parity (k - 1) & 1.
constexpr int kTcMaxBuf = 4;
constexpr int kTcThreads = 192;

__global__ void __launch_bounds__(kTcThreads, 2)
    k_conv_tc(const __grid_constant__ CUtensorMap tin, int i_off, int nx, int ny, int nz, int B, int zl, int y0z,
              int tiles_x, int tiles_l, int taps, int Cin, int Cout, int Cst, int nbuf, const bf16* __restrict__ wimg,
              bf16* __restrict__ out, float* __restrict__ out32, int ldo, int o_off, int relu,
              const bf16* __restrict__ mask, int ldm, int m_off, int mask_lo, unsigned acc_cols,
              int* __restrict__ err) {
  extern __shared__ unsigned char tc_raw[];
  unsigned char* smem = tc_raw + ((kTcAlign - (smem_u32(tc_raw) & (kTcAlign - 1))) & (kTcAlign - 1));
  const unsigned base = smem_u32(smem);
  const unsigned wbar = base;
  const unsigned full0 = base + 8, empty0 = full0 + 8 * kTcMaxBuf;  // [s] at + 8 s
  const unsigned accf0 = empty0 + 8 * kTcMaxBuf, acce0 = accf0 + 16;  // [a] at + 8 a
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(smem + 112);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 116);
  const int NP = Cin / 8;                          // 8-channel planes (2 per 16-channel K step)
  const unsigned wplane = (unsigned)Cout * 16;     // bytes of one weight plane
  const unsigned wbytes = (unsigned)taps * NP * wplane;
  const unsigned bBase = base + kTcHeader;
  const unsigned aBase = bBase + wbytes;           // 128-byte aligned: wplane is a multiple of 256
  const int nzp = taps == 27 ? 3 : 1;              // z-planes (y-planes with z-lines) of a halo tile
  // one 8-channel plane of a halo plane: 2880 bytes written by one box (y-lines), or
  // 2944 (128-byte aligned destinations of the per-plane boxes of the z-lines)
  const unsigned pitch = zl ? (unsigned)(kTcPlane + 64) : (unsigned)kTcPlane;
  const unsigned zBytes = (unsigned)NP * pitch;     // a multiple of 128 (NP is even)
  const unsigned tileBytes = (unsigned)nzp * NP * kTcPlane;
  const unsigned abuf = (nzp * zBytes + kTcAlign - 1) / kTcAlign * kTcAlign;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long Nxy = (long long)nx * ny;
  const int nyz = ny - y0z;                          // y-rows of the z-line tiles
  const long long tiles = (long long)tiles_x * tiles_l * (zl ? (long long)nyz * B : (long long)nz * B);
  const int n = tiles > blockIdx.x ? (int)((tiles - blockIdx.x + gridDim.x - 1) / gridDim.x) : 0;

  if (tid == 0) {
    mbar_init(wbar, 1);
    for (int s = 0; s < kTcMaxBuf; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(accf0 + 8 * a, 1);
      mbar_init(acce0 + 8 * a, 4);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_async_smem();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * acc_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;
  auto give_up = [&]() {
    *abort_flag = 1;
    atomicExch(err, 1);
  };

  if (warp == 4) {
    if (lane == 0) {
      // producer: weights once, then the halo of every tile
      mbar_expect_tx(wbar, wbytes);
      for (unsigned o = 0; o < wbytes; o += 32768u)
        bulk_load(bBase + o, reinterpret_cast<const unsigned char*>(wimg) + o, min(32768u, wbytes - o), wbar);
      int j = 0;
      for (; j < n && !*abort_flag; ++j) {
        const int s = j % nbuf, k = j / nbuf;
        if (k >= 1 && !mbar_wait(empty0 + 8 * s, (unsigned)(k - 1) & 1u)) {
          give_up();
          break;
        }
        const TileCoord tc = tile_coord(blockIdx.x + (long long)j * gridDim.x, tiles_x, tiles_l);
        mbar_expect_tx(full0 + 8 * s, tileBytes);
        if (!zl) {
          // y-lines: one box per z-plane over (8 channels, x, y, plane, z + nz * batch)
          const int z = tc.zb % nz;
          for (int q = 0; q < nzp; ++q) {
            const int dz = nzp == 3 ? q - 1 : 0;
            const int zc = (z + dz >= 0 && z + dz < nz) ? tc.zb + dz : -1;  // -1: a plane of zeros
            tma_load_5d(aBase + (unsigned)s * abuf + (unsigned)q * zBytes, &tin, 0, tc.x0 - 1, tc.y0 - 1, i_off / 8,
                        zc, full0 + 8 * s);
          }
        } else {
          // z-lines: one box per y-plane and 8-channel plane over (channels, x, z, y, batch);
          // a y outside the grid reads zeros
          const int y = y0z + tc.zb % nyz, b = tc.zb / nyz;
          for (int q = 0; q < nzp; ++q)
            for (int p = 0; p < NP; ++p)
              tma_load_5d(aBase + (unsigned)s * abuf + (unsigned)q * zBytes + (unsigned)p * pitch, &tin, i_off + 8 * p,
                          tc.x0 - 1, tc.y0 - 1, y + q - 1, b, full0 + 8 * s);
        }
      }
      if (*abort_flag) {
        // bounded waits for the copies still in flight: the weights and the last nbuf halo loads
        mbar_wait(wbar, 0);
        for (int q = max(0, j - nbuf); q < j; ++q) mbar_wait(full0 + 8 * (q % nbuf), (unsigned)(q / nbuf) & 1u);
      }
    }
  } else if (warp == 5) {
    if (lane == 0) {
      // MMA issuer: M = 128 tile rows, N = Cout, K = 16 per instruction, 9 * Cin / 16 instructions per tile
      const unsigned idesc = idesc_bf16(kTcM, Cout);
      int committed = -1;
      if (!mbar_wait(wbar, 0)) give_up();
      for (int j = 0; j < n && !*abort_flag; ++j) {
        const int s = j % nbuf, a = j & 1;
        if (!mbar_wait(full0 + 8 * s, (unsigned)(j / nbuf) & 1u) ||
            (j >= 2 && !mbar_wait(acce0 + 8 * a, (unsigned)((j >> 1) - 1) & 1u))) {
          give_up();
          break;
        }
        tc_fence_after();
        const unsigned acc = tmem + (unsigned)a * acc_cols;
        const unsigned long long a0 = sdesc(aBase + (unsigned)s * abuf, pitch, kTcHX * 16);
        const unsigned long long b0 = sdesc(bBase, wplane, 128);
        for (int t = 0; t < taps; ++t) {
          // halo plane and row offset of tap t, bytes: the planes run along z and the
          // lines along y, or (z-lines) the planes along y and the lines along z
          const int tz = t / 9, ty = (t / 3) % 3;
          const unsigned tap =
              (unsigned)(zl ? ty : tz) * zBytes + (unsigned)(((zl ? tz : ty) * kTcHX + t % 3) * 16);
          for (int c = 0; c < NP / 2; ++c) {
            const unsigned aoff = (2u * c * pitch + tap) >> 4, boff = ((unsigned)(t * NP + 2 * c) * wplane) >> 4;
            tc_mma(acc, a0 + aoff, b0 + boff, idesc, (t | c) != 0);
          }
        }
        tc_commit(empty0 + 8 * s);  // halo buffer s free once these MMAs have read it
        tc_commit(accf0 + 8 * a);   // accumulator a ready for the epilogue
        committed = j;
      }
      if (*abort_flag && committed >= 0)
        mbar_wait(accf0 + 8 * (committed & 1), (unsigned)(committed >> 1) & 1u);
    }
  } else {
    // epilogue warps 0-3: this thread's accumulator row is tile row warp * 32 + lane
    for (int j = 0; j < n; ++j) {
      const int a = j & 1;
      const bool done = __all_sync(0xffffffffu, mbar_wait(accf0 + 8 * a, (unsigned)(j >> 1) & 1u));
      if (!done) {
        if (lane == 0) give_up();
        break;
      }
      tc_fence_after();
      const TileCoord tc = tile_coord(blockIdx.x + (long long)j * gridDim.x, tiles_x, tiles_l);
      const int row = warp * 32 + lane;
      const int x = tc.x0 + row % kTcTX, l = tc.y0 + row / kTcTX;  // l: y, or z with z-lines
      bool in_grid;
      long long orow;
      if (!zl) {
        in_grid = x < nx && l < ny;
        orow = (long long)tc.zb * Nxy + (long long)l * nx + x;
      } else {
        const int y = y0z + tc.zb % nyz, b = tc.zb / nyz;
        in_grid = x < nx && l < nz;
        orow = ((long long)b * nz + l) * Nxy + (long long)y * nx + x;
      }
      const unsigned acc = tmem + (unsigned)a * acc_cols + ((unsigned)(warp * 32) << 16);
      for (int cb = 0; cb < Cout; cb += 16) {
        float v[16];
        tc_ld16(acc + (unsigned)cb, v);
        if (!in_grid || cb >= Cst) continue;
        const bool half = cb + 16 > Cst;  // 8 channels stored from this chunk
        if (relu) {
#pragma unroll
          for (int k = 0; k < 16; ++k) v[k] = fmaxf(v[k], 0.f);
        }
        if (mask && cb >= mask_lo) {
          const uint4* mp = reinterpret_cast<const uint4*>(mask + orow * ldm + m_off + cb);
          const uint4 m2[2] = {mp[0], half ? make_uint4(0u, 0u, 0u, 0u) : mp[1]};
          const bf16* mh = reinterpret_cast<const bf16*>(m2);
#pragma unroll
          for (int k = 0; k < 16; ++k)
            if (!(__bfloat162float(mh[k]) > 0.f)) v[k] = 0.f;
        }
        if (out32) {
          float4* op = reinterpret_cast<float4*>(out32 + orow * ldo + o_off + cb);
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (q < 2 || !half) op[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        } else {
          uint4* op = reinterpret_cast<uint4*>(out + orow * ldo + o_off + cb);
          op[0] = make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]), pack_bf16x2(v[4], v[5]),
                             pack_bf16x2(v[6], v[7]));
          if (!half)
            op[1] = make_uint4(pack_bf16x2(v[8], v[9]), pack_bf16x2(v[10], v[11]), pack_bf16x2(v[12], v[13]),
                               pack_bf16x2(v[14], v[15]));
        }
      }
      // accumulator a read out: one arrival per warp
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce0 + 8 * a);
      if (*abort_flag) break;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * acc_cols) : "memory");
}

namespace {

size_t tc_weights(int taps, int Cin, int Cout) { return (size_t)taps * (Cin / 8) * Cout * 16; }
// a halo buffer: 3D tiles use the z-lines' plane pitch (2944 bytes) in either mode
size_t tc_halo(int taps, int Cin) {
  return taps == 27 ? (size_t)3 * (Cin / 8) * (kTcPlane + 64)
                    : ((size_t)(Cin / 8) * kTcPlane + kTcAlign - 1) / kTcAlign * kTcAlign;
}
size_t tc_smem(int taps, int Cin, int Cout, int nbuf) {
  return (size_t)kTcAlign + kTcHeader + tc_weights(taps, Cin, Cout) + (size_t)nbuf * tc_halo(taps, Cin);
}
unsigned tc_cols(int Cout) {
  unsigned cols = 32;
  while ((int)cols < Cout) cols <<= 1;
  return cols;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, looked up once through the runtime
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  if (!fn) throw std::runtime_error("conv_tc: cuTensorMapEncodeTiled is not available");
  return fn;
}

void encode(CUtensorMap* map, const void* ptr, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
            const cuuint32_t* box, const char* what) {
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = encode_tiled()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(ptr),
                                    dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error(std::string("conv_tc: tensor map of the ") + what + " rejected");
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

bool conv_tc_supported(int taps, int Cin, int Cout) {
  return (taps == 9 || taps == 27) && Cin % 16 == 0 && Cin >= 16 && Cin <= 256 && Cout % 16 == 0 && Cout >= 16 &&
         Cout <= 256 && tc_smem(taps, Cin, Cout, 1) <= kTcSmemMax;
}

void conv_tc_weight_image(Ctx& ctx, const char* name, int taps, int Cin, int Cout, const bf16* w, int flip, int wcin,
                          int wcout, bf16* img) {
  if (!conv_tc_supported(taps, Cin, Cout)) throw std::runtime_error("conv_tc: unsupported channel counts");
  if (flip ? (wcin != Cout || wcout > Cin) : wcout > Cout)
    throw std::runtime_error("conv_tc: weights of another shape");
  if (!aligned16(img)) throw std::runtime_error("conv_tc: weight image not aligned to 16 bytes");
  const int rows = taps * (Cin / 8) * Cout;
  HZ_LAUNCH(ctx, name, (double)rows * 32.0, k_tc_wimage, (unsigned)((rows + 255) / 256), 256, 0, taps, Cin, Cout, w,
            flip, wcin, wcout, img);
}

void conv_tc_launch(Ctx& ctx, const char* name, const ConvTc& a, int* err) {
  const int taps = a.nz > 1 ? 27 : 9;
  const int Cin = a.Cin, Cout = a.Cout;
  if (a.taps3d != (taps == 27)) throw std::runtime_error("conv_tc: a 3D convolution needs a grid with nz > 1");
  if (!conv_tc_supported(taps, Cin, Cout)) throw std::runtime_error("conv_tc: unsupported channel counts");
  if (a.Cst < 8 || a.Cst > Cout || a.Cst % 8) throw std::runtime_error("conv_tc: stored channels out of range");
  if (a.ldi % 8 || a.i_off % 8 || a.i_off + Cin > a.ldi || !aligned16(a.in) || !aligned16(a.wimg))
    throw std::runtime_error("conv_tc: input or weight layout not aligned to 16 bytes");
  if (a.out32 ? (a.ldo % 4 || a.o_off % 4 || !aligned16(a.out32)) : (a.ldo % 8 || a.o_off % 8 || !aligned16(a.out)))
    throw std::runtime_error("conv_tc: output layout not aligned to 16 bytes");
  if (a.mask && (a.mask_lo % 16 || a.ldm % 8 || a.m_off % 8 || !aligned16(a.mask)))
    throw std::runtime_error("conv_tc: mask layout not aligned to 16 bytes");
  if (a.o_off + a.Cst > a.ldo || (a.mask && a.m_off + a.Cst > a.ldm))
    throw std::runtime_error("conv_tc: channel offset beyond the row");
  if (a.nx < 1 || a.ny < 1 || a.nz < 1 || a.B < 1) throw std::runtime_error("conv_tc: empty grid");

  static std::mutex mu;
  static bool attr_set[kMaxDevices] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("conv_tc: device ordinal out of range");
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!attr_set[dev]) {
      // the largest shared-memory carveout, so that the CTAs counted below stay resident
      cudaError_t e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemMax);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("conv_tc: shared memory attribute: ") + cudaGetErrorString(e));
      }
      attr_set[dev] = true;
    }
  }
  // y-line tiles: activations [B][nz][ny][nx][ldi] as (8 channels, x, y, plane, z + nz * batch), plane after y
  alignas(64) CUtensorMap tin = {};
  {
    const cuuint64_t dims[5] = {8, (cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)(a.ldi / 8),
                                (cuuint64_t)a.nz * a.B};
    const cuuint64_t strides[4] = {(cuuint64_t)a.ldi * 2, (cuuint64_t)a.nx * a.ldi * 2, 16,
                                   (cuuint64_t)a.nx * a.ny * a.ldi * 2};
    const cuuint32_t box[5] = {8, kTcHX, kTcHY, (cuuint32_t)(Cin / 8), 1};
    encode(&tin, a.in, 5, dims, strides, box, "activations");
  }
  // 3D: full y-tiles on y-lines, the remaining y-rows of each plane (ny % 16 of
  // them, one on the 2^k + 1-node grids) on z-line tiles, 16 lines along z, over
  // the activations as (channels, x, z, y, batch)
  const int y0z = taps == 27 ? a.ny / kTcTY * kTcTY : a.ny;
  alignas(64) CUtensorMap tinz = {};
  if (y0z < a.ny) {
    const cuuint64_t dims[5] = {(cuuint64_t)a.ldi, (cuuint64_t)a.nx, (cuuint64_t)a.nz, (cuuint64_t)a.ny,
                                (cuuint64_t)a.B};
    const cuuint64_t strides[4] = {(cuuint64_t)a.ldi * 2, (cuuint64_t)a.nx * a.ny * a.ldi * 2,
                                   (cuuint64_t)a.nx * a.ldi * 2, (cuuint64_t)a.nx * a.ny * a.nz * a.ldi * 2};
    const cuuint32_t box[5] = {8, kTcHX, kTcHY, 1, 1};
    encode(&tinz, a.in, 5, dims, strides, box, "activations (z-lines)");
  }
  // Halo buffers and CTAs per SM.  CTAs per SM come from the kernel's footprint
  // against the SM's shared memory, registers, threads and tensor memory (512
  // columns); the runtime's occupancy query reports one CTA per SM for this
  // kernel at every shared-memory size, so it is not used.  Buffers: the most
  // CTAs per SM with at least two buffers each, then the most buffers (up to
  // four) at that count; one buffer only when two do not fit.
  const unsigned cols = tc_cols(Cout);
  static int sm_smem[kMaxDevices] = {}, sm_regs[kMaxDevices] = {}, blk_resv[kMaxDevices] = {}, k_regs[kMaxDevices] = {};
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!sm_smem[dev]) {
      cudaFuncAttributes fa{};
      if (cudaDeviceGetAttribute(&sm_smem[dev], cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&sm_regs[dev], cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&blk_resv[dev], cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
          cudaFuncGetAttributes(&fa, k_conv_tc) != cudaSuccess) {
        cudaGetLastError();
        sm_smem[dev] = 0;
        throw std::runtime_error("conv_tc: device or kernel attributes unavailable");
      }
      k_regs[dev] = fa.numRegs;
    }
  }
  const long long warp_regs = ((long long)k_regs[dev] * 32 + 255) / 256 * 256;  // allocated per warp in 256s
  auto ctas_per_sm = [&](int nb) {
    return (int)std::max<long long>(
        1, std::min<long long>({(long long)sm_smem[dev] / ((long long)tc_smem(taps, Cin, Cout, nb) + blk_resv[dev]),
                                (long long)sm_regs[dev] / (warp_regs * (kTcThreads / 32)), 2048 / kTcThreads,
                                512 / (2 * (long long)cols)}));
  };
  int nbuf = 1, per_sm = ctas_per_sm(1);
  for (int nb = 2; nb <= kTcMaxBuf && tc_smem(taps, Cin, Cout, nb) <= kTcSmemMax; ++nb) {
    const int k = ctas_per_sm(nb);
    if (nb == 2 || k >= per_sm) {
      nbuf = nb;
      per_sm = k;
    }
  }
  const size_t smem = tc_smem(taps, Cin, Cout, nbuf);
  // tiles of 8 x 16 nodes per plane; partial tiles at the grid's edges (TMA zero fill, stores masked)
  const int tiles_x = (a.nx + kTcTX - 1) / kTcTX;
  const long long N = (long long)a.nx * a.ny * a.nz;
  const double bytes = (double)N * a.B * (Cin * 2.0 + a.Cst * (a.out32 ? 4.0 : 2.0)) + (double)taps * Cin * Cout * 2.0;
  ctx.add_flops(name, 2.0 * taps * Cin * a.Cst * (double)N * a.B);
  if (y0z > 0) {
    const int tiles_y = (y0z + kTcTY - 1) / kTcTY;
    const long long tiles = (long long)tiles_x * tiles_y * a.nz * a.B;
    const int grid = (int)std::min<long long>(tiles, (long long)kSMs * per_sm);
    HZ_LAUNCH(ctx, name, bytes * y0z / a.ny, k_conv_tc, grid, kTcThreads, smem, tin, a.i_off, a.nx, a.ny, a.nz, a.B,
              0, 0, tiles_x, tiles_y, taps, Cin, Cout, a.Cst, nbuf, a.wimg, a.out, a.out32, a.ldo, a.o_off, a.relu,
              a.mask, a.ldm, a.m_off, a.mask_lo, cols, err);
  }
  if (y0z < a.ny) {
    const int tiles_z = (a.nz + kTcTY - 1) / kTcTY;
    const long long tiles = (long long)tiles_x * tiles_z * (a.ny - y0z) * a.B;
    const int grid = (int)std::min<long long>(tiles, (long long)kSMs * per_sm);
    const std::string zn = std::string(name) + "_zlines";
    HZ_LAUNCH(ctx, zn.c_str(), bytes * (a.ny - y0z) / a.ny, k_conv_tc, grid, kTcThreads, smem, tinz, a.i_off, a.nx,
              a.ny, a.nz, a.B, 1, y0z, tiles_x, tiles_z, taps, Cin, Cout, a.Cst, nbuf, a.wimg, a.out, a.out32, a.ldo,
              a.o_off, a.relu, a.mask, a.ldm, a.m_off, a.mask_lo, cols, err);
  }
}

// ---------------------------------------------------------------------------
// Weight gradient on the tensor cores:
//   dW[co][t][ci] += sum_n dout[n][co] * in[n + off_t][ci]
// a GEMM per tap with M = 128 rows (co, zero rows beyond Cout), N = Cin and
// K = the nodes, in slices of 64 nodes.  A CTA owns one tap (blockIdx.z) and a
// range of nodes (blockIdx.y).  Both operands take the K-major layout without
// swizzle of the convolution kernel (core matrix = 8 rows x 8 nodes of 16 bytes):
// each thread loads an 8-node x 8-channel block (8 rows of 16 bytes from
// global memory; zeros where the tap leaves the grid or the range ends),
// transposes it in registers (byte permutes) and stores its 8 channel rows as
// one core matrix.  Two staging buffers: the block stages slice s + 1 while the
// tensor cores run the four MMAs (K = 16 nodes each) of slice s.  The FP32
// accumulator (128 lanes x Cin columns of tensor memory) is added to dW with one
// atomic per weight at the end.  Every wait is bounded (err, as above).  The
// staging (a transpose of every node row, per tap) bounds it: measured slower
// than the warp-level kernels, which the default path keeps.
constexpr int kWgNodes = 64;  // nodes per slice (K)

__device__ __forceinline__ unsigned prmt(unsigned a, unsigned b, unsigned sel) {
  unsigned r;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
  return r;
}

// out[r] holds channel r of the 8 nodes of v (node 2i in the low half of word i)
__device__ __forceinline__ void transpose8x8(const uint4 (&v)[8], uint4 (&out)[8]) {
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const unsigned sel = (r & 1) ? 0x7632u : 0x5410u;
    unsigned w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint4& a = v[2 * i];
      const uint4& b = v[2 * i + 1];
      const int q = r >> 1;
      const unsigned wa = q == 0 ? a.x : q == 1 ? a.y : q == 2 ? a.z : a.w;
      const unsigned wb = q == 0 ? b.x : q == 1 ? b.y : q == 2 ? b.z : b.w;
      w[i] = prmt(wa, wb, sel);
    }
    out[r] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__global__ void __launch_bounds__(128) k_wgrad_tc(int nx, int ny, int nz, long long nodes, int taps, int Cin,
                                                  const bf16* __restrict__ in, int ldi, int Cout,
                                                  const bf16* __restrict__ dout, int ldd, int d_off,
                                                  float* __restrict__ dw, long long kc, unsigned acc_cols,
                                                  int* __restrict__ err) {
  extern __shared__ unsigned char wg_raw[];
  unsigned char* smem = wg_raw + ((kTcAlign - (smem_u32(wg_raw) & (kTcAlign - 1))) & (kTcAlign - 1));
  const unsigned base = smem_u32(smem);
  const unsigned mbar0 = base;  // mma[b] at + 8 b
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(smem + 16);
  const int GA = Cout / 8, GB = Cin / 8;           // 8-channel groups of the two operands
  const unsigned aBytes = 16u * 8u * 128u;         // M = 128 rows x 64 nodes
  const unsigned bBytes = (unsigned)GB * 8u * 128u;
  const unsigned buf0 = base + kTcHeader;           // buffer b: A at buf0 + b (aBytes + bBytes), then B
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int t = blockIdx.z;
  const int dz = taps == 27 ? t / 9 - 1 : 0, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
  const long long off = dx + (long long)dy * nx + (long long)dz * nx * ny;
  const long long n0 = (long long)blockIdx.y * kc;
  const long long n1 = min(nodes, n0 + kc);
  const int ns = n1 > n0 ? (int)((n1 - n0 + kWgNodes - 1) / kWgNodes) : 0;

  if (tid == 0) {
    mbar_init(mbar0, 1);
    mbar_init(mbar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the rows of A beyond Cout stay zero: clear both buffers once
  for (unsigned o = tid * 16u; o < 2u * (aBytes + bBytes); o += 128u * 16u)
    *reinterpret_cast<uint4*>(smem + kTcHeader + o) = make_uint4(0u, 0u, 0u, 0u);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(acc_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;
  const unsigned idesc = idesc_bf16(kTcM, Cin);
  const long long Nxy = (long long)nx * ny;
  bool ok = true;
  int issued = 0;  // slices whose MMAs thread 0 committed
  for (int s = 0; s < ns && ok; ++s) {
    const int b = s & 1;
    // buffer b was last read by the MMAs of slice s - 2
    if (s >= 2) ok = mbar_wait(mbar0 + 8 * b, (unsigned)((s - 2) >> 1) & 1u);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    const unsigned aB = buf0 + (unsigned)b * (aBytes + bBytes), bB = aB + aBytes;
    const long long ns0 = n0 + (long long)s * kWgNodes;
    for (int task = tid; task < 8 * (GA + GB); task += blockDim.x) {
      const int kg = task % 8, gi = task / 8;
      const bool isA = gi < GA;
      const int g = isA ? gi : gi - GA;
      uint4 v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const long long n = ns0 + kg * 8 + j;
        v[j] = make_uint4(0u, 0u, 0u, 0u);
        if (n < n1) {
          if (isA) {
            v[j] = *reinterpret_cast<const uint4*>(dout + n * ldd + d_off + 8 * g);
          } else {
            const int x = (int)(n % nx), y = (int)((n / nx) % ny), z = (int)((n / Nxy) % nz);
            if (x + dx >= 0 && x + dx < nx && y + dy >= 0 && y + dy < ny && z + dz >= 0 && z + dz < nz)
              v[j] = *reinterpret_cast<const uint4*>(in + (n + off) * ldi + 8 * g);
          }
        }
      }
      uint4 w[8];
      transpose8x8(v, w);
      unsigned char* dst = smem + ((isA ? aB : bB) - base) + (unsigned)(kg * (isA ? 16 : GB) + g) * 128u;
#pragma unroll
      for (int r = 0; r < 8; ++r) *reinterpret_cast<uint4*>(dst + r * 16) = w[r];
    }
    fence_async_smem();  // the staged slice is read by the tensor cores (async proxy)
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const unsigned long long a0 = sdesc(aB, 16u * 128u, 128u);        // LBO: next 8 nodes, SBO: next 8 rows
      const unsigned long long b0 = sdesc(bB, (unsigned)GB * 128u, 128u);
#pragma unroll
      for (int q = 0; q < kWgNodes / 16; ++q)
        tc_mma(tmem, a0 + ((2u * q * 16u * 128u) >> 4), b0 + ((2u * q * GB * 128u) >> 4), idesc, (s | q) != 0);
      tc_commit(mbar0 + 8 * b);
      ++issued;
    }
  }
  // the last slice's MMAs (the commit tracks all earlier ones too)
  bool done = true;
  if (ok && ns > 0) done = mbar_wait(mbar0 + 8 * ((ns - 1) & 1), (unsigned)((ns - 1) >> 1) & 1u);
  done = __syncthreads_and(done && ok);
  if (!done) {
    if (tid == 0) {
      atomicExch(err, 1);
      if (issued > 0) mbar_wait(mbar0 + 8 * ((issued - 1) & 1), (unsigned)((issued - 1) >> 1) & 1u);
    }
  } else if (ns > 0) {
    tc_fence_after();
    // epilogue: this thread's accumulator row is co = warp * 32 + lane
    const int co = warp * 32 + lane;
    for (int cb = 0; cb < Cin; cb += 16) {
      float v[16];
      tc_ld16(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)cb, v);
      if (co < Cout) {
#pragma unroll
        for (int k = 0; k < 16; ++k) atomicAdd(&dw[((long long)co * taps + t) * Cin + cb + k], v[k]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(acc_cols) : "memory");
}

bool wgrad_tc_supported(int taps, int Cin, int Cout) {
  return (taps == 9 || taps == 27) && Cin % 16 == 0 && Cin >= 16 && Cin <= 128 && Cout % 8 == 0 && Cout >= 8 &&
         Cout <= 128;
}

void wgrad_tc_launch(Ctx& ctx, const char* name, const WgradTc& a, int* err) {
  const int taps = a.nz > 1 ? 27 : 9;
  if (!wgrad_tc_supported(taps, a.Cin, a.Cout)) throw std::runtime_error("wgrad_tc: unsupported channel counts");
  if (a.ldi % 8 || a.ldd % 8 || a.d_off % 8 || a.d_off + a.Cout > a.ldd || a.Cin > a.ldi || !aligned16(a.in) ||
      !aligned16(a.dout))
    throw std::runtime_error("wgrad_tc: layout not aligned to 16 bytes");
  if (a.nodes < 1 || a.nodes % ((long long)a.nx * a.ny * a.nz)) throw std::runtime_error("wgrad_tc: node count");
  const size_t smem = (size_t)kTcAlign + kTcHeader + 2 * ((size_t)16 * 8 * 128 + (size_t)(a.Cin / 8) * 8 * 128);
  {
    static std::mutex mu;
    static bool attr_set[kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("wgrad_tc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!attr_set[dev]) {
      if (cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemMax) !=
          cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error("wgrad_tc: shared memory attribute");
      }
      attr_set[dev] = true;
    }
  }
  const unsigned cols = tc_cols(a.Cin);
  // 64 slices of 64 nodes per CTA, fewer when that leaves too few CTAs to fill the GPU
  long long kc = 64LL * kWgNodes;
  while (kc > kWgNodes && ((a.nodes + kc - 1) / kc) * taps < 4LL * kSMs) kc /= 2;
  const long long chunks = (a.nodes + kc - 1) / kc;
  if (chunks > 65535) throw std::runtime_error("wgrad_tc: too many nodes");
  ctx.add_flops(name, 2.0 * taps * a.Cin * a.Cout * (double)a.nodes);
  HZ_LAUNCH(ctx, name, (double)a.nodes * (a.Cin + a.Cout) * 2.0 * taps, k_wgrad_tc, dim3(1u, (unsigned)chunks, taps),
            128, smem, a.nx, a.ny, a.nz, a.nodes, taps, a.Cin, a.in, a.ldi, a.Cout, a.dout, a.ldd, a.d_off, a.dw, kc,
            cols, err);
}

}  // namespace hz
