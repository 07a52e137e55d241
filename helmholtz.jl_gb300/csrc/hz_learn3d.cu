// Learned coarse-grid correction, 3D variant: a convolutional encoder-decoder
// over three grid levels with 8-16-32 channels (BF16 weights and activations,
// FP32 accumulation on the tensor cores), trained on the GPU by the kernels of
// this file and applied inside the multigrid cycle in place of the coarse-grid
// correction below a chosen level of a 3D hierarchy.
//
// Network (grids g0 -> g1 -> g2 by node coarsening n -> (n-1)/2+1; NDHWC
// activations, channel counts padded for the tensor cores):
//   e0 = relu(conv(x,  4 -> 8))            on g0
//   e1 = relu(conv(R e0, 8 -> 16))         on g1     R: full weighting per channel
//   e2 = relu(conv(R e1, 16 -> 32))        on g2
//   d1 = relu(conv([P e2, e1], 48 -> 16))  on g1     P: trilinear prolongation per channel
//   d0 = relu(conv([P d1, e0], 24 -> 8))   on g0
//   y  = conv(d0, 8 -> 2)                  on g0     (Re, Im)
// Convolutions are 3x3x3 with zero padding, weights [cout][27][cin] with tap
// t = 9 (dz + 1) + 3 (dy + 1) + (dx + 1).  As in the 2D network there are no
// biases (positive homogeneity: the solver feeds the residual scaled to unit
// RMS and scales the output back) and the skip tensors e0, e1 are written
// straight into the upper channels of the decoder's concatenation buffers.
// The definition is pinned by the CPU oracle oracle/coarse_net3d.py.
//
// Convolutions are implicit GEMMs on the tensor cores (mma.sync m16n8k16,
// BF16 x BF16 -> FP32).  A CTA owns 64 consecutive nodes of one sample; per
// 16-channel chunk it stages the nine strips of input rows the (dy, dz) tap
// planes reach (66 rows each) and the chunk of the weights in shared memory,
// and every warp runs 27 taps x NT MMAs for its 16 nodes.  Taps that leave the
// grid read zeros (a 27-bit validity mask per node), which is the zero padding.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <stdexcept>
#include <vector>

#include "hz_launch.cuh"
#include "hz_learn.h"

namespace hz {

using bf16 = __nv_bfloat16;

namespace {

struct LayerSpec3 {
  int cin, cout, cinp, coutp, lev;
};
// the 6 convolutions in forward order; cinp: inputs padded to 16, coutp: outputs padded to 8
constexpr LayerSpec3 kSpec3[CoarseNet3::kLayers] = {
    {4, 8, 16, 8, 0}, {8, 16, 16, 16, 1}, {16, 32, 16, 32, 2}, {48, 16, 48, 16, 1}, {24, 8, 32, 8, 0}, {8, 2, 16, 8, 0},
};
constexpr int kTaps3 = 27;
inline int round16(int c) { return (c + 15) / 16 * 16; }

// activation slots: grid level and (padded) channel count
//   X  input (4 of 16)            C0 [P d1 (16) | e0 (8) | 0 (8)]   R0 R e0 (8 of 16)
//   C1 [P e2 (32) | e1 (16)]      R1 R e1 (16)                      E2 e2 (32)
//   D1 d1 (16)                    D0 d0 (8 of 16)
enum Slot3 { X3 = 0, C03, R03, C13, R13, E23, D13, D03, NSLOT3 };
constexpr int kSlotLev3[NSLOT3] = {0, 0, 1, 1, 2, 2, 1, 0};
constexpr int kSlotCh3[NSLOT3] = {16, 32, 16, 48, 16, 32, 16, 16};

// tap offsets
__host__ __device__ __forceinline__ void tap3(int t, int& dx, int& dy, int& dz) {
  dx = t % 3 - 1;
  dy = (t / 3) % 3 - 1;
  dz = t / 9 - 1;
}

}  // namespace

// ---------------------------------------------------------------------------
// conv3x3x3 on the tensor cores
//   in  [B][N] rows of ldi bf16, channels i_off .. i_off+Cin (Cin multiple of 16)
//   w   [Cout][27][Cin] bf16
//   out [B][N] rows of ldo, channels o_off + co (bf16, or FP32 into out32)
// epilogue: optional ReLU; optional mask: zero where mask[row*ldm + m_off + co] <= 0
// for co >= mask_lo.  grid.z splits Cout in chunks of 8*NT.
// Shared rows are padded to 24 bf16 (48 bytes) so the 8 rows of a fragment load
// start in different bank groups.
// ---------------------------------------------------------------------------
constexpr int kC3Tile = 64;              // nodes per CTA
constexpr int kC3Strip = kC3Tile + 2;    // rows per strip
constexpr int kC3Strips = 9;             // (dy, dz) planes
constexpr int kC3CK = 16;                // channels per staged chunk
constexpr int kC3SR = kC3CK + 8;         // padded shared row (bf16)

__device__ __forceinline__ void ldsm3_x4(const bf16* p, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void ldsm3_x2(const bf16* p, unsigned& r0, unsigned& r1) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}
__device__ __forceinline__ void mma16816(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// 27-bit mask of the taps of node p that stay inside the grid (0 for p >= N)
__device__ __forceinline__ unsigned tap_mask3(long long p, long long N, int nx, int ny, int nz) {
  if (p >= N) return 0u;
  const int i = (int)(p % nx);
  const long long q = p / nx;
  const int j = (int)(q % ny), k = (int)(q / ny);
  unsigned m = 0u;
#pragma unroll
  for (int t = 0; t < kTaps3; ++t) {
    int dx, dy, dz;
    tap3(t, dx, dy, dz);
    if (i + dx >= 0 && i + dx < nx && j + dy >= 0 && j + dy < ny && k + dz >= 0 && k + dz < nz) m |= 1u << t;
  }
  return m;
}

template <int NT>
__global__ void __launch_bounds__(128) k_conv3_mma(int nx, int ny, int nz, int Cin, int Cout,
                                                   const bf16* __restrict__ in, int ldi, int i_off,
                                                   const bf16* __restrict__ w, bf16* __restrict__ out,
                                                   float* __restrict__ out32, int ldo, int o_off, int relu,
                                                   const bf16* __restrict__ mask, int ldm, int m_off, int mask_lo) {
  extern __shared__ __align__(16) unsigned char c3_smem[];
  bf16* s_in = reinterpret_cast<bf16*>(c3_smem);
  bf16* s_w = s_in + kC3Strips * kC3Strip * kC3SR;
  const long long N = (long long)nx * ny * nz;
  const long long sy = nx, sz = (long long)nx * ny;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const long long p0 = (long long)blockIdx.x * kC3Tile;
  const int bidx = blockIdx.y;
  const int co0 = blockIdx.z * 8 * NT;
  const int g = lane >> 2, tq = lane & 3;
  const long long pa = p0 + warp * 16 + g, pb = pa + 8;
  const bool active = p0 + warp * 16 < N;
  const unsigned ma = tap_mask3(pa, N, nx, ny, nz), mb = tap_mask3(pb, N, nx, ny, nz);
  const bf16* inb = in + (long long)bidx * N * ldi + i_off;
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  float acc[NT][4];
#pragma unroll
  for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
  for (int c0 = 0; c0 < Cin; c0 += kC3CK) {
    __syncthreads();
    for (int e = threadIdx.x; e < kC3Strips * kC3Strip * 2; e += blockDim.x) {
      const int h = e & 1, rr = e >> 1;
      const int sidx = rr / kC3Strip, k = rr % kC3Strip;
      const int dy = sidx % 3 - 1, dz = sidx / 3 - 1;
      const long long gr = p0 + dy * sy + dz * sz - 1 + k;
      uint4 v = zero;
      if (gr >= 0 && gr < N) v = *reinterpret_cast<const uint4*>(inb + gr * ldi + c0 + 8 * h);
      *reinterpret_cast<uint4*>(s_in + rr * kC3SR + 8 * h) = v;
    }
    for (int e = threadIdx.x; e < 8 * NT * kTaps3 * 2; e += blockDim.x) {
      const int h = e & 1, rr = e >> 1;
      const int co = rr / kTaps3, t = rr % kTaps3;
      uint4 v = zero;
      if (co0 + co < Cout)
        v = *reinterpret_cast<const uint4*>(w + ((long long)(co0 + co) * kTaps3 + t) * Cin + c0 + 8 * h);
      *reinterpret_cast<uint4*>(s_w + rr * kC3SR + 8 * h) = v;
    }
    __syncthreads();
    if (active) {
      // ldmatrix row addresses: A matrix m = lane/8 covers local nodes
      // warp*16 + 8(m&1) + lane%8 and channels 8(m>>1)..; B matrix m covers the
      // weight rows of output channel 8(n + (m>>1)) + lane%8, channels 8(m&1)..
      const int lm = lane >> 3, lr = lane & 7;
      const int a_node = warp * 16 + (lm & 1) * 8 + lr;
      const int a_col = (lm >> 1) * 8;
      const int b_row = (lm >> 1) * 8 + lr;
      const int b_col = (lm & 1) * 8;
#pragma unroll 3
      for (int t = 0; t < kTaps3; ++t) {
        int dx, dy, dz;
        tap3(t, dx, dy, dz);
        const int strip = (dy + 1) + 3 * (dz + 1);
        unsigned a0, a1, a2, a3;
        ldsm3_x4(s_in + (strip * kC3Strip + a_node + dx + 1) * kC3SR + a_col, a0, a1, a2, a3);
        // the lane's A rows are its own nodes pa (a0, a2) and pb (a1, a3): zero the taps off the grid
        if (!((ma >> t) & 1u)) a0 = a2 = 0u;
        if (!((mb >> t) & 1u)) a1 = a3 = 0u;
#pragma unroll
        for (int n = 0; n < NT; n += 2) {
          unsigned b0, b1, b2 = 0u, b3 = 0u;
          if (n + 1 < NT)
            ldsm3_x4(s_w + ((n * 8 + b_row) * kTaps3 + t) * kC3SR + b_col, b0, b1, b2, b3);
          else
            ldsm3_x2(s_w + ((n * 8 + lr) * kTaps3 + t) * kC3SR + (lm & 1) * 8, b0, b1);
          mma16816(acc[n], a0, a1, a2, a3, b0, b1);
          if (n + 1 < NT) mma16816(acc[n + 1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
  if (!active) return;
#pragma unroll
  for (int n = 0; n < NT; ++n) {
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const long long p = hh ? pb : pa;
      if (p >= N) continue;
      const long long row = (long long)bidx * N + p;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int co = co0 + n * 8 + tq * 2 + e;
        if (co >= Cout) continue;
        float v = acc[n][hh * 2 + e];
        if (relu) v = fmaxf(v, 0.f);
        if (mask && co >= mask_lo && !(__bfloat162float(mask[row * ldm + m_off + co]) > 0.f)) v = 0.f;
        if (out32)
          out32[row * ldo + o_off + co] = v;
        else
          out[row * ldo + o_off + co] = __float2bfloat16_rn(v);
      }
    }
  }
}

static size_t conv3_smem(int NT) {
  return (size_t)(kC3Strips * kC3Strip + 8 * NT * kTaps3) * kC3SR * sizeof(bf16);
}

template <int NT>
static void conv3_set_smem() {
  // the weights of 8*NT output channels need more than the default 48 KB for NT >= 4
  static int done[kMaxDevices] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices || done[dev]) return;
  const cudaError_t e =
      cudaFuncSetAttribute(k_conv3_mma<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)conv3_smem(NT));
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string("conv3: shared memory attribute: ") + cudaGetErrorString(e));
  }
  done[dev] = 1;
}

static void conv3_launch(Ctx& ctx, const char* name, const int* gd, int B, int Cin, const bf16* in, int ldi, int i_off,
                         int Cout, const bf16* w, bf16* out, float* out32, int ldo, int o_off, int relu,
                         const bf16* mask, int ldm, int m_off, int mask_lo) {
  if (Cin % 16 != 0 || (ldi % 8) || (i_off % 8)) throw std::runtime_error("conv3: channel layout not aligned");
  const long long N = (long long)gd[0] * gd[1] * gd[2];
  const int NT = Cout <= 8 ? 1 : Cout <= 16 ? 2 : Cout <= 32 ? 4 : 8;
  const long long nb = (N + kC3Tile - 1) / kC3Tile;
  if (nb >= (1LL << 31) || B > 65535) throw std::runtime_error("conv3: grid too large");
  const dim3 grid((unsigned)nb, (unsigned)B, (unsigned)((Cout + 8 * NT - 1) / (8 * NT)));
  const double bytes = (double)B * N * (Cin * 2.0 + Cout * (out32 ? 4.0 : 2.0)) + 27.0 * Cin * Cout * 2.0;
  ctx.add_flops(name, 2.0 * 27.0 * Cin * Cout * (double)N * B);
  const size_t smem = conv3_smem(NT);
#define HZ_C3_CASE(K)                                                                                            \
  case K:                                                                                                        \
    conv3_set_smem<K>();                                                                                         \
    HZ_LAUNCH(ctx, name, bytes, k_conv3_mma<K>, grid, 128, smem, gd[0], gd[1], gd[2], Cin, Cout, in, ldi, i_off, w, \
              out, out32, ldo, o_off, relu, mask, ldm, m_off, mask_lo);                                          \
    break;
  switch (NT) {
    HZ_C3_CASE(1)
    HZ_C3_CASE(2)
    HZ_C3_CASE(4)
    default:
      HZ_C3_CASE(8)
  }
#undef HZ_C3_CASE
}

// weights of the data-gradient convolution: wt[ci][t][co] = w[co][26 - t][ci],
// co padded from Cout to K (zero rows)
__global__ void k_wflip3(int Cout, int Cin, int K, const bf16* __restrict__ w, bf16* __restrict__ wt) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= Cin * kTaps3 * K) return;
  const int co = idx % K, t = (idx / K) % kTaps3, ci = idx / (K * kTaps3);
  wt[idx] = (co < Cout) ? w[((long long)co * kTaps3 + (kTaps3 - 1 - t)) * Cin + ci] : __float2bfloat16_rn(0.f);
}

// Weight gradient on the tensor cores: dw[co][t][ci] += sum_n dout[n][co] * in[n + off_t][ci],
// a GEMM with M = Cout, N = Cin and K = the nodes.  One CTA (4 warps) owns one
// tap t (blockIdx.z) and a range of kc nodes (blockIdx.y); it stages 64-node
// slices of the input rows (zeroed where the tap leaves the grid) and of the
// output-gradient rows in shared memory, runs m16n8k16 MMAs over 16-node
// K-steps (warp w owns the 16x8 output tiles w, w+4, ...) and adds its
// partial sums to dw with one atomic per weight.
constexpr int kWg3KS = 64;
constexpr int kWg3MaxTiles = 12;  // 16x8 tiles per warp: Cout <= 32 with Cin <= 48

__device__ __forceinline__ unsigned pack2bf(bf16 lo, bf16 hi) {
  return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

__global__ void __launch_bounds__(128) k_wgrad3_mma(int nx, int ny, int nz, long long total, int Cin, int Cout,
                                                    const bf16* __restrict__ in, int ldi,
                                                    const bf16* __restrict__ dout, int ldd, int d_off,
                                                    float* __restrict__ dw, long long kc) {
  extern __shared__ __align__(16) unsigned char wg3_smem[];
  const long long N = (long long)nx * ny * nz;
  const int t = blockIdx.z;
  int dx, dy, dz;
  tap3(t, dx, dy, dz);
  const long long toff = dx + (long long)dy * nx + (long long)dz * nx * ny;
  const int C16 = (Cout + 15) / 16 * 16;
  const int sIn = Cin + 8, sD = C16 + 8;
  bf16* s_in = reinterpret_cast<bf16*>(wg3_smem);
  bf16* s_d = s_in + kWg3KS * sIn;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tq = lane & 3;
  const int NTn = Cin / 8, T = (C16 / 16) * NTn;
  float acc[kWg3MaxTiles][4];
#pragma unroll
  for (int k = 0; k < kWg3MaxTiles; ++k) acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.f;
  const long long q0 = (long long)blockIdx.y * kc;
  const long long q1 = min(total, q0 + kc);
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  for (long long qs = q0; qs < q1; qs += kWg3KS) {
    __syncthreads();
    const int cin8 = Cin / 8, cd8 = C16 / 8;
    for (int e = threadIdx.x; e < kWg3KS * cin8; e += blockDim.x) {
      const int r = e / cin8, c8 = e % cin8;
      const long long q = qs + r;
      uint4 v = zero;
      if (q < q1) {
        const long long p = q % N;
        const int i = (int)(p % nx) + dx;
        const long long pq = p / nx;
        const int j = (int)(pq % ny) + dy, k = (int)(pq / ny) + dz;
        if (i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz)
          v = *reinterpret_cast<const uint4*>(in + (q + toff) * ldi + c8 * 8);
      }
      *reinterpret_cast<uint4*>(s_in + r * sIn + c8 * 8) = v;
    }
    for (int e = threadIdx.x; e < kWg3KS * cd8; e += blockDim.x) {
      const int r = e / cd8, c8 = e % cd8;
      const long long q = qs + r;
      uint4 v = zero;
      if (q < q1 && c8 * 8 < Cout) v = *reinterpret_cast<const uint4*>(dout + q * ldd + d_off + c8 * 8);
      *reinterpret_cast<uint4*>(s_d + r * sD + c8 * 8) = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int kb = 0; kb < kWg3KS; kb += 16) {
      const bf16* d0 = s_d + (kb + tq * 2) * sD;
      const bf16* i0 = s_in + (kb + tq * 2) * sIn;
#pragma unroll
      for (int k = 0; k < kWg3MaxTiles; ++k) {
        const int tile = warp + 4 * k;
        if (tile < T) {
          const int co = (tile / NTn) * 16 + g;
          const int ci = (tile % NTn) * 8 + g;
          const unsigned a0 = pack2bf(d0[co], d0[sD + co]);
          const unsigned a1 = pack2bf(d0[co + 8], d0[sD + co + 8]);
          const unsigned a2 = pack2bf(d0[8 * sD + co], d0[9 * sD + co]);
          const unsigned a3 = pack2bf(d0[8 * sD + co + 8], d0[9 * sD + co + 8]);
          const unsigned b0 = pack2bf(i0[ci], i0[sIn + ci]);
          const unsigned b1 = pack2bf(i0[8 * sIn + ci], i0[9 * sIn + ci]);
          mma16816(acc[k], a0, a1, a2, a3, b0, b1);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kWg3MaxTiles; ++k) {
    const int tile = warp + 4 * k;
    if (tile >= T) break;
    const int co = (tile / NTn) * 16 + g;
    const int ci = (tile % NTn) * 8 + tq * 2;
    if (co < Cout) {
      atomicAdd(&dw[((long long)co * kTaps3 + t) * Cin + ci], acc[k][0]);
      atomicAdd(&dw[((long long)co * kTaps3 + t) * Cin + ci + 1], acc[k][1]);
    }
    if (co + 8 < Cout) {
      atomicAdd(&dw[((long long)(co + 8) * kTaps3 + t) * Cin + ci], acc[k][2]);
      atomicAdd(&dw[((long long)(co + 8) * kTaps3 + t) * Cin + ci + 1], acc[k][3]);
    }
  }
}

// Per-channel resampling between 3D grid levels (NDHWC bf16, FP32 arithmetic),
// the 3D counterparts of the 2D network's transfers:
// mode 0, restriction (fine -> coarse): full weighting, weights 1, 1/2 per axis,
// normalised by the weights that fall inside the grid (the product of the 1D sums).
// mode 1, prolongation (coarse -> fine): trilinear, the mean of c[i0] and c[i1]
// per axis with i0 = i / 2, i1 = (i + 1) / 2.
// transpose = 1 applies the adjoint.  The result, zeroed where mask <= 0 (mask
// may be null), is written or, with accum, added to out (rounded to bf16 once).
// One thread per (node, 8 channels): 16-byte loads and stores.
struct F8x {
  float v[8];
};
__device__ __forceinline__ void ld8x(const bf16* p, F8x& f) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float2 x = __bfloat1622float2(h[k]);
    f.v[2 * k] = x.x;
    f.v[2 * k + 1] = x.y;
  }
}
__device__ __forceinline__ void axpy8x(float a, const bf16* p, F8x& acc) {
  F8x f;
  ld8x(p, f);
#pragma unroll
  for (int k = 0; k < 8; ++k) acc.v[k] = fmaf(a, f.v[k], acc.v[k]);
}
// 1D full-weighting sum of coarse node I on an axis of nf fine nodes
__device__ __forceinline__ float fw_sum(int I, int nf) {
  return 1.f + (2 * I - 1 >= 0 ? 0.5f : 0.f) + (2 * I + 1 < nf ? 0.5f : 0.f);
}

__global__ void k_resample3(int mode, int transpose, int nxf, int nyf, int nzf, int nxc, int nyc, int nzc, int B,
                            int C, const bf16* __restrict__ in, int ldi, int i_off, bf16* __restrict__ out, int ldo,
                            int o_off, int accum, const bf16* __restrict__ mask, int ldm, int m_off) {
  const long long Nf = (long long)nxf * nyf * nzf, Nc = (long long)nxc * nyc * nzc;
  const bool to_coarse = (mode == 0) != (transpose != 0);
  const long long No = to_coarse ? Nc : Nf, Ni = to_coarse ? Nf : Nc;
  const int C8 = C / 8;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)B * No * C8) return;
  const int c = (int)(idx % C8) * 8;
  const long long q = idx / C8;
  const int b = (int)(q / No);
  const long long po = q % No;
  const bf16* ib = in + (long long)b * Ni * ldi + i_off + c;
  F8x acc;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc.v[k] = 0.f;
  const int nxo = to_coarse ? nxc : nxf, nyo = to_coarse ? nyc : nyf;
  const int io = (int)(po % nxo);
  const long long t = po / nxo;
  const int jo = (int)(t % nyo), ko = (int)(t / nyo);
  if (mode == 0 && !transpose) {  // restriction: coarse (io, jo, ko) <- fine 2I + d
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          const int fi = 2 * io + di, fj = 2 * jo + dj, fk = 2 * ko + dk;
          if (fi < 0 || fi >= nxf || fj < 0 || fj >= nyf || fk < 0 || fk >= nzf) continue;
          const float wg = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f);
          axpy8x(wg, ib + (fi + (long long)nxf * (fj + (long long)nyf * fk)) * ldi, acc);
        }
    const float inv = 1.f / (fw_sum(io, nxf) * fw_sum(jo, nyf) * fw_sum(ko, nzf));
#pragma unroll
    for (int k = 0; k < 8; ++k) acc.v[k] *= inv;
  } else if (mode == 0) {  // adjoint of the restriction: fine (io, jo, ko) <- coarse parents
    for (int K = ko / 2 - 1; K <= ko / 2 + 1; ++K)
      for (int J = jo / 2 - 1; J <= jo / 2 + 1; ++J)
        for (int I = io / 2 - 1; I <= io / 2 + 1; ++I) {
          if (I < 0 || I >= nxc || J < 0 || J >= nyc || K < 0 || K >= nzc) continue;
          const int di = io - 2 * I, dj = jo - 2 * J, dk = ko - 2 * K;
          if (di < -1 || di > 1 || dj < -1 || dj > 1 || dk < -1 || dk > 1) continue;
          const float wg = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f) /
                           (fw_sum(I, nxf) * fw_sum(J, nyf) * fw_sum(K, nzf));
          axpy8x(wg, ib + (I + (long long)nxc * (J + (long long)nyc * K)) * ldi, acc);
        }
  } else if (!transpose) {  // prolongation: fine (io, jo, ko) <- 8 coarse corners
    const int i0 = io >> 1, i1 = (io + 1) >> 1, j0 = jo >> 1, j1 = (jo + 1) >> 1, k0 = ko >> 1, k1 = (ko + 1) >> 1;
    const int is[2] = {i0, i1}, js[2] = {j0, j1}, ks[2] = {k0, k1};
#pragma unroll
    for (int a = 0; a < 8; ++a)
      axpy8x(0.125f, ib + (is[a & 1] + (long long)nxc * (js[(a >> 1) & 1] + (long long)nyc * ks[a >> 2])) * ldi,
             acc);
  } else {  // adjoint of the prolongation: coarse (io, jo, ko) <- fine children
    for (int fk = 2 * ko - 1; fk <= 2 * ko + 1; ++fk)
      for (int fj = 2 * jo - 1; fj <= 2 * jo + 1; ++fj)
        for (int fi = 2 * io - 1; fi <= 2 * io + 1; ++fi) {
          if (fi < 0 || fi >= nxf || fj < 0 || fj >= nyf || fk < 0 || fk >= nzf) continue;
          const float wg = (fi == 2 * io ? 1.f : 0.5f) * (fj == 2 * jo ? 1.f : 0.5f) * (fk == 2 * ko ? 1.f : 0.5f);
          axpy8x(wg, ib + (fi + (long long)nxf * (fj + (long long)nyf * fk)) * ldi, acc);
        }
  }
  const long long row = (long long)b * No + po;
  if (mask) {
    F8x mk;
    ld8x(mask + row * ldm + m_off + c, mk);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (!(mk.v[k] > 0.f)) acc.v[k] = 0.f;
  }
  bf16* o = out + row * ldo + o_off + c;
  if (accum) {
    F8x old;
    ld8x(o, old);
#pragma unroll
    for (int k = 0; k < 8; ++k) acc.v[k] += old.v[k];
  }
  __align__(16) __nv_bfloat162 r[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) r[k] = __floats2bfloat162_rn(acc.v[2 * k], acc.v[2 * k + 1]);
  *reinterpret_cast<uint4*>(o) = *reinterpret_cast<const uint4*>(r);
}

static void resample3(Ctx& ctx, int mode, int transpose, const int (*gd)[3], int lf, int B, int C, const bf16* in,
                      int ldi, int i_off, bf16* out, int ldo, int o_off, int accum, const bf16* mask = nullptr,
                      int ldm = 0, int m_off = 0) {
  if (C % 8 || ldi % 8 || i_off % 8 || ldo % 8 || o_off % 8 || (mask && (ldm % 8 || m_off % 8)))
    throw std::runtime_error("resample3: channel layout not aligned");
  const int* f = gd[lf];
  const int* cg = gd[lf + 1];
  const bool to_coarse = (mode == 0) != (transpose != 0);
  const long long nf = (long long)f[0] * f[1] * f[2], nc = (long long)cg[0] * cg[1] * cg[2];
  const long long no = to_coarse ? nc : nf, ni = to_coarse ? nf : nc;
  const long long total = (long long)B * no * (C / 8);
  const long long nblk = (total + 255) / 256;
  if (nblk >= (1LL << 31)) throw std::runtime_error("resample3: batch too large");
  HZ_LAUNCH(ctx, "net3_resample", (double)B * (no + ni) * C * 2.0, k_resample3, (unsigned)nblk, 256, 0, mode,
            transpose, f[0], f[1], f[2], cg[0], cg[1], cg[2], B, C, in, ldi, i_off, out, ldo, o_off, accum, mask, ldm,
            m_off);
}

// ---------------------------------------------------------------------------
// CoarseNet3
// ---------------------------------------------------------------------------
long long CoarseNet3::num_params() {
  long long n = 0;
  for (const auto& L : kSpec3) n += (long long)L.cout * kTaps3 * L.cin;
  return n;
}

void CoarseNet3::layer_shape(int l, int* cin, int* cout) {
  *cin = kSpec3[l].cin;
  *cout = kSpec3[l].cout;
}

bool CoarseNet3::supports(long long nx, long long ny, long long nz) {
  auto ok = [](long long n) { return n >= 5 && (n - 1) % 4 == 0; };
  return ok(nx) && ok(ny) && ok(nz) && nx * ny * nz < (1LL << 30);
}

static void cuda_ok3(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string("coarse net 3D: ") + what + ": " + cudaGetErrorString(e));
  }
}
template <typename P> static void dalloc3(P** p, size_t bytes) {
  cuda_ok3(cudaMalloc(reinterpret_cast<void**>(p), bytes), "cudaMalloc");
}
template <typename P> static void dfree3(P*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

CoarseNet3::CoarseNet3(unsigned seed) {
  cuda_ok3(cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking), "stream");
  long long off = 0;
  for (int l = 0; l < kLayers; ++l) {
    woff_[l] = off;
    off += (long long)kSpec3[l].coutp * kTaps3 * kSpec3[l].cinp;
  }
  wtotal_ = off;
  for (int l = 0; l < kLayers; ++l) {
    imgoff_[l] = imgtotal_;
    imgtotal_ += (long long)round16(kSpec3[l].coutp) * kTaps3 * kSpec3[l].cinp;
  }
  dalloc3(&tc_err_, sizeof(int));
  cuda_ok3(cudaMemset(tc_err_, 0, sizeof(int)), "tensor-core status");
  dalloc3(&w32_, off * 4);
  dalloc3(&wbf_, off * 2);
  dalloc3(&g32_, off * 4);
  dalloc3(&m_, off * 4);
  dalloc3(&v_, off * 4);
  // He-normal initialisation (last layer scaled down), from a seeded host generator
  std::vector<float> w((size_t)num_params());
  std::mt19937 rng(seed);
  size_t k = 0;
  for (int l = 0; l < kLayers; ++l) {
    const auto& L = kSpec3[l];
    std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / (27.0f * L.cin)) * (l == kLayers - 1 ? 0.5f : 1.0f));
    for (long long q = 0; q < (long long)L.cout * kTaps3 * L.cin; ++q) w[k++] = nd(rng);
  }
  set_weights(w.data());
}

CoarseNet3::~CoarseNet3() {
  release_acts();
  dfree3(tc_err_);
  dfree3(wimg_);
  dfree3(w32_);
  dfree3(wbf_);
  dfree3(g32_);
  dfree3(m_);
  dfree3(v_);
  dfree3(wt_);
  dfree3(x4_);
  dfree3(scale_);
  dfree3(loss_);
  dfree3(bx_);
  dfree3(bt_);
  dfree3(perm_);
  ctx.release();
  if (ctx.stream) cudaStreamDestroy(ctx.stream);
}

// host (unpadded, layer after layer [cout][27][cin]) <-> device (padded [coutp][27][cinp])
static void pad_weights3(const float* host, const long long* woff, long long total, std::vector<float>& dev) {
  dev.assign((size_t)total, 0.f);
  size_t k = 0;
  for (int l = 0; l < CoarseNet3::kLayers; ++l) {
    const auto& L = kSpec3[l];
    for (int co = 0; co < L.cout; ++co)
      for (int t = 0; t < kTaps3; ++t)
        for (int ci = 0; ci < L.cin; ++ci)
          dev[(size_t)(woff[l] + ((long long)co * kTaps3 + t) * L.cinp + ci)] = host[k++];
  }
}
static void unpad_weights3(const std::vector<float>& dev, const long long* woff, float* host) {
  size_t k = 0;
  for (int l = 0; l < CoarseNet3::kLayers; ++l) {
    const auto& L = kSpec3[l];
    for (int co = 0; co < L.cout; ++co)
      for (int t = 0; t < kTaps3; ++t)
        for (int ci = 0; ci < L.cin; ++ci)
          host[k++] = dev[(size_t)(woff[l] + ((long long)co * kTaps3 + t) * L.cinp + ci)];
  }
}

void CoarseNet3::set_weights(const float* host) {
  std::vector<float> w;
  pad_weights3(host, woff_, wtotal_, w);
  cuda_ok3(cudaStreamSynchronize(ctx.stream), "sync");
  cuda_ok3(cudaMemcpy(w32_, w.data(), wtotal_ * 4, cudaMemcpyHostToDevice), "upload weights");
  cuda_ok3(cudaMemset(m_, 0, wtotal_ * 4), "adam m");
  cuda_ok3(cudaMemset(v_, 0, wtotal_ * 4), "adam v");
  step_ = 0;
  k_f2bf<<<256, 256, 0, ctx.stream>>>(wtotal_, w32_, wbf_);
  cuda_ok3(cudaGetLastError(), "weights to bf16");
  refresh_images(ctx);
  cuda_ok3(cudaStreamSynchronize(ctx.stream), "sync");
}

static void download_unpadded3(const float* dev, long long total, const long long* woff, float* host) {
  std::vector<float> w((size_t)total);
  cuda_ok3(cudaMemcpy(w.data(), dev, total * 4, cudaMemcpyDeviceToHost), "download");
  unpad_weights3(w, woff, host);
}

void CoarseNet3::get_weights(float* host) const {
  cuda_ok3(cudaStreamSynchronize(ctx.stream), "sync");
  download_unpadded3(w32_, wtotal_, woff_, host);
}

void CoarseNet3::get_grad(float* host) const {
  cuda_ok3(cudaStreamSynchronize(ctx.stream), "sync");
  download_unpadded3(g32_, wtotal_, woff_, host);
}

// ---- file format -----------------------------------------------------------
// "HZCNET3D" | u32 version | u32 layers | layers x (i32 cin, i32 cout) |
// i64 nparams | i64 adam step | f32 weights[n] | f32 m[n] | f32 v[n]
// (little-endian; unpadded, layer after layer [cout][27][cin])
static const char kNet3Magic[8] = {'H', 'Z', 'C', 'N', 'E', 'T', '3', 'D'};
static constexpr unsigned kNet3Version = 1;

void CoarseNet3::save(const char* path) const {
  cuda_ok3(cudaStreamSynchronize(ctx.stream), "sync");
  const long long n = num_params();
  std::vector<float> w((size_t)n), m((size_t)n), v((size_t)n);
  download_unpadded3(w32_, wtotal_, woff_, w.data());
  download_unpadded3(m_, wtotal_, woff_, m.data());
  download_unpadded3(v_, wtotal_, woff_, v.data());
  FILE* f = std::fopen(path, "wb");
  if (!f) throw std::runtime_error(std::string("coarse net 3D: cannot write ") + path);
  const unsigned hdr[2] = {kNet3Version, (unsigned)kLayers};
  bool ok = std::fwrite(kNet3Magic, 1, 8, f) == 8 && std::fwrite(hdr, 4, 2, f) == 2;
  for (int l = 0; l < kLayers && ok; ++l) {
    const int sh[2] = {kSpec3[l].cin, kSpec3[l].cout};
    ok = std::fwrite(sh, 4, 2, f) == 2;
  }
  const long long meta[2] = {n, step_};
  ok = ok && std::fwrite(meta, 8, 2, f) == 2;
  ok = ok && std::fwrite(w.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fwrite(m.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fwrite(v.data(), 4, (size_t)n, f) == (size_t)n;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) throw std::runtime_error(std::string("coarse net 3D: write failed: ") + path);
}

int CoarseNet3::file_info(const char* path, long long* nparams, long long* step) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return -1;
  char mg[8];
  unsigned hdr[2];
  int rc = 0;
  if (std::fread(mg, 1, 8, f) != 8 || std::memcmp(mg, kNet3Magic, 8) != 0) rc = -2;
  if (!rc && std::fread(hdr, 4, 2, f) != 2) rc = -5;
  if (!rc && hdr[0] != kNet3Version) rc = -3;
  if (!rc && hdr[1] != (unsigned)kLayers) rc = -4;
  for (int l = 0; l < kLayers && !rc; ++l) {
    int sh[2];
    if (std::fread(sh, 4, 2, f) != 2)
      rc = -5;
    else if (sh[0] != kSpec3[l].cin || sh[1] != kSpec3[l].cout)
      rc = -4;
  }
  long long meta[2] = {0, 0};
  if (!rc && std::fread(meta, 8, 2, f) != 2) rc = -5;
  if (!rc && meta[0] != num_params()) rc = -4;
  if (!rc) {
    const long long need = 3LL * meta[0] * 4;
    const long pos = std::ftell(f);
    if (std::fseek(f, 0, SEEK_END) != 0 || std::ftell(f) - pos < need) rc = -5;
  }
  std::fclose(f);
  if (!rc) {
    if (nparams) *nparams = meta[0];
    if (step) *step = meta[1];
  }
  return rc;
}

void CoarseNet3::load(const char* path) {
  long long n = 0, st = 0;
  const int rc = file_info(path, &n, &st);
  static const char* why[] = {"", "cannot read", "not a 3D coarse-network file", "unsupported version",
                              "layer shapes differ", "truncated"};
  if (rc < 0) throw std::runtime_error(std::string("coarse net 3D: ") + path + ": " + why[-rc]);
  std::vector<float> w((size_t)n), m((size_t)n), v((size_t)n);
  FILE* f = std::fopen(path, "rb");
  if (!f) throw std::runtime_error(std::string("coarse net 3D: cannot read ") + path);
  const long hdr_bytes = 8 + 8 + kLayers * 8 + 16;
  bool ok = std::fseek(f, hdr_bytes, SEEK_SET) == 0;
  ok = ok && std::fread(w.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fread(m.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fread(v.data(), 4, (size_t)n, f) == (size_t)n;
  std::fclose(f);
  if (!ok) throw std::runtime_error(std::string("coarse net 3D: truncated ") + path);
  for (long long i = 0; i < n; ++i)
    if (!std::isfinite(w[(size_t)i]) || !std::isfinite(m[(size_t)i]) || !(v[(size_t)i] >= 0.f))
      throw std::runtime_error(std::string("coarse net 3D: non-finite weights or state in ") + path);
  set_weights(w.data());  // resets the moments; restore them below
  std::vector<float> pm, pv;
  pad_weights3(m.data(), woff_, wtotal_, pm);
  pad_weights3(v.data(), woff_, wtotal_, pv);
  cuda_ok3(cudaMemcpy(m_, pm.data(), wtotal_ * 4, cudaMemcpyHostToDevice), "upload moments");
  cuda_ok3(cudaMemcpy(v_, pv.data(), wtotal_ * 4, cudaMemcpyHostToDevice), "upload moments");
  step_ = st;
}

void CoarseNet3::release_acts() {
  for (int i = 0; i < NSLOT3; ++i) {
    dfree3(act_[i]);
    dfree3(grd_[i]);
  }
  dfree3(y32_);
  g_[0][0] = g_[0][1] = g_[0][2] = 0;
  B_ = 0;
  grads_ = false;
}

void CoarseNet3::ensure(int nx, int ny, int nz, int B, bool grads) {
  if (!supports(nx, ny, nz)) throw std::runtime_error("coarse net 3D: grid must have (n - 1) divisible by 4, n >= 5");
  if (nx == g_[0][0] && ny == g_[0][1] && nz == g_[0][2] && B <= B_ && (grads_ || !grads)) return;
  cudaDeviceSynchronize();  // buffers may be in use on the caller's stream
  release_acts();
  B_ = B;
  grads_ = grads;
  g_[0][0] = nx;
  g_[0][1] = ny;
  g_[0][2] = nz;
  for (int l = 1; l < 3; ++l)
    for (int d = 0; d < 3; ++d) g_[l][d] = (g_[l - 1][d] - 1) / 2 + 1;
  for (int i = 0; i < NSLOT3; ++i) {
    const int* gd = g_[kSlotLev3[i]];
    const size_t n = (size_t)B * gd[0] * gd[1] * gd[2] * kSlotCh3[i];
    dalloc3(&act_[i], n * 2);
    // padding channels are never written: they must read as zeros
    cuda_ok3(cudaMemset(act_[i], 0, n * 2), "zero activations");
    if (grads) {
      dalloc3(&grd_[i], n * 2);
      cuda_ok3(cudaMemset(grd_[i], 0, n * 2), "zero gradients");
    }
  }
  dalloc3(&y32_, (size_t)B * nx * ny * nz * 8 * 4);
  if (!loss_) dalloc3(&loss_, 8);
  // the zero fills run on the legacy stream: complete them before the caller's
  // (non-blocking) stream reads the padding channels
  cuda_ok3(cudaDeviceSynchronize(), "zero activations");
}

float* CoarseNet3::input_staging(int nx, int ny, int nz, int B) {
  const long long need = (long long)B * nx * ny * nz * 4;
  if (need > x4cap_) {
    cudaDeviceSynchronize();
    dfree3(x4_);
    dalloc3(&x4_, need * 4);
    x4cap_ = need;
  }
  return x4_;
}

float* CoarseNet3::scale_staging(int B) {
  if (B > scalecap_) {
    cudaDeviceSynchronize();
    dfree3(scale_);
    dalloc3(&scale_, (size_t)B * 4);
    scalecap_ = B;
  }
  return scale_;
}

// The tensor-core path: N = Cout rounded up to 16 (the 8-channel layers compute
// 8 zero channels more and store 8), the weights as images (hz_conv_tc.cu), tiles
// of 8 x 16 nodes per z-plane and z-line tiles for the last y-rows of a plane.
// tc_waste: the MMA work over the useful work on a grid level (partial tiles
// times the padding of N); the default path takes the tensor cores where it is
// at most 3.5.  On a 33^3 x 32 batch every layer ran faster on the tensor cores
// (waste 1.5-3.2: 96, 30, 14, 93, 205 and 96 us against 192, 45, 16, 105, 335
// and 191 us warp-level); a 5^3 level (waste 5.1) stays warp-level.
static double tc_waste(const int* gd, int Cout) {
  const int nx = gd[0], ny = gd[1], nz = gd[2];
  const double wx = (nx + 7) / 8 * 8.0 / nx;
  const int y0z = ny / 16 * 16;
  const double wyz = (y0z + (ny - y0z) * ((nz + 15) / 16 * 16.0 / nz)) / ny;
  return wx * wyz * round16(Cout) / (double)Cout;
}

bool CoarseNet3::use_tc(int Cin, int Cout, int lev) const {
  if (conv_path_ == 0 || !conv_tc_supported(kTaps3, Cin, round16(Cout))) return false;
  return conv_path_ == 1 || lev < 0 || tc_waste(g_[lev], Cout) <= 3.5;
}

// Weight images of the forward layers, rewritten on c's stream whenever the BF16
// weights change.
void CoarseNet3::refresh_images(Ctx& c) {
  if (conv_path_ == 0) return;
  if (!wimg_) dalloc3(&wimg_, imgtotal_ * 2);
  for (int l = 0; l < kLayers; ++l) {
    const auto& L = kSpec3[l];
    if (use_tc(L.cinp, L.coutp, -1))  // every layer the path may run on the tensor cores
      conv_tc_weight_image(c, "net3_wimage", kTaps3, L.cinp, round16(L.coutp), wbf_ + woff_[l], 0, 0, L.coutp,
                           wimg_ + imgoff_[l]);
  }
}

void CoarseNet3::set_conv_path(int path) {
  if (path < 0 || path > 2)
    throw std::runtime_error("coarse net 3D: conv path must be 0 (warp MMA), 1 (tcgen05) or 2 (per layer)");
  conv_path_ = path;
  refresh_images(ctx);
  cuda_ok3(cudaStreamSynchronize(ctx.stream), "sync");
}

bool CoarseNet3::tc_failed() {
  int e = 0;
  cuda_ok3(cudaMemcpy(&e, tc_err_, sizeof(int), cudaMemcpyDeviceToHost), "tensor-core status");
  return e != 0;
}

void CoarseNet3::conv_fwd(Ctx& c, int l, int B, const bf16* in, int ldi, int i_off, bf16* out, int ldo, int o_off,
                          int relu, float* out32) {
  const auto& L = kSpec3[l];
  const int* gd = g_[L.lev];
  if (use_tc(L.cinp, L.coutp, L.lev)) {
    const ConvTc a{gd[0], gd[1], gd[2], B, true, L.cinp, in, ldi, i_off, round16(L.coutp), L.coutp,
                   wimg_ + imgoff_[l], out, out32, ldo, o_off, relu, nullptr, 0, 0, 0};
    conv_tc_launch(c, "net3_conv_fwd_tc", a, tc_err_);
    return;
  }
  conv3_launch(c, "net3_conv_fwd", gd, B, L.cinp, in, ldi, i_off, L.coutp, wbf_ + woff_[l], out, out32, ldo, o_off,
               relu, nullptr, 0, 0, 0);
}

void CoarseNet3::forward(Ctx& c, const float* x4, int nx, int ny, int nz, int B, bool train) {
  const bool same = nx == g_[0][0] && ny == g_[0][1] && nz == g_[0][2];
  ensure(nx, ny, nz, B, train || (grads_ && same));
  const long long BN0 = (long long)B * nx * ny * nz;
  HZ_LAUNCH(c, "net3_pack_in", (double)BN0 * 48.0, k_pack_in, (unsigned)((BN0 + 255) / 256), 256, 0, BN0,
            reinterpret_cast<const float4*>(x4), act_[X3]);
  // encoder (the skips e0, e1 go straight into the upper channels of C0, C1)
  conv_fwd(c, 0, B, act_[X3], 16, 0, act_[C03], 32, 16, 1, nullptr);
  resample3(c, 0, 0, g_, 0, B, 8, act_[C03], 32, 16, act_[R03], 16, 0, 0);
  conv_fwd(c, 1, B, act_[R03], 16, 0, act_[C13], 48, 32, 1, nullptr);
  resample3(c, 0, 0, g_, 1, B, 16, act_[C13], 48, 32, act_[R13], 16, 0, 0);
  conv_fwd(c, 2, B, act_[R13], 16, 0, act_[E23], 32, 0, 1, nullptr);
  // decoder
  resample3(c, 1, 0, g_, 1, B, 32, act_[E23], 32, 0, act_[C13], 48, 0, 0);
  conv_fwd(c, 3, B, act_[C13], 48, 0, act_[D13], 16, 0, 1, nullptr);
  resample3(c, 1, 0, g_, 0, B, 16, act_[D13], 16, 0, act_[C03], 32, 0, 0);
  conv_fwd(c, 4, B, act_[C03], 32, 0, act_[D03], 16, 0, 1, nullptr);
  conv_fwd(c, 5, B, act_[D03], 16, 0, nullptr, 8, 0, 0, y32_);
}

// Weight gradient of layer l (in: its input, dout: gradient of its output), then
// the data gradient into din (null: skipped), masked for channels >= mask_lo by
// the input activation (ReLU derivative of the skip tensors).
void CoarseNet3::conv_bwd(Ctx& c, int l, int B, const bf16* in, int ldi, const bf16* dout, int ldd, int d_off,
                          bf16* din, int ldn, int n_off, const bf16* mask, int ldm, int mask_lo) {
  const auto& L = kSpec3[l];
  const int* gd = g_[L.lev];
  const long long nodes = (long long)gd[0] * gd[1] * gd[2] * B;
  if (L.cinp % 8 || L.cinp > 48 || L.coutp > 32 || ldi % 8 || ldd % 8 || d_off % 8)
    throw std::runtime_error("coarse net 3D: weight-gradient layout not supported");
  // the weight gradient on the tensor cores with the tcgen05 path only: the
  // warp-level kernel measured faster (7.47 against 9.95 ms per 33^3 x 32 step)
  if (conv_path_ == 1 && wgrad_tc_supported(kTaps3, L.cinp, L.coutp)) {
    const WgradTc a{gd[0], gd[1], gd[2], nodes, L.cinp, in, ldi, L.coutp, dout, ldd, d_off, g32_ + woff_[l]};
    wgrad_tc_launch(c, "net3_wgrad_tc", a, tc_err_);
  } else {
    // node range per CTA: a few waves of (27 taps x chunks) CTAs, few atomics
    long long kc = (nodes + 44) / 45;
    kc = std::max<long long>(kWg3KS, (kc + kWg3KS - 1) / kWg3KS * kWg3KS);
    const long long nch = (nodes + kc - 1) / kc;
    if (nch > 65535) throw std::runtime_error("coarse net 3D: batch too large for the weight gradient");
    const dim3 grid(1u, (unsigned)nch, 27u);
    const size_t smem = (size_t)kWg3KS * ((L.cinp + 8) + (round16(L.coutp) + 8)) * 2;
    c.add_flops("net3_wgrad", 2.0 * 27.0 * L.cinp * L.coutp * (double)nodes);
    HZ_LAUNCH(c, "net3_wgrad", (double)nodes * (L.cinp + L.coutp) * 2.0 * 27.0, k_wgrad3_mma, grid, 128, smem,
              gd[0], gd[1], gd[2], nodes, L.cinp, L.coutp, in, ldi, dout, ldd, d_off, g32_ + woff_[l], kc);
  }
  if (!din) return;
  const int K = round16(L.coutp);
  const int tot = L.cinp * kTaps3 * K;
  if (use_tc(K, L.cinp, L.lev)) {
    conv_tc_weight_image(c, "net3_wflip", kTaps3, K, L.cinp, wbf_ + woff_[l], 1, L.cinp, L.coutp, wt_);
    const ConvTc a{gd[0], gd[1], gd[2], B, true, K, dout, ldd, d_off, L.cinp, L.cinp, wt_, din, nullptr, ldn, n_off,
                   0, mask, ldm, 0, mask_lo};
    conv_tc_launch(c, "net3_conv_bwd_tc", a, tc_err_);
    return;
  }
  HZ_LAUNCH(c, "net3_wflip", (double)tot * 4.0, k_wflip3, (unsigned)((tot + 255) / 256), 256, 0, L.coutp, L.cinp, K,
            wbf_ + woff_[l], wt_);
  conv3_launch(c, "net3_conv_bwd", gd, B, K, dout, ldd, d_off, L.cinp, wt_, din, nullptr, ldn, n_off, 0, mask, ldm,
               0, mask_lo);
}

double CoarseNet3::backward(Ctx& c, const float* t, int nx, int ny, int nz, int B) {
  if (nx != g_[0][0] || ny != g_[0][1] || nz != g_[0][2] || B > B_ || !grads_)
    throw std::runtime_error("coarse net 3D: backward needs forward");
  if (!wt_) {
    long long mx = 0;
    for (const auto& L : kSpec3) mx = std::max(mx, (long long)L.cinp * kTaps3 * round16(L.coutp));
    dalloc3(&wt_, mx * 2);
  }
  const int N0 = nx * ny * nz;
  cuda_ok3(cudaMemsetAsync(loss_, 0, 8, c.stream), "loss reset");
  cuda_ok3(cudaMemsetAsync(g32_, 0, wtotal_ * 4, c.stream), "grad reset");
  bf16* gY = grd_[X3];  // the input needs no gradient: its slot holds dL/dy (16 channels)
  HZ_LAUNCH(c, "net3_loss", (double)N0 * B * 72.0, k_loss, B, 256, 0, N0, B, y32_, t, gY, loss_);
  conv_bwd(c, 5, B, act_[D03], 16, gY, 16, 0, grd_[D03], 16, 0, act_[D03], 16, 0);
  conv_bwd(c, 4, B, act_[C03], 32, grd_[D03], 16, 0, grd_[C03], 32, 0, act_[C03], 32, 16);
  resample3(c, 1, 1, g_, 0, B, 16, grd_[C03], 32, 0, grd_[D13], 16, 0, 0, act_[D13], 16, 0);
  conv_bwd(c, 3, B, act_[C13], 48, grd_[D13], 16, 0, grd_[C13], 48, 0, act_[C13], 48, 32);
  resample3(c, 1, 1, g_, 1, B, 32, grd_[C13], 48, 0, grd_[E23], 32, 0, 0, act_[E23], 32, 0);
  conv_bwd(c, 2, B, act_[R13], 16, grd_[E23], 32, 0, grd_[R13], 16, 0, nullptr, 0, 0);
  resample3(c, 0, 1, g_, 1, B, 16, grd_[R13], 16, 0, grd_[C13], 48, 32, 1, act_[C13], 48, 32);
  conv_bwd(c, 1, B, act_[R03], 16, grd_[C13], 48, 32, grd_[R03], 16, 0, nullptr, 0, 0);
  resample3(c, 0, 1, g_, 0, B, 8, grd_[R03], 16, 0, grd_[C03], 32, 16, 1, act_[C03], 32, 16);
  conv_bwd(c, 0, B, act_[X3], 16, grd_[C03], 32, 16, nullptr, 0, 0, nullptr, 0, 0);
  double l = 0.0;
  cuda_ok3(cudaMemcpyAsync(&l, loss_, 8, cudaMemcpyDeviceToHost, c.stream), "loss");
  cuda_ok3(cudaStreamSynchronize(c.stream), "sync");
  c.resolve();
  if (conv_path_ != 0 && tc_failed()) throw std::runtime_error("coarse net 3D: tensor-core convolution timed out");
  return l;
}

void CoarseNet3::adam(Ctx& c, double lr) {
  ++step_;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)step_), c2 = 1.f - std::pow(b2, (float)step_);
  HZ_LAUNCH(c, "net3_adam", (double)wtotal_ * 22.0, k_adam, 304, 256, 0, wtotal_, w32_, g32_, m_, v_, wbf_, (float)lr,
            b1, b2, 1e-8f, c1, c2);
  refresh_images(c);
}

void CoarseNet3::train(Ctx& c, const float* x, const float* t, int nx, int ny, int nz, long long nsamples, int batch,
                       int epochs, double lr, unsigned seed, double* loss_hist) {
  if (batch < 1 || nsamples < 1 || epochs < 1) throw std::runtime_error("coarse net 3D: bad training sizes");
  if (nsamples >= (1LL << 31)) throw std::runtime_error("coarse net 3D: too many training pairs");
  batch = (int)std::min<long long>(batch, nsamples);
  const long long N = (long long)nx * ny * nz;
  if ((long long)batch * N * 4 > bcap_) {
    cudaDeviceSynchronize();
    dfree3(bx_);
    dfree3(bt_);
    dalloc3(&bx_, (size_t)batch * N * 16);
    dalloc3(&bt_, (size_t)batch * N * 8);
    bcap_ = (long long)batch * N * 4;
  }
  cudaDeviceSynchronize();
  dfree3(perm_);
  dalloc3(&perm_, (size_t)nsamples * sizeof(int));
  ensure(nx, ny, nz, batch, true);
  std::mt19937 rng(seed);
  std::vector<int> perm((size_t)nsamples);
  const long long steps_per_epoch = nsamples / batch;
  const long long total = steps_per_epoch * epochs;
  long long it = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    std::iota(perm.begin(), perm.end(), 0);
    std::shuffle(perm.begin(), perm.end(), rng);
    cuda_ok3(cudaMemcpyAsync(perm_, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream),
             "perm");
    double sum = 0.0;
    for (long long s = 0; s < steps_per_epoch; ++s, ++it) {
      const long long tot = (long long)batch * N;
      HZ_LAUNCH(c, "net3_gather", (double)tot * 48.0, k_gather_pairs, (unsigned)((tot + 255) / 256), 256, 0, batch,
                N, perm_ + s * batch, reinterpret_cast<const float4*>(x), reinterpret_cast<const float2*>(t),
                reinterpret_cast<float4*>(bx_), reinterpret_cast<float2*>(bt_));
      forward(c, bx_, nx, ny, nz, batch, true);
      sum += backward(c, bt_, nx, ny, nz, batch);
      // cosine decay to lr / 20
      const double f = total > 1 ? (double)it / (double)(total - 1) : 1.0;
      adam(c, lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(M_PI * f))));
    }
    if (loss_hist) loss_hist[ep] = sum / (double)std::max<long long>(1, steps_per_epoch);
  }
  cuda_ok3(cudaStreamSynchronize(c.stream), "sync");
  c.resolve();
}

}  // namespace hz
