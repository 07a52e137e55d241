// Learned coarse-grid correction: a small 2D convolutional encoder-decoder
// with BF16 weights and activations and FP32 accumulation, trained on the GPU
// by the kernels of this file, and applied inside the multigrid cycle in place
// of the coarse-grid correction below a chosen level.
//
// Network (grids g0 -> g1 -> g2 -> g3 by node coarsening n -> (n-1)/2+1; NHWC
// activations, channel counts padded to multiples of 16 for the tensor cores):
//   e0 = relu(conv(x,  4 -> 16))          on g0
//   e1 = relu(conv(R e0, 16 -> 32))       on g1     R: full weighting per channel
//   e2 = relu(conv(R e1, 32 -> 64))       on g2
//   e3 = relu(conv(R e2, 64 -> 64))       on g3
//   d2 = relu(conv([P e3, e2], 128 -> 64)) on g2    P: bilinear prolongation per channel
//   d1 = relu(conv([P d2, e1],  96 -> 32)) on g1
//   d0 = relu(conv([P d1, e0],  48 -> 16)) on g0
//   y  = conv(d0, 16 -> 2)                on g0     (Re, Im)
// No biases: the map is positively homogeneous, and the solver feeds it the
// residual scaled to unit RMS and scales the output back.  The skip tensors
// e0, e1, e2 are written straight into the upper channels of the concatenation
// buffers, so the decoder needs no copies.
//
// Convolutions (3x3, zero padding) are implicit GEMMs on the tensor cores
// (mma.sync m16n8k16, BF16 x BF16 -> FP32): one warp computes 16 nodes x 8*NT
// output channels, the 9 taps x Cin/16 K-steps reading the input rows and the
// weight rows straight from L1/L2.  The data gradient is the same kernel with
// flipped taps and transposed weights; the weight gradient is an FP32
// reduction over the nodes.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "hz_launch.cuh"
#include "hz_learn.h"

namespace hz {

using bf16 = __nv_bfloat16;

namespace {

struct LayerSpec {
  int cin, cout, cinp, coutp, lev;
};
// the 8 convolutions in forward order; cinp: input channels padded to 16, coutp: outputs padded to 8
constexpr LayerSpec kSpec[CoarseNet::kLayers] = {
    {4, 16, 16, 16, 0},    {16, 32, 16, 32, 1}, {32, 64, 32, 64, 2}, {64, 64, 64, 64, 3},
    {128, 64, 128, 64, 2}, {96, 32, 96, 32, 1}, {48, 16, 48, 16, 0}, {16, 2, 16, 8, 0},
};
inline int round16(int c) { return (c + 15) / 16 * 16; }

// activation slots: buffer, grid level and channel count
enum Slot { X = 0, C0, R0, C1, R1, C2, R2, E3, D2, D1, D0, NSLOT };
constexpr int kSlotLev[NSLOT] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 1, 0};
constexpr int kSlotCh[NSLOT] = {16, 48, 16, 96, 32, 128, 64, 64, 64, 32, 16};

}  // namespace

// ---------------------------------------------------------------------------
// conv3x3 on the tensor cores
//   in  [B][N] rows of ldi bf16, channels i_off .. i_off+Cin (Cin multiple of 16)
//   w   [Cout][9][Cin] bf16
//   out [B][N] rows of ldo, channels o_off + co (bf16, or FP32 into out32)
// epilogue: optional ReLU; optional mask: zero where mask[row*ldm + m_off + co] <= 0
// for co >= mask_lo.  grid.z splits Cout in chunks of 8*NT.
//
// A CTA (4 warps) owns 64 consecutive nodes of one sample.  Per 16-channel
// chunk it stages, with 16-byte loads, the three strips of input rows the
// 3x3 taps reach (66 rows each: rows p0 + dy*nx - 1 .. p0 + dy*nx + 64) and
// the chunk of the weights, then every warp runs 9 taps x NT MMAs for its 16
// nodes.  Shared rows are padded to 24 bf16 (12 words), so the 8 rows of a
// fragment load start in 8 different bank groups.  Taps that leave the grid
// read zeros (checked per node and tap), which is the zero padding.
// ---------------------------------------------------------------------------
constexpr int kConvTile = 64;               // nodes per CTA
constexpr int kConvStrip = kConvTile + 2;   // rows per strip
constexpr int kConvCK = 16;                 // channels per staged chunk
constexpr int kConvSR = kConvCK + 8;        // padded shared row (bf16)

// ldmatrix: four (two) 8x8 b16 matrices from shared memory, rows addressed by
// lanes 0-7, 8-15, 16-23, 24-31 (0-7, 8-15); lane l receives row l/4, columns
// 2(l%4), 2(l%4)+1 of matrix i in register i -- the m16n8k16 fragment layout.
__device__ __forceinline__ void ldsm_x4(const bf16* p, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void ldsm_x2(const bf16* p, unsigned& r0, unsigned& r1) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}

template <int NT>
__global__ void __launch_bounds__(128) k_conv_mma(int nx, int ny, int Cin, int Cout, const bf16* __restrict__ in,
                                                  int ldi, int i_off, const bf16* __restrict__ w,
                                                  bf16* __restrict__ out, float* __restrict__ out32, int ldo,
                                                  int o_off, int relu, const bf16* __restrict__ mask, int ldm,
                                                  int m_off, int mask_lo) {
  __shared__ __align__(16) bf16 s_in[3 * kConvStrip * kConvSR];
  __shared__ __align__(16) bf16 s_w[8 * NT * 9 * kConvSR];
  const int N = nx * ny;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int p0 = blockIdx.x * kConvTile;
  const int bidx = blockIdx.y;
  const int co0 = blockIdx.z * 8 * NT;
  const int g = lane >> 2, tq = lane & 3;
  const int la = warp * 16 + g;  // local node of fragment rows g (and g + 8)
  const int pa = p0 + la, pb = pa + 8;
  const bool active = p0 + warp * 16 < N;
  // per-tap validity of the two nodes (bit t)
  unsigned ma = 0u, mb = 0u;
  {
    const int ia = pa % nx, ja = pa / nx, ib = pb % nx, jb = pb / nx;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int dx = t % 3 - 1, dy = t / 3 - 1;
      if (pa < N && ia + dx >= 0 && ia + dx < nx && ja + dy >= 0 && ja + dy < ny) ma |= 1u << t;
      if (pb < N && ib + dx >= 0 && ib + dx < nx && jb + dy >= 0 && jb + dy < ny) mb |= 1u << t;
    }
  }
  const bf16* inb = in + (long long)bidx * N * ldi + i_off;
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  float acc[NT][4];
#pragma unroll
  for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
  for (int c0 = 0; c0 < Cin; c0 += kConvCK) {
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * kConvStrip * 2; e += blockDim.x) {
      const int h = e & 1, rr = e >> 1;
      const int sidx = rr / kConvStrip, k = rr % kConvStrip;
      const int gr = p0 + (sidx - 1) * nx - 1 + k;
      uint4 v = zero;
      if (gr >= 0 && gr < N) v = *reinterpret_cast<const uint4*>(inb + (long long)gr * ldi + c0 + 8 * h);
      *reinterpret_cast<uint4*>(s_in + rr * kConvSR + 8 * h) = v;
    }
    for (int e = threadIdx.x; e < 8 * NT * 9 * 2; e += blockDim.x) {
      const int h = e & 1, rr = e >> 1;
      const int co = rr / 9, t = rr % 9;
      uint4 v = zero;
      if (co0 + co < Cout) v = *reinterpret_cast<const uint4*>(w + ((long long)(co0 + co) * 9 + t) * Cin + c0 + 8 * h);
      *reinterpret_cast<uint4*>(s_w + rr * kConvSR + 8 * h) = v;
    }
    __syncthreads();
    if (active) {
      // ldmatrix row addresses of this lane: A matrix m = lane/8 covers nodes
      // warp*16 + 8(m&1) + lane%8 and channels 8(m>>1)..; B matrix m covers the
      // weight rows of output channel 8(n + (m>>1)) + lane%8, channels 8(m&1)..
      const int lm = lane >> 3, lr = lane & 7;
      const int a_node = warp * 16 + (lm & 1) * 8 + lr;
      const int a_col = (lm >> 1) * 8;
      const int b_row = (lm >> 1) * 8 + lr;
      const int b_col = (lm & 1) * 8;
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int dx = t % 3 - 1, dy = t / 3 - 1;
        unsigned a0, a1, a2, a3;
        ldsm_x4(s_in + ((dy + 1) * kConvStrip + a_node + dx + 1) * kConvSR + a_col, a0, a1, a2, a3);
        // lane's A rows are its own nodes pa (a0, a2) and pb (a1, a3): zero the taps off the grid
        if (!((ma >> t) & 1u)) a0 = a2 = 0u;
        if (!((mb >> t) & 1u)) a1 = a3 = 0u;
#pragma unroll
        for (int n = 0; n < NT; n += 2) {
          unsigned b0, b1, b2 = 0u, b3 = 0u;
          if (n + 1 < NT)
            ldsm_x4(s_w + ((n * 8 + b_row) * 9 + t) * kConvSR + b_col, b0, b1, b2, b3);
          else
            ldsm_x2(s_w + ((n * 8 + (lr & 7)) * 9 + t) * kConvSR + (lm & 1) * 8, b0, b1);
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
              "{%0,%1,%2,%3};\n"
              : "+f"(acc[n][0]), "+f"(acc[n][1]), "+f"(acc[n][2]), "+f"(acc[n][3])
              : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
          if (n + 1 < NT)
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(acc[n + 1][0]), "+f"(acc[n + 1][1]), "+f"(acc[n + 1][2]), "+f"(acc[n + 1][3])
                : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b2), "r"(b3));
        }
      }
    }
  }
  if (!active) return;
#pragma unroll
  for (int n = 0; n < NT; ++n) {
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int p = hh ? pb : pa;
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

static void conv_launch(Ctx& ctx, const char* name, int nx, int ny, int B, int Cin, const bf16* in, int ldi,
                        int i_off, int Cout, const bf16* w, bf16* out, float* out32, int ldo, int o_off, int relu,
                        const bf16* mask, int ldm, int m_off, int mask_lo) {
  if (Cin % 16 != 0 || (ldi % 8) || (i_off % 8) || (Cin % 16))
    throw std::runtime_error("conv: channel layout not aligned");
  const int N = nx * ny;
  const int NT = Cout <= 8 ? 1 : Cout <= 16 ? 2 : Cout <= 32 ? 4 : 8;
  const dim3 grid((unsigned)((N + kConvTile - 1) / kConvTile), (unsigned)B, (unsigned)((Cout + 8 * NT - 1) / (8 * NT)));
  const double bytes = (double)B * N * (Cin * 2.0 + Cout * (out32 ? 4.0 : 2.0)) + 9.0 * Cin * Cout * 2.0;
  ctx.add_flops(name, 2.0 * 9.0 * Cin * Cout * (double)N * B);
  switch (NT) {
    case 1:
      HZ_LAUNCH(ctx, name, bytes, k_conv_mma<1>, grid, 128, 0, nx, ny, Cin, Cout, in, ldi, i_off, w, out, out32, ldo,
                o_off, relu, mask, ldm, m_off, mask_lo);
      break;
    case 2:
      HZ_LAUNCH(ctx, name, bytes, k_conv_mma<2>, grid, 128, 0, nx, ny, Cin, Cout, in, ldi, i_off, w, out, out32, ldo,
                o_off, relu, mask, ldm, m_off, mask_lo);
      break;
    case 4:
      HZ_LAUNCH(ctx, name, bytes, k_conv_mma<4>, grid, 128, 0, nx, ny, Cin, Cout, in, ldi, i_off, w, out, out32, ldo,
                o_off, relu, mask, ldm, m_off, mask_lo);
      break;
    default:
      HZ_LAUNCH(ctx, name, bytes, k_conv_mma<8>, grid, 128, 0, nx, ny, Cin, Cout, in, ldi, i_off, w, out, out32, ldo,
                o_off, relu, mask, ldm, m_off, mask_lo);
      break;
  }
}

// weights of the data-gradient convolution: wt[ci][t][co] = w[co][8 - t][ci],
// co padded from Cout to K (zero rows)
__global__ void k_wflip(int Cout, int Cin, int K, const bf16* __restrict__ w, bf16* __restrict__ wt) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= Cin * 9 * K) return;
  const int co = idx % K, t = (idx / K) % 9, ci = idx / (K * 9);
  wt[idx] = (co < Cout) ? w[((long long)co * 9 + (8 - t)) * Cin + ci] : __float2bfloat16_rn(0.f);
}

// Weight gradient on the tensor cores: dw[co][t][ci] += sum_n dout[n][co] * in[n + off_t][ci],
// a GEMM with M = Cout, N = Cin and K = the nodes.  One CTA (4 warps) owns one
// tap t (blockIdx.z) and a range of kc nodes (blockIdx.y); it stages KS-node
// slices of the input rows (zeroed where the tap leaves the grid, so the
// zero padding is exact) and of the output-gradient rows in shared memory,
// runs m16n8k16 MMAs over 16-node K-steps (warp w owns the 16x8 output tiles
// w, w+4, ...), and adds its partial sums to dw with one atomic per weight.
// Row strides in shared memory are padded by 8 bf16 so the four node rows a
// fragment load touches fall in different banks.
constexpr int kWgKS = 64;        // nodes per staged slice
constexpr int kWgMaxTiles = 16;  // 16x8 tiles per warp (Cout <= 64, Cin <= 128)

__device__ __forceinline__ unsigned pack2(bf16 lo, bf16 hi) {
  return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

__global__ void __launch_bounds__(128) k_wgrad_mma(int nx, int ny, int total, int Cin, int Cout,
                                                   const bf16* __restrict__ in, int ldi, const bf16* __restrict__ dout,
                                                   int ldd, int d_off, float* __restrict__ dw, int kc) {
  extern __shared__ __align__(16) unsigned char wg_smem[];
  const int N = nx * ny;
  const int t = blockIdx.z;
  const int dx = t % 3 - 1, dy = t / 3 - 1;
  const int C16 = (Cout + 15) / 16 * 16;
  const int sIn = Cin + 8, sD = C16 + 8;
  bf16* s_in = reinterpret_cast<bf16*>(wg_smem);
  bf16* s_d = s_in + kWgKS * sIn;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tq = lane & 3;
  const int NTn = Cin / 8, T = (C16 / 16) * NTn;
  float acc[kWgMaxTiles][4];
#pragma unroll
  for (int k = 0; k < kWgMaxTiles; ++k) acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.f;
  const int q0 = blockIdx.y * kc;
  const int q1 = min(total, q0 + kc);
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  for (int qs = q0; qs < q1; qs += kWgKS) {
    __syncthreads();
    const int cin8 = Cin / 8, cd8 = C16 / 8;
    for (int e = threadIdx.x; e < kWgKS * cin8; e += blockDim.x) {
      const int r = e / cin8, c8 = e % cin8;
      const int q = qs + r;
      uint4 v = zero;
      if (q < q1) {
        const int p = q % N;
        const int i = p % nx + dx, j = p / nx + dy;
        if (i >= 0 && i < nx && j >= 0 && j < ny)
          v = *reinterpret_cast<const uint4*>(in + (long long)(q + dx + dy * nx) * ldi + c8 * 8);
      }
      *reinterpret_cast<uint4*>(s_in + r * sIn + c8 * 8) = v;
    }
    for (int e = threadIdx.x; e < kWgKS * cd8; e += blockDim.x) {
      const int r = e / cd8, c8 = e % cd8;
      const int q = qs + r;
      uint4 v = zero;
      if (q < q1 && c8 * 8 < Cout) v = *reinterpret_cast<const uint4*>(dout + (long long)q * ldd + d_off + c8 * 8);
      *reinterpret_cast<uint4*>(s_d + r * sD + c8 * 8) = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int kb = 0; kb < kWgKS; kb += 16) {
      const bf16* d0 = s_d + (kb + tq * 2) * sD;
      const bf16* i0 = s_in + (kb + tq * 2) * sIn;
#pragma unroll
      for (int k = 0; k < kWgMaxTiles; ++k) {
        const int tile = warp + 4 * k;
        if (tile < T) {
          const int co = (tile / NTn) * 16 + g;
          const int ci = (tile % NTn) * 8 + g;
          const unsigned a0 = pack2(d0[co], d0[sD + co]);
          const unsigned a1 = pack2(d0[co + 8], d0[sD + co + 8]);
          const unsigned a2 = pack2(d0[8 * sD + co], d0[9 * sD + co]);
          const unsigned a3 = pack2(d0[8 * sD + co + 8], d0[9 * sD + co + 8]);
          const unsigned b0 = pack2(i0[ci], i0[sIn + ci]);
          const unsigned b1 = pack2(i0[8 * sIn + ci], i0[9 * sIn + ci]);
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
              "{%0,%1,%2,%3};\n"
              : "+f"(acc[k][0]), "+f"(acc[k][1]), "+f"(acc[k][2]), "+f"(acc[k][3])
              : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kWgMaxTiles; ++k) {
    const int tile = warp + 4 * k;
    if (tile >= T) break;
    const int co = (tile / NTn) * 16 + g;
    const int ci = (tile % NTn) * 8 + tq * 2;
    if (co < Cout) {
      atomicAdd(&dw[((long long)co * 9 + t) * Cin + ci], acc[k][0]);
      atomicAdd(&dw[((long long)co * 9 + t) * Cin + ci + 1], acc[k][1]);
    }
    if (co + 8 < Cout) {
      atomicAdd(&dw[((long long)(co + 8) * 9 + t) * Cin + ci], acc[k][2]);
      atomicAdd(&dw[((long long)(co + 8) * 9 + t) * Cin + ci + 1], acc[k][3]);
    }
  }
}

// Per-channel resampling between grid levels (NHWC bf16, FP32 arithmetic).
// mode 0, restriction (fine -> coarse): full weighting with weights 1, 1/2 per
// axis, normalised by the weights that fall inside the grid.
// mode 1, prolongation (coarse -> fine): bilinear, (c[i0] + c[i1]) / 2 per axis
// with i0 = i / 2, i1 = (i + 1) / 2.
// transpose = 1 applies the adjoint (fine <- coarse for mode 0, coarse <- fine for
// mode 1).  The result, zeroed where mask <= 0 (mask may be null), is written or,
// with accum, added to out (rounded to bf16 once).

// One thread per (node, 8 channels): 16-byte loads and stores (every channel
// count and offset is a multiple of 8).
struct F8 {
  float v[8];
};
__device__ __forceinline__ void ld8(const bf16* p, F8& f) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float2 x = __bfloat1622float2(h[k]);
    f.v[2 * k] = x.x;
    f.v[2 * k + 1] = x.y;
  }
}
__device__ __forceinline__ void axpy8(float a, const bf16* p, F8& acc) {
  F8 f;
  ld8(p, f);
#pragma unroll
  for (int k = 0; k < 8; ++k) acc.v[k] = fmaf(a, f.v[k], acc.v[k]);
}

__global__ void k_resample(int mode, int transpose, int nxf, int nyf, int nxc, int nyc, int B, int C,
                           const bf16* __restrict__ in, int ldi, int i_off, bf16* __restrict__ out, int ldo, int o_off,
                           int accum, const bf16* __restrict__ mask, int ldm, int m_off) {
  const int Nf = nxf * nyf, Nc = nxc * nyc;
  const bool to_coarse = (mode == 0) != (transpose != 0);
  const int No = to_coarse ? Nc : Nf, Ni = to_coarse ? Nf : Nc;
  const int C8 = C / 8;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * No * C8) return;
  const int c = (idx % C8) * 8;
  const int q = idx / C8;
  const int b = q / No, po = q % No;
  const bf16* ib = in + (long long)b * Ni * ldi + i_off + c;
  F8 acc;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc.v[k] = 0.f;
  if (mode == 0 && !transpose) {  // restriction
    const int I = po % nxc, J = po / nxc;
    float wsum = 0.f;
    for (int dj = -1; dj <= 1; ++dj)
      for (int di = -1; di <= 1; ++di) {
        const int fi = 2 * I + di, fj = 2 * J + dj;
        if (fi < 0 || fi >= nxf || fj < 0 || fj >= nyf) continue;
        const float wg = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f);
        axpy8(wg, ib + (long long)(fi + fj * nxf) * ldi, acc);
        wsum += wg;
      }
    const float inv = 1.f / wsum;
#pragma unroll
    for (int k = 0; k < 8; ++k) acc.v[k] *= inv;
  } else if (mode == 0) {  // adjoint of the restriction: fine <- coarse parents I with |i - 2I| <= 1
    const int i = po % nxf, j = po / nxf;
    for (int J = j / 2 - 1; J <= j / 2 + 1; ++J)
      for (int I = i / 2 - 1; I <= i / 2 + 1; ++I) {
        if (I < 0 || I >= nxc || J < 0 || J >= nyc) continue;
        const int di = i - 2 * I, dj = j - 2 * J;
        if (di < -1 || di > 1 || dj < -1 || dj > 1) continue;
        const float sx = 1.f + (2 * I - 1 >= 0 ? 0.5f : 0.f) + (2 * I + 1 < nxf ? 0.5f : 0.f);
        const float sy = 1.f + (2 * J - 1 >= 0 ? 0.5f : 0.f) + (2 * J + 1 < nyf ? 0.5f : 0.f);
        axpy8((di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) / (sx * sy), ib + (long long)(I + J * nxc) * ldi, acc);
      }
  } else if (!transpose) {  // prolongation
    const int i = po % nxf, j = po / nxf;
    const int i0 = i >> 1, i1 = (i + 1) >> 1, j0 = j >> 1, j1 = (j + 1) >> 1;
    axpy8(1.f, ib + (long long)(i0 + j0 * nxc) * ldi, acc);
    axpy8(1.f, ib + (long long)(i1 + j0 * nxc) * ldi, acc);
    axpy8(1.f, ib + (long long)(i0 + j1 * nxc) * ldi, acc);
    axpy8(1.f, ib + (long long)(i1 + j1 * nxc) * ldi, acc);
#pragma unroll
    for (int k = 0; k < 8; ++k) acc.v[k] *= 0.25f;
  } else {  // adjoint of the prolongation: coarse <- fine children
    const int I = po % nxc, J = po / nxc;
    for (int fj = 2 * J - 1; fj <= 2 * J + 1; ++fj)
      for (int fi = 2 * I - 1; fi <= 2 * I + 1; ++fi) {
        if (fi < 0 || fi >= nxf || fj < 0 || fj >= nyf) continue;
        axpy8((fi == 2 * I ? 1.f : 0.5f) * (fj == 2 * J ? 1.f : 0.5f), ib + (long long)(fi + fj * nxf) * ldi, acc);
      }
  }
  const long long row = (long long)b * No + po;
  if (mask) {
    F8 mk;
    ld8(mask + row * ldm + m_off + c, mk);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (!(mk.v[k] > 0.f)) acc.v[k] = 0.f;
  }
  bf16* o = out + row * ldo + o_off + c;
  if (accum) {
    F8 old;
    ld8(o, old);
#pragma unroll
    for (int k = 0; k < 8; ++k) acc.v[k] += old.v[k];
  }
  __align__(16) __nv_bfloat162 r[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) r[k] = __floats2bfloat162_rn(acc.v[2 * k], acc.v[2 * k + 1]);
  *reinterpret_cast<uint4*>(o) = *reinterpret_cast<const uint4*>(r);
}

static void resample(Ctx& ctx, int mode, int transpose, const int* gx, const int* gy, int lf, int B, int C,
                     const bf16* in, int ldi, int i_off, bf16* out, int ldo, int o_off, int accum,
                     const bf16* mask = nullptr, int ldm = 0, int m_off = 0) {
  if (C % 8 || ldi % 8 || i_off % 8 || ldo % 8 || o_off % 8 || (mask && (ldm % 8 || m_off % 8)))
    throw std::runtime_error("resample: channel layout not aligned");
  const int nxf = gx[lf], nyf = gy[lf], nxc = gx[lf + 1], nyc = gy[lf + 1];
  const bool to_coarse = (mode == 0) != (transpose != 0);
  const long long no = to_coarse ? (long long)nxc * nyc : (long long)nxf * nyf;
  const long long ni = to_coarse ? (long long)nxf * nyf : (long long)nxc * nyc;
  const long long total = (long long)B * no * (C / 8);
  if (total >= (1LL << 31)) throw std::runtime_error("resample: batch too large");
  HZ_LAUNCH(ctx, "net_resample", (double)B * (no + ni) * C * 2.0, k_resample, (unsigned)((total + 255) / 256), 256, 0,
            mode, transpose, nxf, nyf, nxc, nyc, B, C, in, ldi, i_off, out, ldo, o_off, accum, mask, ldm, m_off);
}

// input assembly: X[b][p][0..16) = (x4[b][p][0..4), 0...) in bf16
__global__ void k_pack_in(long long BN, const float4* __restrict__ x4, bf16* __restrict__ x16) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= BN) return;
  const float4 v = x4[i];
  __align__(16) __nv_bfloat162 q[8];
  q[0] = __floats2bfloat162_rn(v.x, v.y);
  q[1] = __floats2bfloat162_rn(v.z, v.w);
#pragma unroll
  for (int k = 2; k < 8; ++k) q[k] = __floats2bfloat162_rn(0.f, 0.f);
  uint4* dst = reinterpret_cast<uint4*>(x16 + i * 16);
  dst[0] = *reinterpret_cast<uint4*>(&q[0]);
  dst[1] = *reinterpret_cast<uint4*>(&q[4]);
}

// loss_b = ||y_b - t_b||^2 / ||t_b||^2 (channels 0, 1 of y) accumulated as the
// batch mean into *loss, and the output gradient dy = 2 (y - t) / ||t_b||^2 / B
// as bf16 into 16-channel rows (channels 2..15 zero).
__global__ void __launch_bounds__(256) k_loss(int N, int B, const float* __restrict__ y, const float* __restrict__ t,
                                              bf16* __restrict__ dy, double* __restrict__ loss) {
  const int b = blockIdx.x;
  __shared__ double sh_e[256], sh_t[256];
  double e = 0.0, tt = 0.0;
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    const long long r = (long long)b * N + p;
    for (int c = 0; c < 2; ++c) {
      const double tv = t[r * 2 + c];
      const double d = (double)y[r * 8 + c] - tv;
      e += d * d;
      tt += tv * tv;
    }
  }
  sh_e[threadIdx.x] = e;
  sh_t[threadIdx.x] = tt;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh_e[threadIdx.x] += sh_e[threadIdx.x + s];
      sh_t[threadIdx.x] += sh_t[threadIdx.x + s];
    }
    __syncthreads();
  }
  const double tn = sh_t[0] > 0.0 ? sh_t[0] : 1.0;
  if (threadIdx.x == 0) atomicAdd(loss, sh_e[0] / tn / B);
  const double sc = 2.0 / tn / B;
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    const long long r = (long long)b * N + p;
    __align__(16) __nv_bfloat162 q[8];
    q[0] = __floats2bfloat162_rn((float)(sc * ((double)y[r * 8] - t[r * 2])),
                                 (float)(sc * ((double)y[r * 8 + 1] - t[r * 2 + 1])));
#pragma unroll
    for (int k = 1; k < 8; ++k) q[k] = __floats2bfloat162_rn(0.f, 0.f);
    uint4* dst = reinterpret_cast<uint4*>(dy + r * 16);
    dst[0] = *reinterpret_cast<uint4*>(&q[0]);
    dst[1] = *reinterpret_cast<uint4*>(&q[4]);
  }
}

// Adam on the FP32 master weights; the BF16 copy is refreshed in the same pass
__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, bf16* __restrict__ wb, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void k_f2bf(long long n, const float* __restrict__ a, bf16* __restrict__ b) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}

// mini-batch gather of training pairs: rows perm[k] of x (4 floats per node) and t (2 per node)
__global__ void k_gather_pairs(int B, long long N, const int* __restrict__ perm, const float4* __restrict__ x,
                               const float2* __restrict__ t, float4* __restrict__ bx, float2* __restrict__ bt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)B * N) return;
  const int k = (int)(i / N);
  const long long p = i % N;
  const long long src = (long long)perm[k] * N + p;
  bx[i] = x[src];
  bt[i] = t[src];
}

// ---------------------------------------------------------------------------
// CoarseNet
// ---------------------------------------------------------------------------
long long CoarseNet::num_params() {
  long long n = 0;
  for (const auto& L : kSpec) n += (long long)L.cout * 9 * L.cin;
  return n;
}

void CoarseNet::layer_shape(int l, int* cin, int* cout) {
  *cin = kSpec[l].cin;
  *cout = kSpec[l].cout;
}

bool CoarseNet::supports(long long nx, long long ny) {
  return nx >= 9 && ny >= 9 && (nx - 1) % 8 == 0 && (ny - 1) % 8 == 0 && nx * ny < (1LL << 30);
}

static void cuda_ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string("coarse net: ") + what + ": " + cudaGetErrorString(e));
  }
}

template <typename P> static void dalloc(P** p, size_t bytes) {
  cuda_ok(cudaMalloc(reinterpret_cast<void**>(p), bytes), "cudaMalloc");
}
template <typename P> static void dfree(P*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

CoarseNet::CoarseNet(unsigned seed) {
  cuda_ok(cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking), "stream");
  long long off = 0;
  for (int l = 0; l < kLayers; ++l) {
    woff_[l] = off;
    off += (long long)kSpec[l].coutp * 9 * kSpec[l].cinp;
  }
  wtotal_ = off;
  dalloc(&w32_, off * 4);
  dalloc(&wbf_, off * 2);
  dalloc(&g32_, off * 4);
  dalloc(&m_, off * 4);
  dalloc(&v_, off * 4);
  dalloc(&tc_err_, sizeof(int));
  cuda_ok(cudaMemset(tc_err_, 0, sizeof(int)), "tensor-core status");
  // He-normal initialisation (last layer scaled down), from a seeded host generator
  std::vector<float> w((size_t)num_params());
  std::mt19937 rng(seed);
  size_t k = 0;
  for (int l = 0; l < kLayers; ++l) {
    const auto& L = kSpec[l];
    std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / (9.0f * L.cin)) * (l == kLayers - 1 ? 0.5f : 1.0f));
    for (long long q = 0; q < (long long)L.cout * 9 * L.cin; ++q) w[k++] = nd(rng);
  }
  set_weights(w.data());
}

CoarseNet::~CoarseNet() {
  release_acts();
  dfree(tc_err_);
  dfree(wimg_);
  dfree(w32_);
  dfree(wbf_);
  dfree(g32_);
  dfree(m_);
  dfree(v_);
  dfree(wt_);
  dfree(x4_);
  dfree(scale_);
  dfree(loss_);
  dfree(bx_);
  dfree(bt_);
  dfree(perm_);
  ctx.release();
  if (ctx.stream) cudaStreamDestroy(ctx.stream);
}

void CoarseNet::set_weights(const float* host) {
  std::vector<float> w((size_t)wtotal_, 0.f);
  size_t k = 0;
  for (int l = 0; l < kLayers; ++l) {
    const auto& L = kSpec[l];
    for (int co = 0; co < L.cout; ++co)
      for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < L.cin; ++ci) w[(size_t)(woff_[l] + ((long long)co * 9 + t) * L.cinp + ci)] = host[k++];
  }
  cuda_ok(cudaStreamSynchronize(ctx.stream), "sync");
  cuda_ok(cudaMemcpy(w32_, w.data(), wtotal_ * 4, cudaMemcpyHostToDevice), "upload weights");
  cuda_ok(cudaMemset(m_, 0, wtotal_ * 4), "adam m");
  cuda_ok(cudaMemset(v_, 0, wtotal_ * 4), "adam v");
  step_ = 0;
  k_f2bf<<<256, 256, 0, ctx.stream>>>(wtotal_, w32_, wbf_);
  cuda_ok(cudaGetLastError(), "weights to bf16");
  refresh_images(ctx);
  cuda_ok(cudaStreamSynchronize(ctx.stream), "sync");
}

static void unpack_padded(const std::vector<float>& w, const long long* woff, float* host) {
  size_t k = 0;
  for (int l = 0; l < CoarseNet::kLayers; ++l) {
    const auto& L = kSpec[l];
    for (int co = 0; co < L.cout; ++co)
      for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < L.cin; ++ci) host[k++] = w[(size_t)(woff[l] + ((long long)co * 9 + t) * L.cinp + ci)];
  }
}

void CoarseNet::get_weights(float* host) const {
  std::vector<float> w((size_t)wtotal_);
  cuda_ok(cudaStreamSynchronize(ctx.stream), "sync");
  cuda_ok(cudaMemcpy(w.data(), w32_, wtotal_ * 4, cudaMemcpyDeviceToHost), "download weights");
  unpack_padded(w, woff_, host);
}

void CoarseNet::get_grad(float* host) const {
  std::vector<float> w((size_t)wtotal_);
  cuda_ok(cudaStreamSynchronize(ctx.stream), "sync");
  cuda_ok(cudaMemcpy(w.data(), g32_, wtotal_ * 4, cudaMemcpyDeviceToHost), "download gradient");
  unpack_padded(w, woff_, host);
}

// ---- file format -----------------------------------------------------------
// "HZCNET01" | u32 version | u32 layers | layers x (i32 cin, i32 cout) |
// i64 nparams | i64 adam step | f32 weights[n] | f32 m[n] | f32 v[n]
// (little-endian; weights and moments unpadded, layer after layer [cout][9][cin])
static const char kNetMagic[8] = {'H', 'Z', 'C', 'N', 'E', 'T', '0', '1'};
static constexpr unsigned kNetVersion = 1;

static void download_unpadded(const float* dev, long long total, const long long* woff, float* host) {
  std::vector<float> w((size_t)total);
  cuda_ok(cudaMemcpy(w.data(), dev, total * 4, cudaMemcpyDeviceToHost), "download");
  unpack_padded(w, woff, host);
}

static void upload_unpadded(const float* host, long long total, const long long* woff, float* dev) {
  std::vector<float> w((size_t)total, 0.f);
  size_t k = 0;
  for (int l = 0; l < CoarseNet::kLayers; ++l) {
    const auto& L = kSpec[l];
    for (int co = 0; co < L.cout; ++co)
      for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < L.cin; ++ci) w[(size_t)(woff[l] + ((long long)co * 9 + t) * L.cinp + ci)] = host[k++];
  }
  cuda_ok(cudaMemcpy(dev, w.data(), total * 4, cudaMemcpyHostToDevice), "upload");
}

void CoarseNet::save(const char* path) const {
  cuda_ok(cudaStreamSynchronize(ctx.stream), "sync");
  const long long n = num_params();
  std::vector<float> w((size_t)n), m((size_t)n), v((size_t)n);
  download_unpadded(w32_, wtotal_, woff_, w.data());
  download_unpadded(m_, wtotal_, woff_, m.data());
  download_unpadded(v_, wtotal_, woff_, v.data());
  FILE* f = std::fopen(path, "wb");
  if (!f) throw std::runtime_error(std::string("coarse net: cannot write ") + path);
  const unsigned hdr[2] = {kNetVersion, (unsigned)kLayers};
  bool ok = std::fwrite(kNetMagic, 1, 8, f) == 8 && std::fwrite(hdr, 4, 2, f) == 2;
  for (int l = 0; l < kLayers && ok; ++l) {
    const int sh[2] = {kSpec[l].cin, kSpec[l].cout};
    ok = std::fwrite(sh, 4, 2, f) == 2;
  }
  const long long meta[2] = {n, step_};
  ok = ok && std::fwrite(meta, 8, 2, f) == 2;
  ok = ok && std::fwrite(w.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fwrite(m.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fwrite(v.data(), 4, (size_t)n, f) == (size_t)n;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) throw std::runtime_error(std::string("coarse net: write failed: ") + path);
}

int CoarseNet::file_info(const char* path, long long* nparams, long long* step) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return -1;
  char mg[8];
  unsigned hdr[2];
  int rc = 0;
  if (std::fread(mg, 1, 8, f) != 8 || std::memcmp(mg, kNetMagic, 8) != 0) rc = -2;
  if (!rc && std::fread(hdr, 4, 2, f) != 2) rc = -5;
  if (!rc && hdr[0] != kNetVersion) rc = -3;
  if (!rc && hdr[1] != (unsigned)kLayers) rc = -4;
  for (int l = 0; l < kLayers && !rc; ++l) {
    int sh[2];
    if (std::fread(sh, 4, 2, f) != 2) rc = -5;
    else if (sh[0] != kSpec[l].cin || sh[1] != kSpec[l].cout) rc = -4;
  }
  long long meta[2] = {0, 0};
  if (!rc && std::fread(meta, 8, 2, f) != 2) rc = -5;
  if (!rc && meta[0] != num_params()) rc = -4;
  if (!rc) {
    // the three arrays must be present in full
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

void CoarseNet::load(const char* path) {
  long long n = 0, st = 0;
  const int rc = file_info(path, &n, &st);
  static const char* why[] = {"", "cannot read", "not a coarse-network file", "unsupported version",
                              "layer shapes differ", "truncated"};
  if (rc < 0) throw std::runtime_error(std::string("coarse net: ") + path + ": " + why[-rc]);
  std::vector<float> w((size_t)n), m((size_t)n), v((size_t)n);
  FILE* f = std::fopen(path, "rb");
  if (!f) throw std::runtime_error(std::string("coarse net: cannot read ") + path);
  const long hdr_bytes = 8 + 8 + kLayers * 8 + 16;
  bool ok = std::fseek(f, hdr_bytes, SEEK_SET) == 0;
  ok = ok && std::fread(w.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fread(m.data(), 4, (size_t)n, f) == (size_t)n;
  ok = ok && std::fread(v.data(), 4, (size_t)n, f) == (size_t)n;
  std::fclose(f);
  if (!ok) throw std::runtime_error(std::string("coarse net: truncated ") + path);
  for (long long i = 0; i < n; ++i)
    if (!std::isfinite(w[(size_t)i]) || !std::isfinite(m[(size_t)i]) || !(v[(size_t)i] >= 0.f))
      throw std::runtime_error(std::string("coarse net: non-finite weights or state in ") + path);
  set_weights(w.data());  // resets the moments; restore them below
  cuda_ok(cudaStreamSynchronize(ctx.stream), "sync");
  upload_unpadded(m.data(), wtotal_, woff_, m_);
  upload_unpadded(v.data(), wtotal_, woff_, v_);
  step_ = st;
}

void CoarseNet::release_acts() {
  for (int i = 0; i < NSLOT; ++i) {
    dfree(act_[i]);
    dfree(grd_[i]);
  }
  dfree(y32_);
  nx_ = ny_ = B_ = 0;
  grads_ = false;
}

void CoarseNet::ensure(int nx, int ny, int B, bool grads) {
  if (!supports(nx, ny)) throw std::runtime_error("coarse net: grid must have (n - 1) divisible by 8, n >= 9");
  if (nx == nx_ && ny == ny_ && B <= B_ && (grads_ || !grads)) return;
  cudaDeviceSynchronize();  // buffers may be in use on the caller's stream
  release_acts();
  nx_ = nx;
  ny_ = ny;
  B_ = B;
  grads_ = grads;
  gx_[0] = nx;
  gy_[0] = ny;
  for (int l = 1; l < 4; ++l) {
    gx_[l] = (gx_[l - 1] - 1) / 2 + 1;
    gy_[l] = (gy_[l - 1] - 1) / 2 + 1;
  }
  for (int i = 0; i < NSLOT; ++i) {
    const size_t n = (size_t)B * gx_[kSlotLev[i]] * gy_[kSlotLev[i]] * kSlotCh[i];
    dalloc(&act_[i], n * 2);
    if (grads) dalloc(&grd_[i], n * 2);
  }
  dalloc(&y32_, (size_t)B * nx * ny * 8 * 4);
  if (!loss_) dalloc(&loss_, 8);
}

float* CoarseNet::input_staging(int nx, int ny, int B) {
  const long long need = (long long)B * nx * ny * 4;
  if (need > x4cap_) {
    cudaDeviceSynchronize();
    dfree(x4_);
    dalloc(&x4_, need * 4);
    x4cap_ = need;
  }
  return x4_;
}

float* CoarseNet::scale_staging(int B) {
  if (B > scalecap_) {
    cudaDeviceSynchronize();
    dfree(scale_);
    dalloc(&scale_, (size_t)B * 4);
    scalecap_ = B;
  }
  return scale_;
}

// One convolution: on the 5th-generation tensor cores (tcgen05) when that path
// is selected and the channel counts suit it (w is then the layer's weight
// image), else the warp-level MMA kernel.
bool CoarseNet::use_tc(int Cin, int Cout) const { return conv_path_ != 0 && conv_tc_supported(9, Cin, Cout); }

void CoarseNet::conv(Ctx& c, const char* name, int nx, int ny, int B, int Cin, const bf16* in, int ldi, int i_off,
                     int Cout, const bf16* w, bf16* out, float* out32, int ldo, int o_off, int relu, const bf16* mask,
                     int ldm, int m_off, int mask_lo) {
  if (use_tc(Cin, Cout)) {
    const char* tc_name = std::strcmp(name, "net_conv_fwd") == 0 ? "net_conv_fwd_tc" : "net_conv_bwd_tc";
    const ConvTc a{nx, ny, 1, B, false, Cin, in, ldi, i_off, Cout, Cout, w, out, out32, ldo, o_off, relu, mask, ldm,
                   m_off, mask_lo};
    conv_tc_launch(c, tc_name, a, tc_err_);
    return;
  }
  conv_launch(c, name, nx, ny, B, Cin, in, ldi, i_off, Cout, w, out, out32, ldo, o_off, relu, mask, ldm, m_off,
              mask_lo);
}

// Weight images of the forward layers on the tensor-core path, rewritten on c's
// stream whenever the BF16 weights change.
void CoarseNet::refresh_images(Ctx& c) {
  if (conv_path_ == 0) return;
  if (!wimg_) dalloc(&wimg_, wtotal_ * 2);
  for (int l = 0; l < kLayers; ++l) {
    const auto& L = kSpec[l];
    if (use_tc(L.cinp, L.coutp))
      conv_tc_weight_image(c, "net_wimage", 9, L.cinp, L.coutp, wbf_ + woff_[l], 0, 0, L.coutp, wimg_ + woff_[l]);
  }
}

void CoarseNet::set_conv_path(int path) {
  if (path < 0 || path > 2)
    throw std::runtime_error("coarse net: conv path must be 0 (warp MMA), 1 (tcgen05) or 2 (per layer)");
  conv_path_ = path;
  refresh_images(ctx);
  cuda_ok(cudaStreamSynchronize(ctx.stream), "sync");
}

bool CoarseNet::tc_failed() {
  int e = 0;
  cuda_ok(cudaMemcpy(&e, tc_err_, sizeof(int), cudaMemcpyDeviceToHost), "tensor-core status");
  return e != 0;
}

void CoarseNet::conv_fwd(Ctx& c, int l, int lev, int B, const bf16* in, int ldi, int i_off, bf16* out, int ldo,
                         int o_off, int relu, float* out32) {
  const auto& L = kSpec[l];
  const bf16* w = (use_tc(L.cinp, L.coutp) ? wimg_ : wbf_) + woff_[l];
  conv(c, "net_conv_fwd", gx_[lev], gy_[lev], B, L.cinp, in, ldi, i_off, L.coutp, w, out, out32, ldo, o_off, relu,
       nullptr, 0, 0, 0);
}

void CoarseNet::forward(Ctx& c, const float* x4, int nx, int ny, int B, bool train) {
  ensure(nx, ny, B, train || (grads_ && nx == nx_ && ny == ny_));
  const long long BN0 = (long long)B * nx * ny;
  HZ_LAUNCH(c, "net_pack_in", (double)BN0 * 48.0, k_pack_in, (unsigned)((BN0 + 255) / 256), 256, 0, BN0,
            reinterpret_cast<const float4*>(x4), act_[X]);
  // encoder (skips written into the upper channels of the concatenation buffers)
  conv_fwd(c, 0, 0, B, act_[X], 16, 0, act_[C0], 48, 32, 1, nullptr);
  resample(c, 0, 0, gx_, gy_, 0, B, 16, act_[C0], 48, 32, act_[R0], 16, 0, 0);
  conv_fwd(c, 1, 1, B, act_[R0], 16, 0, act_[C1], 96, 64, 1, nullptr);
  resample(c, 0, 0, gx_, gy_, 1, B, 32, act_[C1], 96, 64, act_[R1], 32, 0, 0);
  conv_fwd(c, 2, 2, B, act_[R1], 32, 0, act_[C2], 128, 64, 1, nullptr);
  resample(c, 0, 0, gx_, gy_, 2, B, 64, act_[C2], 128, 64, act_[R2], 64, 0, 0);
  conv_fwd(c, 3, 3, B, act_[R2], 64, 0, act_[E3], 64, 0, 1, nullptr);
  // decoder
  resample(c, 1, 0, gx_, gy_, 2, B, 64, act_[E3], 64, 0, act_[C2], 128, 0, 0);
  conv_fwd(c, 4, 2, B, act_[C2], 128, 0, act_[D2], 64, 0, 1, nullptr);
  resample(c, 1, 0, gx_, gy_, 1, B, 64, act_[D2], 64, 0, act_[C1], 96, 0, 0);
  conv_fwd(c, 5, 1, B, act_[C1], 96, 0, act_[D1], 32, 0, 1, nullptr);
  resample(c, 1, 0, gx_, gy_, 0, B, 32, act_[D1], 32, 0, act_[C0], 48, 0, 0);
  conv_fwd(c, 6, 0, B, act_[C0], 48, 0, act_[D0], 16, 0, 1, nullptr);
  conv_fwd(c, 7, 0, B, act_[D0], 16, 0, nullptr, 8, 0, 0, y32_);
}

// Weight gradient of layer l (in: its input, dout: gradient of its output), then
// the data gradient into din (null: skipped), masked for channels >= mask_lo by
// the input activation (ReLU derivative of the skip tensors).
void CoarseNet::conv_bwd(Ctx& c, int l, int lev, int B, const bf16* in, int ldi, int i_off, const bf16* dout, int ldd,
                         int d_off, bf16* din, int ldn, int n_off, const bf16* mask, int ldm, int mask_lo) {
  const auto& L = kSpec[l];
  const int nx = gx_[lev], ny = gy_[lev];
  const long long nodes = (long long)nx * ny * B;
  if (nodes >= (1LL << 31)) throw std::runtime_error("coarse net: batch too large for the weight gradient");
  if (L.cinp % 8 || L.cinp > 128 || L.coutp > 64 || ldi % 8 || ldd % 8 || d_off % 8 || i_off != 0)
    throw std::runtime_error("coarse net: weight-gradient layout not supported");
  // node range per CTA: enough CTAs (9 taps x chunks) for a few waves, few atomics
  long long kc = (nodes + 134) / 135;
  kc = std::max<long long>(kWgKS, (kc + kWgKS - 1) / kWgKS * kWgKS);
  // the weight gradient on the tensor cores with the tcgen05 path only: the
  // warp-level kernel measured faster (1.94 against 2.56 ms per 129^2 x 32 step)
  if (conv_path_ == 1 && wgrad_tc_supported(9, L.cinp, L.coutp)) {
    const WgradTc a{nx, ny, 1, nodes, L.cinp, in, ldi, L.coutp, dout, ldd, d_off, g32_ + woff_[l]};
    wgrad_tc_launch(c, "net_wgrad_tc", a, tc_err_);
  } else {
    const dim3 grid(1u, (unsigned)((nodes + kc - 1) / kc), 9u);
    const size_t smem = (size_t)kWgKS * ((L.cinp + 8) + (round16(L.coutp) + 8)) * 2;
    c.add_flops("net_wgrad", 2.0 * 9.0 * L.cinp * L.coutp * (double)nodes);
    HZ_LAUNCH(c, "net_wgrad", (double)nodes * (L.cinp + L.coutp) * 2.0 * 9.0, k_wgrad_mma, grid, 128, smem, nx, ny,
              (int)nodes, L.cinp, L.coutp, in, ldi, dout, ldd, d_off, g32_ + woff_[l], (int)kc);
  }
  if (!din) return;
  const int K = round16(L.coutp);
  const int tot = L.cinp * 9 * K;
  if (use_tc(K, L.cinp)) {
    conv_tc_weight_image(c, "net_wflip", 9, K, L.cinp, wbf_ + woff_[l], 1, L.cinp, L.coutp, wt_);
  } else {
    HZ_LAUNCH(c, "net_wflip", (double)tot * 4.0, k_wflip, (unsigned)((tot + 255) / 256), 256, 0, L.coutp, L.cinp, K,
              wbf_ + woff_[l], wt_);
  }
  conv(c, "net_conv_bwd", nx, ny, B, K, dout, ldd, d_off, L.cinp, wt_, din, nullptr, ldn, n_off, 0, mask, ldm, i_off,
       mask_lo);
}

double CoarseNet::backward(Ctx& c, const float* t, int nx, int ny, int B) {
  if (nx != nx_ || ny != ny_ || B > B_ || !grads_) throw std::runtime_error("coarse net: backward needs forward");
  if (!wt_) {
    long long mx = 0;
    for (const auto& L : kSpec) mx = std::max(mx, (long long)L.cinp * 9 * round16(L.coutp));
    dalloc(&wt_, mx * 2);
  }
  const int N0 = nx * ny;
  cuda_ok(cudaMemsetAsync(loss_, 0, 8, c.stream), "loss reset");
  cuda_ok(cudaMemsetAsync(g32_, 0, wtotal_ * 4, c.stream), "grad reset");
  bf16* gY = grd_[X];  // the input needs no gradient: its slot holds dL/dy (16 channels)
  HZ_LAUNCH(c, "net_loss", (double)N0 * B * 72.0, k_loss, B, 256, 0, N0, B, y32_, t, gY, loss_);
  conv_bwd(c, 7, 0, B, act_[D0], 16, 0, gY, 16, 0, grd_[D0], 16, 0, act_[D0], 16, 0);
  conv_bwd(c, 6, 0, B, act_[C0], 48, 0, grd_[D0], 16, 0, grd_[C0], 48, 0, act_[C0], 48, 32);
  resample(c, 1, 1, gx_, gy_, 0, B, 32, grd_[C0], 48, 0, grd_[D1], 32, 0, 0, act_[D1], 32, 0);
  conv_bwd(c, 5, 1, B, act_[C1], 96, 0, grd_[D1], 32, 0, grd_[C1], 96, 0, act_[C1], 96, 64);
  resample(c, 1, 1, gx_, gy_, 1, B, 64, grd_[C1], 96, 0, grd_[D2], 64, 0, 0, act_[D2], 64, 0);
  conv_bwd(c, 4, 2, B, act_[C2], 128, 0, grd_[D2], 64, 0, grd_[C2], 128, 0, act_[C2], 128, 64);
  resample(c, 1, 1, gx_, gy_, 2, B, 64, grd_[C2], 128, 0, grd_[E3], 64, 0, 0, act_[E3], 64, 0);
  conv_bwd(c, 3, 3, B, act_[R2], 64, 0, grd_[E3], 64, 0, grd_[R2], 64, 0, nullptr, 0, 0);
  resample(c, 0, 1, gx_, gy_, 2, B, 64, grd_[R2], 64, 0, grd_[C2], 128, 64, 1, act_[C2], 128, 64);
  conv_bwd(c, 2, 2, B, act_[R1], 32, 0, grd_[C2], 128, 64, grd_[R1], 32, 0, nullptr, 0, 0);
  resample(c, 0, 1, gx_, gy_, 1, B, 32, grd_[R1], 32, 0, grd_[C1], 96, 64, 1, act_[C1], 96, 64);
  conv_bwd(c, 1, 1, B, act_[R0], 16, 0, grd_[C1], 96, 64, grd_[R0], 16, 0, nullptr, 0, 0);
  resample(c, 0, 1, gx_, gy_, 0, B, 16, grd_[R0], 16, 0, grd_[C0], 48, 32, 1, act_[C0], 48, 32);
  conv_bwd(c, 0, 0, B, act_[X], 16, 0, grd_[C0], 48, 32, nullptr, 0, 0, nullptr, 0, 0);
  double l = 0.0;
  cuda_ok(cudaMemcpyAsync(&l, loss_, 8, cudaMemcpyDeviceToHost, c.stream), "loss");
  cuda_ok(cudaStreamSynchronize(c.stream), "sync");
  c.resolve();
  if (conv_path_ != 0 && tc_failed()) throw std::runtime_error("coarse net: tensor-core convolution timed out");
  return l;
}

void CoarseNet::adam(Ctx& c, double lr) {
  ++step_;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)step_), c2 = 1.f - std::pow(b2, (float)step_);
  HZ_LAUNCH(c, "net_adam", (double)wtotal_ * 22.0, k_adam, 304, 256, 0, wtotal_, w32_, g32_, m_, v_, wbf_, (float)lr,
            b1, b2, 1e-8f, c1, c2);
  refresh_images(c);
}

void CoarseNet::train(Ctx& c, const float* x, const float* t, int nx, int ny, long long nsamples, int batch,
                      int epochs, double lr, unsigned seed, double* loss_hist) {
  if (batch < 1 || nsamples < 1 || epochs < 1) throw std::runtime_error("coarse net: bad training sizes");
  if (nsamples >= (1LL << 31)) throw std::runtime_error("coarse net: too many training pairs");
  batch = (int)std::min<long long>(batch, nsamples);
  const long long N = (long long)nx * ny;
  if ((long long)batch * N * 4 > bcap_) {
    cudaDeviceSynchronize();
    dfree(bx_);
    dfree(bt_);
    dalloc(&bx_, (size_t)batch * N * 16);
    dalloc(&bt_, (size_t)batch * N * 8);
    bcap_ = (long long)batch * N * 4;
  }
  cudaDeviceSynchronize();
  dfree(perm_);
  dalloc(&perm_, (size_t)nsamples * sizeof(int));
  ensure(nx, ny, batch, true);
  std::mt19937 rng(seed);
  std::vector<int> perm((size_t)nsamples);
  const long long steps_per_epoch = nsamples / batch;
  const long long total = steps_per_epoch * epochs;
  long long it = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    std::iota(perm.begin(), perm.end(), 0);
    std::shuffle(perm.begin(), perm.end(), rng);
    cuda_ok(cudaMemcpyAsync(perm_, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream), "perm");
    double sum = 0.0;
    for (long long s = 0; s < steps_per_epoch; ++s, ++it) {
      const long long tot = (long long)batch * N;
      HZ_LAUNCH(c, "net_gather", (double)tot * 48.0, k_gather_pairs, (unsigned)((tot + 255) / 256), 256, 0, batch, N,
                perm_ + s * batch, reinterpret_cast<const float4*>(x), reinterpret_cast<const float2*>(t),
                reinterpret_cast<float4*>(bx_), reinterpret_cast<float2*>(bt_));
      forward(c, bx_, nx, ny, batch, true);
      sum += backward(c, bt_, nx, ny, batch);
      // cosine decay to lr / 20
      const double f = total > 1 ? (double)it / (double)(total - 1) : 1.0;
      adam(c, lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(M_PI * f))));
    }
    if (loss_hist) loss_hist[ep] = sum / (double)std::max<long long>(1, steps_per_epoch);
  }
  cuda_ok(cudaStreamSynchronize(c.stream), "sync");
  c.resolve();
}

// ---------------------------------------------------------------------------
// Solver-side packing
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_col_rms(long long N, const cplx<T>* __restrict__ b, long long ld,
                                                 const int* __restrict__ cols, float* __restrict__ scale) {
  const int k = blockIdx.x;
  const cplx<T>* col = b + (long long)(cols ? cols[k] : k) * ld;
  double s = 0.0;
  for (long long p = threadIdx.x; p < N; p += blockDim.x) {
    const double re = (double)col[p].x, im = (double)col[p].y;
    s += re * re + im * im;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) scale[k] = (float)sqrt(sh[0] / (double)N);
}

template <typename T>
__global__ void k_net_pack(long long N, const cplx<T>* __restrict__ b, long long ld, const int* __restrict__ cols,
                           int nc, const float2* __restrict__ feat, int conj, const float* __restrict__ scale,
                           float4* __restrict__ x4) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nc * N) return;
  const int k = (int)(i / N);
  const long long p = i % N;
  const float s = scale[k];
  const float inv = s > 0.f ? 1.f / s : 0.f;
  const cplx<T> v = b[(long long)cols[k] * ld + p];
  const float2 f = feat[p];
  x4[i] = make_float4((float)v.x * inv, (conj ? -(float)v.y : (float)v.y) * inv, f.x, f.y);
}

template <typename T>
__global__ void k_net_unpack(long long N, const float* __restrict__ y, const float* __restrict__ scale, double h2,
                             int conj, cplx<T>* __restrict__ out, long long ld, const int* __restrict__ cols, int nc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nc * N) return;
  const int k = (int)(i / N);
  const long long p = i % N;
  const double s = (double)scale[k] * h2;
  const float2 v = *reinterpret_cast<const float2*>(y + i * 8);
  out[(long long)cols[k] * ld + p] = mk<T>((T)(s * v.x), (T)(conj ? -s * v.y : s * v.y));
}

template <typename T>
void launch_net_pack(Ctx& ctx, long long N, const cplx<T>* b, long long ld, const int* cols, int nc,
                     const float2* feat, int conj, float* scale, float* x4) {
  HZ_LAUNCH(ctx, "net_col_rms", (double)nc * N * sizeof(cplx<T>), k_col_rms<T>, nc, 256, 0, N, b, ld, cols, scale);
  const long long tot = (long long)nc * N;
  HZ_LAUNCH(ctx, "net_pack", (double)tot * (sizeof(cplx<T>) + 24.0), k_net_pack<T>, (unsigned)((tot + 255) / 256),
            256, 0, N, b, ld, cols, nc, feat, conj, scale, reinterpret_cast<float4*>(x4));
}

template <typename T>
void launch_net_unpack(Ctx& ctx, long long N, const float* y, const float* scale, double h2, int conj, cplx<T>* out,
                       long long ld, const int* cols, int nc) {
  const long long tot = (long long)nc * N;
  HZ_LAUNCH(ctx, "net_unpack", (double)tot * (8.0 + sizeof(cplx<T>)), k_net_unpack<T>, (unsigned)((tot + 255) / 256),
            256, 0, N, y, scale, h2, conj, out, ld, cols, nc);
}

template void launch_net_pack<float>(Ctx&, long long, const float2*, long long, const int*, int, const float2*, int,
                                     float*, float*);
template void launch_net_pack<double>(Ctx&, long long, const double2*, long long, const int*, int, const float2*, int,
                                      float*, float*);
template void launch_net_unpack<float>(Ctx&, long long, const float*, const float*, double, int, float2*, long long,
                                       const int*, int);
template void launch_net_unpack<double>(Ctx&, long long, const float*, const float*, double, int, double2*,
                                        long long, const int*, int);

__global__ void k_pair_pack(long long N, const double2* __restrict__ r, const double2* __restrict__ e, int nc,
                            const float2* __restrict__ feat, double h2, const float* __restrict__ scale,
                            float4* __restrict__ x4, float2* __restrict__ t2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nc * N) return;
  const int k = (int)(i / N);
  const long long p = i % N;
  const double s = (double)scale[k];
  const double inv = s > 0.0 ? 1.0 / s : 0.0;
  const double2 rv = r[i], ev = e[i];
  const float2 f = feat[p];
  x4[i] = make_float4((float)(rv.x * inv), (float)(rv.y * inv), f.x, f.y);
  t2[i] = make_float2((float)(ev.x * inv / h2), (float)(ev.y * inv / h2));
}

void launch_pair_pack(Ctx& ctx, long long N, const double2* r, const double2* e, int nc, const float2* feat, double h2,
                      float* scale, float* x4, float* t2) {
  HZ_LAUNCH(ctx, "net_col_rms", (double)nc * N * 16.0, k_col_rms<double>, nc, 256, 0, N, r, N, (const int*)nullptr,
            scale);
  const long long tot = (long long)nc * N;
  HZ_LAUNCH(ctx, "net_pair_pack", (double)tot * 64.0, k_pair_pack, (unsigned)((tot + 255) / 256), 256, 0, N, r, e, nc,
            feat, h2, scale, reinterpret_cast<float4*>(x4), reinterpret_cast<float2*>(t2));
}

__global__ void k_gather_cols(long long N, const double2* __restrict__ src, long long ld, const int* __restrict__ cols,
                              int nc, double2* __restrict__ dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nc * N) return;
  dst[i] = src[(long long)cols[i / N] * ld + i % N];
}

void launch_gather_cols(Ctx& ctx, long long N, const double2* src, long long ld, const int* cols, int nc,
                        double2* dst) {
  const long long tot = (long long)nc * N;
  HZ_LAUNCH(ctx, "net_capture", (double)tot * 32.0, k_gather_cols, (unsigned)((tot + 255) / 256), 256, 0, N, src, ld,
            cols, nc, dst);
}

__global__ void k_axpy_compact(long long n, const double2* __restrict__ e, double2* __restrict__ x) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 a = x[i], b = e[i];
  x[i] = make_double2(a.x + b.x, a.y + b.y);
}

void launch_axpy_compact(Ctx& ctx, long long N, int nc, const double2* e, double2* x) {
  const long long tot = (long long)nc * N;
  HZ_LAUNCH(ctx, "net_axpy", (double)tot * 48.0, k_axpy_compact, (unsigned)((tot + 255) / 256), 256, 0, tot, e, x);
}

__global__ void __launch_bounds__(256) k_diff_norms(long long N, const double2* __restrict__ a,
                                                    const double2* __restrict__ b, double* __restrict__ out) {
  const int k = blockIdx.x;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (long long p = threadIdx.x; p < N; p += blockDim.x) {
    const double2 u = a[(long long)k * N + p], v = b[(long long)k * N + p];
    const double dx = u.x - v.x, dy = u.y - v.y;
    s0 += dx * dx + dy * dy;
    s1 += u.x * u.x + u.y * u.y;
    s2 += v.x * v.x + v.y * v.y;
  }
  __shared__ double sh[3][256];
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 3; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) out[3 * k + threadIdx.x] = sh[threadIdx.x][0];
}

void launch_diff_norms(Ctx& ctx, long long N, int nc, const double2* a, const double2* b, double* out) {
  HZ_LAUNCH(ctx, "net_norms", (double)nc * N * 32.0, k_diff_norms, nc, 256, 0, N, a, b, out);
}

}  // namespace hz
