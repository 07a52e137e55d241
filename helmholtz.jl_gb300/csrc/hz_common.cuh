// Shared device/host definitions for the helmgpu CUDA library.
//
// Complex numbers are stored interleaved (re, im) as double2 / float2 so a
// complex FP64 value is one 128-bit load and two complex FP32 values are one
// 128-bit load.  Node arrays are column-major with axis 1 fastest; a block of
// right-hand sides is stored column by column with leading dimension ld >= N.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace hz {

template <typename T> struct cvec;
template <> struct cvec<double> { using type = double2; };
template <> struct cvec<float> { using type = float2; };
// Emulated-FP64 complex (float4: re_hi, im_hi, re_lo, im_lo); as a right-hand
// side of a complex-FP32 kernel only .x/.y (the high parts) are read.
struct df64_tag {};
template <> struct cvec<df64_tag> { using type = float4; };
template <typename T> using cplx = typename cvec<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T re, T im) {
  cplx<T> z;
  z.x = re;
  z.y = im;
  return z;
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x + b.x, a.y + b.y);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x - b.x, a.y - b.y);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// acc + a*b
template <typename T> __host__ __device__ __forceinline__ cplx<T> cfma(cplx<T> a, cplx<T> b, cplx<T> acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// acc + conj(a)*b
template <typename T> __host__ __device__ __forceinline__ cplx<T> cfma_conj(cplx<T> a, cplx<T> b, cplx<T> acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
// acc - a*b
template <typename T> __host__ __device__ __forceinline__ cplx<T> cfms(cplx<T> a, cplx<T> b, cplx<T> acc) {
  acc.x = fma(-a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cscale(T s, cplx<T> a) {
  return mk<T>(s * a.x, s * a.y);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cconj(cplx<T> a) { return mk<T>(a.x, -a.y); }

// FP32 -> FP64 widening from the IEEE-754 bit layouts, exact for every input,
// with no FP64 operation.  GB300's FP64 pipe also executes the hardware
// conversion, and the FP64 kernels that read FP32 data (H z with z from the
// complex-FP32 cycle, x += Z y) are bound by that pipe, so no conversion of
// theirs may land there, not even a predicated one for the rare inputs.  The
// high and low words of the FP64 result:
//  - normal: the 8-bit exponent is re-biased (127 -> 1023), the 23-bit fraction
//    moves to the top of the 52-bit fraction;
//  - subnormal: scaled by 2^24 in FP32 (exact, the product is normal), widened
//    as a normal number, then 24 taken off the exponent;
//  - a zero keeps its sign, an infinity stays infinite, a NaN keeps its payload
//    (moved up with the fraction) and becomes quiet.
__host__ __device__ __forceinline__ void widen_f32_hilo(uint32_t u, uint32_t& hi, uint32_t& lo) {
  const uint32_t sg = u & 0x80000000u;
  uint32_t a = u & 0x7fffffffu;
  uint32_t bias = 0x38000000u;  // (1023 - 127) << 20
  if (a - 0x00800000u >= 0x7f000000u) {  // exponent field 0 or 255
    if (a >= 0x7f800000u) {
      hi = sg | 0x7ff00000u | ((a & 0x007fffffu) >> 3) | (a > 0x7f800000u ? 0x00080000u : 0u);
      lo = a << 29;
      return;
    }
    if (a == 0u) {
      hi = sg;
      lo = 0u;
      return;
    }
    float f, g;
#ifdef __CUDA_ARCH__
    f = __uint_as_float(a);
    g = f * 16777216.0f;
    a = __float_as_uint(g);
#else
    memcpy(&f, &a, 4);
    g = f * 16777216.0f;
    memcpy(&a, &g, 4);
#endif
    bias -= 24u << 20;
  }
  hi = sg | ((a >> 3) + bias);
  lo = a << 29;
}

__host__ __device__ __forceinline__ uint64_t widen_f32_bits(uint32_t u) {
  uint32_t hi, lo;
  widen_f32_hilo(u, hi, lo);
  return ((uint64_t)hi << 32) | lo;
}

#ifdef __CUDACC__
__device__ __forceinline__ double widen_f32(float f) {
  uint32_t hi, lo;
  widen_f32_hilo(__float_as_uint(f), hi, lo);
  return __hiloint2double((int)hi, (int)lo);
}
#endif

template <typename To, typename From> __host__ __device__ __forceinline__ cplx<To> ccast(cplx<From> a) {
  return mk<To>((To)a.x, (To)a.y);
}
template <> __host__ __device__ __forceinline__ cplx<double> ccast<double, float>(cplx<float> a) {
#ifdef __CUDA_ARCH__
  return mk<double>(widen_f32(a.x), widen_f32(a.y));
#else
  return mk<double>((double)a.x, (double)a.y);
#endif
}

// Node grid of one multigrid level.  2D grids have nz == 1.
struct Grid {
  int nx, ny, nz;
  long long N;
};

}  // namespace hz
