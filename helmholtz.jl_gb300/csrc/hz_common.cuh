// Shared device/host definitions for the helmgpu CUDA library.
//
// Complex numbers are stored interleaved (re, im) as double2 / float2 so a
// complex FP64 value is one 128-bit load and two complex FP32 values are one
// 128-bit load.  Node arrays are column-major with axis 1 fastest; a block of
// right-hand sides is stored column by column with leading dimension ld >= N.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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

// FP32 -> FP64 widening from the IEEE-754 bit layouts, exact: for a normal
// number the 8-bit exponent is re-biased (127 -> 1023) and the 23-bit fraction
// moves to the top of the 52-bit fraction, with integer operations only.
// Returns false for zero, subnormal, infinite and NaN inputs (the caller uses
// the hardware conversion for those).  GB300's FP64 pipe also executes the
// hardware conversion, so FP64 kernels that widen FP32 data (H z with z from
// the complex-FP32 cycle, x += Z y) use this to keep the conversions off it.
__host__ __device__ __forceinline__ bool widen_f32_bits(uint32_t u, uint32_t& hi, uint32_t& lo) {
  const uint32_t a = u & 0x7fffffffu;
  if (a - 0x00800000u >= 0x7f000000u) return false;
  hi = ((a >> 3) + 0x38000000u) | (u & 0x80000000u);
  lo = u << 29;
  return true;
}

#ifdef __CUDACC__
__device__ __forceinline__ double widen_f32(float f) {
  uint32_t hi, lo;
  if (!widen_f32_bits(__float_as_uint(f), hi, lo)) return (double)f;
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
