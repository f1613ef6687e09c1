// Shared types and helpers for the PIV kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/piv_gb300.h"

#define PIV_HD __host__ __device__ __forceinline__
#define PIV_D __device__ __forceinline__

namespace piv {

template <typename T> struct Cplx;
template <> struct __align__(8) Cplx<float> { float x, y; };
template <> struct __align__(16) Cplx<double> { double x, y; };

template <typename T> PIV_D Cplx<T> cmake(T a, T b) { Cplx<T> r; r.x = a; r.y = b; return r; }
template <typename T> PIV_D Cplx<T> cadd(Cplx<T> a, Cplx<T> b) { return cmake<T>(a.x + b.x, a.y + b.y); }
template <typename T> PIV_D Cplx<T> csub(Cplx<T> a, Cplx<T> b) { return cmake<T>(a.x - b.x, a.y - b.y); }
template <typename T> PIV_D Cplx<T> cmul(Cplx<T> a, Cplx<T> b) {
  return cmake<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> PIV_D Cplx<T> cmulconj(Cplx<T> a, Cplx<T> b) {
  return cmake<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T> PIV_D Cplx<T> cconj(Cplx<T> a) { return cmake<T>(a.x, -a.y); }

// Round-to-nearest arithmetic without FMA contraction, used where the host
// oracle evaluates an expression as separate IEEE operations.
// Small unsigned integers as floats, exactly and without an integer-to-float
// conversion (a reduced-rate instruction): the integer (below 2^16) becomes
// the low mantissa bits of 2^23 (0x4B00xxxx = 2^23 + x), and 2^23 is
// subtracted.
PIV_D float u16_to_float(uint32_t x) { return __uint_as_float(0x4B000000u | x) - 8388608.0f; }
// Byte k (0..3) of w, placed by a byte permute.
PIV_D float u8_to_float(uint32_t w, int k) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u + (uint32_t)k)) - 8388608.0f;
}
// A pixel of any supported type as a float.
template <typename P>
PIV_D float pixel_to_float(P v) {
  return (float)v;
}
template <>
PIV_D float pixel_to_float<uint8_t>(uint8_t v) {
  return u16_to_float(v);
}
template <>
PIV_D float pixel_to_float<uint16_t>(uint16_t v) {
  return u16_to_float(v);
}

PIV_D float add_rn(float a, float b) { return __fadd_rn(a, b); }
PIV_D float sub_rn(float a, float b) { return __fsub_rn(a, b); }
PIV_D float mul_rn(float a, float b) { return __fmul_rn(a, b); }
PIV_D float div_rn(float a, float b) { return __fdiv_rn(a, b); }
PIV_D double add_rn(double a, double b) { return __dadd_rn(a, b); }
PIV_D double sub_rn(double a, double b) { return __dsub_rn(a, b); }
PIV_D double mul_rn(double a, double b) { return __dmul_rn(a, b); }
PIV_D double div_rn(double a, double b) { return __ddiv_rn(a, b); }

PIV_D bool is_nan(float v) { return isnan(v); }
PIV_D bool is_nan(double v) { return isnan(v); }

// Loads pixel `idx` of a frame of the given pixel type as T.
template <typename T> PIV_D T load_pixel(const void* base, int pixel_type, long long idx) {
  switch (pixel_type) {
    case PIV_PIXEL_U8: return (T)__ldg(((const uint8_t*)base) + idx);
    case PIV_PIXEL_U16: return (T)__ldg(((const uint16_t*)base) + idx);
    case PIV_PIXEL_F32: return (T)__ldg(((const float*)base) + idx);
    default: return (T)__ldg(((const double*)base) + idx);
  }
}

PIV_HD int div_up(int a, int b) { return (a + b - 1) / b; }

// Index checks of the checked build (compiled with -DPIV_BOUNDS_CHECK, see
// piv_bounds_check): a failed check counts a violation in this translation
// unit's device counter and the guarded access is skipped. In the normal
// build every check is the constant true and compiles away.
#ifdef PIV_BOUNDS_CHECK
static __device__ int g_bounds_violations;
PIV_D bool in_bounds(bool ok) {
  if (!ok) atomicAdd(&g_bounds_violations, 1);
  return ok;
}
// Whether [p, p + bytes) lies in the CTA's dynamic shared memory.
PIV_D bool in_dyn_smem(const void* p, unsigned bytes) {
  extern __shared__ __align__(16) unsigned char piv_dyn_smem[];
  unsigned size;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(size));
  const unsigned a = (unsigned)__cvta_generic_to_shared(p), b = (unsigned)__cvta_generic_to_shared(piv_dyn_smem);
  return in_bounds(a >= b && a + bytes <= b + size);
}
#else
PIV_D constexpr bool in_bounds(bool) { return true; }
PIV_D constexpr bool in_dyn_smem(const void*, unsigned) { return true; }
#endif
// Host side: the device counter of the checked build's translation unit
// (read and reset); -1 in the normal build.
#define PIV_DEFINE_BOUNDS_COUNTER(fn)                                                     \
  int fn() {                                                                              \
    PIV_BOUNDS_COUNTER_BODY                                                               \
  }
#ifdef PIV_BOUNDS_CHECK
#define PIV_BOUNDS_COUNTER_BODY                                                           \
  int v = 0, z = 0;                                                                       \
  if (cudaMemcpyFromSymbol(&v, g_bounds_violations, sizeof(int)) != cudaSuccess) return -2; \
  if (cudaMemcpyToSymbol(g_bounds_violations, &z, sizeof(int)) != cudaSuccess) return -2;   \
  return v;
#else
#define PIV_BOUNDS_COUNTER_BODY return -1;
#endif

// Number of SMs of the current device (cached per process).
int sm_count();

}  // namespace piv
