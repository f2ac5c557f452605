// ep_common.cuh - shared types and helpers of the eff_pot CUDA library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define EP_DEV __device__ __forceinline__
#define EP_HD __host__ __device__ __forceinline__

#include "ep_dd.cuh"

// ---------------------------------------------------------------------------
// Complex numbers as CUDA vector types (x = re, y = im).
template <class T> struct cpx_traits;
template <> struct cpx_traits<double> { typedef double2 type; };
template <> struct cpx_traits<float> { typedef float2 type; };
template <> struct cpx_traits<dfloat> { typedef dfloat2 type; };
template <class T> using C2 = typename cpx_traits<T>::type;

EP_HD double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
EP_HD double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
EP_HD double2 operator*(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
// FP32 complex sums and scalings are paired instructions on the device (the
// same rounding as the two scalar ones: a - b is b * -1 + a, exact).
EP_HD float2 operator+(float2 a, float2 b) {
#if defined(__CUDA_ARCH__)
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
EP_HD float2 operator-(float2 a, float2 b) {
#if defined(__CUDA_ARCH__)
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
EP_HD float2 operator*(float s, float2 a) {
#if defined(__CUDA_ARCH__)
  return __fmul2_rn(make_float2(s, s), a);
#else
  return make_float2(s * a.x, s * a.y);
#endif
}

template <class T> EP_HD C2<T> cmk(T a, T b) { C2<T> r; r.x = a; r.y = b; return r; }

// A value of any field precision as an FP64 number.
EP_HD double dbl(double v) { return v; }
EP_HD double dbl(float v) { return v; }
EP_HD double dbl(dfloat v) { return (double)v; }

// Complex (re, im) arithmetic as one vector operation: on sm_100+ an FP32
// pair is one paired instruction (FADD2 / FMUL2 / FFMA2), half the issue
// slots of two scalar ones; FP64 pairs are two scalar operations with the
// same rounding as the contracted scalar expressions (s*a + c -> fma).
EP_DEV float2 vadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
EP_DEV float2 vsub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
EP_DEV float2 vmul(float s, float2 a) { return __fmul2_rn(make_float2(s, s), a); }
EP_DEV float2 vfma(float s, float2 a, float2 c) { return __ffma2_rn(make_float2(s, s), a, c); }
EP_DEV double2 vadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
EP_DEV double2 vsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
EP_DEV double2 vmul(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
EP_DEV double2 vfma(double s, double2 a, double2 c) { return make_double2(fma(s, a.x, c.x), fma(s, a.y, c.y)); }
EP_DEV dfloat2 vadd(dfloat2 a, dfloat2 b) { return a + b; }
EP_DEV dfloat2 vsub(dfloat2 a, dfloat2 b) { return a - b; }
EP_DEV dfloat2 vmul(dfloat s, dfloat2 a) { return s * a; }
EP_DEV dfloat2 vfma(dfloat s, dfloat2 a, dfloat2 c) { return s * a + c; }
template <class T2> EP_HD T2 cmul(T2 a, T2 b) {
  T2 r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template <class T2> EP_HD T2 cmulc(T2 a, T2 b) {
  T2 r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
template <class T2> EP_HD T2 conjg(T2 a) { T2 r; r.x = a.x; r.y = -a.y; return r; }
// i*a
template <class T2> EP_HD T2 mul_i(T2 a) { T2 r; r.x = -a.y; r.y = a.x; return r; }
// -i*a
template <class T2> EP_HD T2 mul_mi(T2 a) { T2 r; r.x = a.y; r.y = -a.x; return r; }

// ---------------------------------------------------------------------------
// Device-side scalar block shared by all kernels of a context.  Reductions
// are accumulated in FP64 whatever the field precision.
struct DevScalars {
  double sums[40];      // finalize outputs (named by the producing kernel)
  double scale;         // pending imaginary-time renormalisation factor
  double errHe, norm, mu;
  unsigned int flags;   // bit 0: non-finite detected; bit 1: den <= 0
  unsigned int counter; // blocks done (last-block finalisation), reset to 0
  unsigned int counter2;
  // Lazy renormalisation: the logical value of rotating state buffer k is
  // stored * bscale[k]; den's logical value is stored * den_scale.
  double bscale[8];
  double den_scale;
  // bscale rounded to FP32 once, by the thread that writes bscale: FP32
  // kernels read these instead of converting bscale in every thread (a
  // double -> float conversion runs on the FP64 pipe)
  float bscale_f[8];
};
#define EP_NSLOTS 8
// EP_FLAG_TIMEOUT: a bounded wait on a TMA copy ran out (the block stopped
// its march and the host reports EP_ERR_TIMEOUT).
enum { EP_FLAG_NONFINITE = 1u, EP_FLAG_DEN_NONPOS = 2u, EP_FLAG_TIMEOUT = 4u };

// ---------------------------------------------------------------------------
// 1-D FFT plan: length and radix sequence (radices 8,4,2,3,5).
struct FftPlan {
  int n;
  int nst;
  int rad[12];
};

// Radix sequence for n = 2^a 3^b 5^c: as many 8s as possible, a 4 or 2 for
// the rest of the power of two (two 4s instead of 8*2), then 3s and 5s.
inline bool make_plan(int n, FftPlan& p) {
  p.n = n;
  p.nst = 0;
  int m = n, e = 0;
  while (m % 2 == 0) { m /= 2; ++e; }
  int n8 = e / 3, rem = e % 3;
  if (rem == 1 && n8 > 0) { --n8; rem = 4; }
  for (int i = 0; i < n8; ++i) p.rad[p.nst++] = 8;
  if (rem == 4) { p.rad[p.nst++] = 4; p.rad[p.nst++] = 4; }
  else if (rem == 2) p.rad[p.nst++] = 4;
  else if (rem == 1) p.rad[p.nst++] = 2;
  while (m % 3 == 0) { m /= 3; p.rad[p.nst++] = 3; }
  while (m % 5 == 0) { m /= 5; p.rad[p.nst++] = 5; }
  return m == 1 && p.nst <= 12;
}

// Geometry of a grid (passed by value to kernels).
struct Geo {
  int nx, ny, nz, nxh;
  long long N, Nh;
};

#define EP_MAX_NPD 25
#define EP_MAX_R 12

// ---------------------------------------------------------------------------
// Asynchronous global->shared copies (cp.async, sm_80+): the copy engine
// fills shared memory while the threads compute.
template <int BYTES>
EP_DEV void cp_async(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if (BYTES == 4) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
  else if (BYTES == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
EP_DEV void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
EP_DEV void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
