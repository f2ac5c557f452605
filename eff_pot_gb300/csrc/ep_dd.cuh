// ep_dd.cuh - double-float arithmetic: a real number as the unevaluated sum
// hi + lo of two FP32 values (|lo| <= ulp(hi)/2), about 48 significant bits.
//
// The FP64 pipe of this part runs at 1/64 of the FP32 rate; a double-float
// operation costs 4-11 FP32 instructions, so the FP64-class engine computed in
// double-float (Engine<dfloat>) runs on the FP32 pipes.  The operations follow
// the published error-free transformations: Knuth's TwoSum for the sum of two
// FP32 values, the FMA product error (a*b - fl(a*b) = fma(a, b, -fl(a*b))),
// Dekker's Fast2Sum for the renormalisation, and the double-float sum of
// one TwoSum of the high parts, whose error is within about 2^-44 (|a| + |b|);
// the product's about 2^-45 |a b|.  The FP32 range applies (normal values down to 1.2e-38; below about
// 1e-31 the low part is subnormal or zero and the relative precision falls
// towards FP32's).  Every step that must be rounded on its own is written
// with the _rn intrinsics, which the compiler never contracts into an FMA.
#pragma once
#include <cuda_runtime.h>

#ifndef EP_HD
#define EP_HD __host__ __device__ __forceinline__
#endif

struct __align__(8) dfloat {
  float hi, lo;
  dfloat() = default;
  EP_HD constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  EP_HD constexpr dfloat(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  EP_HD constexpr dfloat(float f) : hi(f), lo(0.0f) {}
  EP_HD constexpr dfloat(int i) : dfloat((double)i) {}
  EP_HD explicit constexpr operator double() const { return (double)hi + (double)lo; }
  EP_HD explicit constexpr operator float() const { return hi + lo; }
};

struct __align__(16) dfloat2 {
  dfloat x, y;
};

#if defined(__CUDA_ARCH__)
#define EP_DD_ADD(a, b) __fadd_rn(a, b)
#define EP_DD_SUB(a, b) __fsub_rn(a, b)
#define EP_DD_MUL(a, b) __fmul_rn(a, b)
#define EP_DD_FMA(a, b, c) __fmaf_rn(a, b, c)
#else
#define EP_DD_ADD(a, b) ((a) + (b))
#define EP_DD_SUB(a, b) ((a) - (b))
#define EP_DD_MUL(a, b) ((a) * (b))
#define EP_DD_FMA(a, b, c) fmaf(a, b, c)
#endif

// Fast2Sum (|a| >= |b|): s + e == a + b exactly.
EP_HD dfloat dd_fast2sum(float a, float b) {
  const float s = EP_DD_ADD(a, b);
  return dfloat(s, EP_DD_SUB(b, EP_DD_SUB(s, a)));
}

EP_HD dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }

// TwoSum: s + e == a + b exactly.
EP_HD dfloat dd_two_sum(float a, float b) {
  const float s = EP_DD_ADD(a, b);
  const float bb = EP_DD_SUB(s, a);
  return dfloat(s, EP_DD_ADD(EP_DD_SUB(a, EP_DD_SUB(s, bb)), EP_DD_SUB(b, bb)));
}

// The double-float sum: one TwoSum of the high parts, the low parts added,
// one Fast2Sum (error within about 2^-44 of |a| + |b|).  The form with a
// second TwoSum for the low parts (error within 2^-48 of the result) gave the
// same parity figures and a 40 % slower step.
EP_HD dfloat operator+(dfloat a, dfloat b) {
  const dfloat s = dd_two_sum(a.hi, b.hi);
  return dd_fast2sum(s.hi, EP_DD_ADD(s.lo, EP_DD_ADD(a.lo, b.lo)));
}
EP_HD dfloat operator-(dfloat a, dfloat b) { return a + (-b); }

EP_HD dfloat operator*(dfloat a, dfloat b) {
  const float p = EP_DD_MUL(a.hi, b.hi);
  float e = EP_DD_FMA(a.hi, b.hi, -p);
  e = EP_DD_FMA(a.hi, b.lo, e);
  e = EP_DD_FMA(a.lo, b.hi, e);
  return dd_fast2sum(p, e);
}

// a / b: one FP32 quotient, its remainder in double-float, one correction.
EP_HD dfloat operator/(dfloat a, dfloat b) {
  const float q1 = a.hi / b.hi;
  const dfloat r = a - b * dfloat(q1);
  const float q2 = r.hi / b.hi;
  return dd_fast2sum(q1, q2);
}

EP_HD dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
EP_HD dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
EP_HD dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }

EP_HD bool operator<(dfloat a, dfloat b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
EP_HD bool operator>(dfloat a, dfloat b) { return b < a; }
EP_HD bool operator<=(dfloat a, dfloat b) { return !(b < a); }
EP_HD bool operator>=(dfloat a, dfloat b) { return !(a < b); }
EP_HD bool operator==(dfloat a, dfloat b) { return a.hi == b.hi && a.lo == b.lo; }
EP_HD bool operator!=(dfloat a, dfloat b) { return !(a == b); }

EP_HD dfloat fabs(dfloat a) { return a.hi < 0.0f ? -a : a; }
EP_HD dfloat fma(dfloat a, dfloat b, dfloat c) { return a * b + c; }
EP_HD dfloat fmin(dfloat a, dfloat b) { return b < a ? b : a; }
EP_HD dfloat fmax(dfloat a, dfloat b) { return a < b ? b : a; }
EP_HD bool isfinite(dfloat a) { return isfinite(a.hi); }
// sqrt: the FP32 root and one Newton correction in double-float.
EP_HD dfloat sqrt(dfloat a) {
  if (!(a.hi > 0.0f)) return dfloat(sqrtf(a.hi), 0.0f);
  const float r = sqrtf(a.hi);
  const dfloat d = a - dfloat(r) * dfloat(r);
  return dd_fast2sum(r, d.hi / (2.0f * r));
}

#if defined(__CUDACC__)
__device__ __forceinline__ dfloat __shfl_sync(unsigned m, dfloat v, int src) {
  return dfloat(__shfl_sync(m, v.hi, src), __shfl_sync(m, v.lo, src));
}
__device__ __forceinline__ dfloat __shfl_down_sync(unsigned m, dfloat v, unsigned d) {
  return dfloat(__shfl_down_sync(m, v.hi, d), __shfl_down_sync(m, v.lo, d));
}
__device__ __forceinline__ dfloat __shfl_xor_sync(unsigned m, dfloat v, int d) {
  return dfloat(__shfl_xor_sync(m, v.hi, d), __shfl_xor_sync(m, v.lo, d));
}
__device__ __forceinline__ dfloat __ldg(const dfloat* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return dfloat(v.x, v.y);
}
__device__ __forceinline__ dfloat __ldcg(const dfloat* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return dfloat(v.x, v.y);
}
#endif

// Complex double-float.  On the device the real and imaginary parts go
// through the same error-free steps side by side as FP32 pairs (FADD2 /
// FMUL2 / FFMA2: one instruction for both parts; x * -1 + y is the exact
// y - x).  The host forms are the scalar operators.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ float2 dd_neg2(float2 a) { return make_float2(-a.x, -a.y); }
// (h, l) pairs of the two parts: hi parts in h, lo parts in l.
__device__ __forceinline__ dfloat2 dd_pack(float2 h, float2 l) {
  return dfloat2{dfloat(h.x, l.x), dfloat(h.y, l.y)};
}
__device__ __forceinline__ dfloat2 dd_add2(float2 ah, float2 al, float2 bh, float2 bl) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  const float2 s = __fadd2_rn(ah, bh);
  const float2 bb = __ffma2_rn(ah, m1, s);                    // s - a
  const float2 e1 = __ffma2_rn(__ffma2_rn(bb, m1, s), m1, ah);  // a - (s - bb)
  const float2 e2 = __ffma2_rn(bb, m1, bh);                   // b - bb
  const float2 e = __fadd2_rn(__fadd2_rn(e1, e2), __fadd2_rn(al, bl));
  const float2 h = __fadd2_rn(s, e);
  return dd_pack(h, __ffma2_rn(__ffma2_rn(s, m1, h), m1, e));   // e - (h - s)
}
__device__ __forceinline__ dfloat2 operator+(dfloat2 a, dfloat2 b) {
  return dd_add2(make_float2(a.x.hi, a.y.hi), make_float2(a.x.lo, a.y.lo), make_float2(b.x.hi, b.y.hi),
                 make_float2(b.x.lo, b.y.lo));
}
__device__ __forceinline__ dfloat2 operator-(dfloat2 a, dfloat2 b) {
  return dd_add2(make_float2(a.x.hi, a.y.hi), make_float2(a.x.lo, a.y.lo), make_float2(-b.x.hi, -b.y.hi),
                 make_float2(-b.x.lo, -b.y.lo));
}
// s * (ah + al) for a double-float s: the FMA product error of both parts.
__device__ __forceinline__ void dd_scale2(dfloat s, float2 ah, float2 al, float2& ph, float2& pe) {
  const float2 sh = make_float2(s.hi, s.hi), sl = make_float2(s.lo, s.lo);
  ph = __fmul2_rn(sh, ah);
  float2 e = __ffma2_rn(sh, ah, dd_neg2(ph));
  e = __ffma2_rn(sh, al, e);
  pe = __ffma2_rn(sl, ah, e);
}
__device__ __forceinline__ dfloat2 operator*(dfloat s, dfloat2 a) {
  float2 p, e;
  dd_scale2(s, make_float2(a.x.hi, a.y.hi), make_float2(a.x.lo, a.y.lo), p, e);
  const float2 h = __fadd2_rn(p, e);
  return dd_pack(h, __ffma2_rn(__ffma2_rn(p, make_float2(-1.0f, -1.0f), h), make_float2(-1.0f, -1.0f), e));
}
// Complex products: the two real-by-complex products side by side, then one
// complex sum (a * b and a * conj(b)).
__device__ __forceinline__ dfloat2 cmul(dfloat2 a, dfloat2 b) {
  float2 tp, te, up, ue;
  dd_scale2(a.x, make_float2(b.x.hi, b.y.hi), make_float2(b.x.lo, b.y.lo), tp, te);
  dd_scale2(a.y, make_float2(-b.y.hi, b.x.hi), make_float2(-b.y.lo, b.x.lo), up, ue);
  return dd_add2(tp, te, up, ue);
}
__device__ __forceinline__ dfloat2 cmulc(dfloat2 a, dfloat2 b) {
  float2 tp, te, up, ue;
  dd_scale2(a.x, make_float2(b.x.hi, -b.y.hi), make_float2(b.x.lo, -b.y.lo), tp, te);
  dd_scale2(a.y, make_float2(b.y.hi, b.x.hi), make_float2(b.y.lo, b.x.lo), up, ue);
  return dd_add2(tp, te, up, ue);
}
// Stencil sums w_k (x_k + y_k) of complex double-float values as unnormalised
// accumulators (Ogita, Rump and Oishi's Sum2 with the FMA product error): the
// running sum is h + l with the error terms gathered in l by plain FP32 pair
// additions and one Fast2Sum at the end, about 20 paired operations a term
// against 27 for a normalised double-float product and sum.
struct dd2_acc {
  float2 h, l;
};
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  s = __fadd2_rn(a, b);
  const float2 bb = __ffma2_rn(a, m1, s);                                            // s - a
  e = __fadd2_rn(__ffma2_rn(__ffma2_rn(bb, m1, s), m1, a), __ffma2_rn(bb, m1, b));  // (a - (s - bb)) + (b - bb)
}
// w (x + y), unnormalised: the pair sum by TwoSum of the high parts, the
// product's error by FMA
__device__ __forceinline__ void dd2_wsum(dfloat w, dfloat2 x, dfloat2 y, float2& ph, float2& pl) {
  float2 sh, se;
  two_sum2(make_float2(x.x.hi, x.y.hi), make_float2(y.x.hi, y.y.hi), sh, se);
  const float2 sl = __fadd2_rn(se, __fadd2_rn(make_float2(x.x.lo, x.y.lo), make_float2(y.x.lo, y.y.lo)));
  const float2 wh = make_float2(w.hi, w.hi), wl = make_float2(w.lo, w.lo);
  ph = __fmul2_rn(wh, sh);
  pl = __ffma2_rn(wh, sl, __ffma2_rn(wl, sh, __ffma2_rn(wh, sh, dd_neg2(ph))));
}
// w (x - y), unnormalised
__device__ __forceinline__ void dd2_wdiff(dfloat w, dfloat2 x, dfloat2 y, float2& ph, float2& pl) {
  dd2_wsum(w, x, dfloat2{dfloat(-y.x.hi, -y.x.lo), dfloat(-y.y.hi, -y.y.lo)}, ph, pl);
}
// w c, unnormalised
__device__ __forceinline__ dd2_acc dd2_start(dfloat w, dfloat2 c) {
  const float2 wh = make_float2(w.hi, w.hi), wl = make_float2(w.lo, w.lo), ch = make_float2(c.x.hi, c.y.hi);
  dd2_acc a;
  a.h = __fmul2_rn(wh, ch);
  a.l = __ffma2_rn(wh, make_float2(c.x.lo, c.y.lo), __ffma2_rn(wl, ch, __ffma2_rn(wh, ch, dd_neg2(a.h))));
  return a;
}
__device__ __forceinline__ void dd2_add(dd2_acc& a, float2 ph, float2 pl) {
  float2 s, e;
  two_sum2(a.h, ph, s, e);
  a.h = s;
  a.l = __fadd2_rn(a.l, __fadd2_rn(e, pl));
}
__device__ __forceinline__ dfloat2 dd2_value(const dd2_acc& a) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  const float2 h = __fadd2_rn(a.h, a.l);
  return dd_pack(h, __ffma2_rn(__ffma2_rn(a.h, m1, h), m1, a.l));  // l - (h - a.h)
}
#else
inline dfloat2 operator+(dfloat2 a, dfloat2 b) { return dfloat2{a.x + b.x, a.y + b.y}; }
inline dfloat2 operator-(dfloat2 a, dfloat2 b) { return dfloat2{a.x - b.x, a.y - b.y}; }
inline dfloat2 operator*(dfloat s, dfloat2 a) { return dfloat2{s * a.x, s * a.y}; }
#endif
