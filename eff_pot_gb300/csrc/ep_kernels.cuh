// ep_kernels.cuh - device kernels of the eff_pot hot path, templated on the
// field precision T (double or float).  Reductions always accumulate in FP64.
#pragma once
#include <type_traits>
#include "ep_common.cuh"
#include "ep_fft.cuh"
#include "ep_reduce.cuh"
#include "ep_pairpot.h"
#include "ep_tma.cuh"

// ---------------------------------------------------------------------------
// Kernel parameter blocks.
template <class T> struct FdW {
  T w1[3][EP_MAX_R + 1];  // first derivative, weight at +k (at -k: -w1)
  T w2[3][EP_MAX_R + 1];  // second derivative, weight at +-k; [0] = centre
  int R;
  int periodic;           // icon 8 (1) or icon 13 (0)
};

// The functional's constants in FP32, rounded once on the host.
struct PhysF {
  float cp4, cpp4, a0, a1, rden0s, h2o2m4, alphas, C, beta, den_m, renor;
};
// The same constants split into double-float pairs on the host, for the
// double-float kernels.
struct PhysD {
  dfloat cp4, cpp4, a0, a1, rden0s, h2o2m4, alphas, C, beta, den_m, renor;
};
struct Phys {
  double cp4, cpp4, a0, a1, den0s, h2o2m4, alphas, C, beta, den_m;
  double renor, dxyz;
  double rden0s;          // 1 / den0s
  int core;               // EP_CORE_*
  int time_mode;          // 0 imaginary, 1 real
  PhysF f;                // the same constants for the FP32 kernels
  PhysD d;                // and for the double-float kernels
};

// Phys in the field precision T.  FP32 kernels take the host-rounded copies:
// a double -> float conversion or a double division in every thread would
// run on the FP64 pipe (1/64 of the FP32 rate on this part) before any
// point is processed.
template <class T> struct PConst;
template <> struct PConst<double> {
  double cp4, cpp4, a0, a1, rden0s, h2o2m4, alphas, C, beta, den_m, renor;
  EP_DEV explicit PConst(const Phys& p)
      : cp4(p.cp4), cpp4(p.cpp4), a0(p.a0), a1(p.a1), rden0s(p.rden0s), h2o2m4(p.h2o2m4), alphas(p.alphas),
        C(p.C), beta(p.beta), den_m(p.den_m), renor(p.renor) {}
};
template <> struct PConst<dfloat> {
  dfloat cp4, cpp4, a0, a1, rden0s, h2o2m4, alphas, C, beta, den_m, renor;
  EP_DEV explicit PConst(const Phys& p)
      : cp4(p.d.cp4), cpp4(p.d.cpp4), a0(p.d.a0), a1(p.d.a1), rden0s(p.d.rden0s), h2o2m4(p.d.h2o2m4),
        alphas(p.d.alphas), C(p.d.C), beta(p.d.beta), den_m(p.d.den_m), renor(p.d.renor) {}
};
template <> struct PConst<float> {
  float cp4, cpp4, a0, a1, rden0s, h2o2m4, alphas, C, beta, den_m, renor;
  EP_DEV explicit PConst(const Phys& p)
      : cp4(p.f.cp4), cpp4(p.f.cpp4), a0(p.f.a0), a1(p.f.a1), rden0s(p.f.rden0s), h2o2m4(p.f.h2o2m4),
        alphas(p.f.alphas), C(p.f.C), beta(p.f.beta), den_m(p.f.den_m), renor(p.f.renor) {}
};

// Buffer scale k of the lazy renormalisation in the field precision.
template <class T> EP_DEV T bscale_of(const DevScalars* sc, int k);
template <> EP_DEV double bscale_of<double>(const DevScalars* sc, int k) { return sc->bscale[k]; }
template <> EP_DEV float bscale_of<float>(const DevScalars* sc, int k) { return sc->bscale_f[k]; }
template <> EP_DEV dfloat bscale_of<dfloat>(const DevScalars* sc, int k) { return dfloat(sc->bscale[k]); }

// Lines of a strided pass: element k of line L lives at
//   (L % Mi) + (L / Mi) * So + k * Sa.
struct LineSet {
  long long Mi, So, Sa, nlines;
};

template <class T> struct Arr8 { C2<T>* a[8]; };

template <class T> struct ConvSpec {
  const C2<T>* in[4];
  C2<T>* out[4][3];
  const T* ker[4][3];
  int nout[4];
};

// ---------------------------------------------------------------------------
// Small helpers.
EP_DEV int wrapi(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// f at offset k along an axis of length n (index i, element stride st), with
// the boundary mode of the finite differences.
template <class T>
EP_DEV T nbr(const T* __restrict__ f, long long p, int i, int k, int n, long long st, int periodic) {
  int ii = i + k;
  if (ii < 0 || ii >= n) {
    if (!periodic) return T(0);
    ii = wrapi(ii, n);
  }
  return f[p + (long long)(ii - i) * st];
}

// First derivative along an axis from global memory (pairs +k/-k); points
// at least R away from both ends skip the boundary logic.
template <class T>
EP_DEV T d1_global(const T* __restrict__ f, long long p, int i, int n, long long st, const T* w, int R, int periodic) {
  T s = T(0);
  if (i >= R && i < n - R) {
    const T* c = f + p;
    for (int k = 1; k <= R; ++k) s += w[k] * (__ldg(c + k * st) - __ldg(c - k * st));
    return s;
  }
  for (int k = 1; k <= R; ++k) s += w[k] * (nbr(f, p, i, k, n, st, periodic) - nbr(f, p, i, -k, n, st, periodic));
  return s;
}

// First derivative along a line held in shared memory (length n).
template <class T>
EP_DEV T d1_line(const T* __restrict__ line, int i, int n, const T* w, int R, int periodic) {
  T s = T(0);
  for (int k = 1; k <= R; ++k) {
    int ip = i + k, im = i - k;
    T fp, fm;
    if (ip >= n) fp = periodic ? line[ip - n] : T(0); else fp = line[ip];
    if (im < 0) fm = periodic ? line[im + n] : T(0); else fm = line[im];
    s += w[k] * (fp - fm);
  }
  return s;
}

// Solid penalty C*(1 + t + beta*den*(1 - t^2)), t = tanh(beta*(den - den_m))
// (poten.f90:80-81).  The FP32 form is written without the cancellation of
// 1 + tanh(x) for x << 0: 1 + t = 2/(1 + e^{-2x}), 1 - t^2 = 4e^{2x}/(1+e^{2x})^2.
// Penalty constants in the field precision, converted once per thread (a
// double -> float conversion per point would run on the FP64 pipe).
template <class T> struct Pen {
  T C, beta, den_m;
  EP_DEV explicit Pen(const Phys& ph) {
    const PConst<T> k(ph);
    C = k.C;
    beta = k.beta;
    den_m = k.den_m;
  }
};
EP_DEV double penalty_of(const Pen<double>& pn, double den) {
  const double t = tanh(pn.beta * (den - pn.den_m));
  return pn.C * (1.0 + t + pn.beta * den * (1.0 - t * t));
}
EP_DEV float penalty_of(const Pen<float>& pn, float den) {
  const float x = pn.beta * (den - pn.den_m);
  const float e = __expf(2.0f * x);
  const float onept = 2.0f * e / (1.0f + e);
  const float omt2 = 4.0f * e / ((1.0f + e) * (1.0f + e));
  return pn.C * (onept + pn.beta * den * omt2);
}
// Double-float fields: the penalty in FP32 (at the densities of a liquid it
// is below 1e-7 K, and a density near den_m is far outside the method).
template <> struct Pen<dfloat> {
  Pen<float> f;
  EP_DEV explicit Pen(const Phys& ph) : f(ph) {}
};
EP_DEV dfloat penalty_of(const Pen<dfloat>& pn, dfloat den) { return dfloat(penalty_of(pn.f, den.hi)); }

// H-apply of steppc.f90:53 / steprk.f90:74-75:
//   imaginary time: (lap*h2o2m4 - pot4*psi) - uimp*psi
//   real time:      i*(lap*h2o2m4 - pot4*psi) - i*uimp*psi
// hbar^2/2m_4 in the field precision and the time mode, built once per thread.
template <class T> struct HCoef {
  T h;
  int real_time;
  EP_DEV explicit HCoef(const Phys& ph) : h(PConst<T>(ph).h2o2m4), real_time(ph.time_mode == 1) {}
};
template <class T>
EP_DEV C2<T> happly(const HCoef<T>& hc, C2<T> lap, C2<T> psi, T pot4, T uimp) {
  if constexpr (sizeof(T) == 4) {  // paired FP32 instructions
    const C2<T> L = vfma(hc.h, lap, vmul(-pot4, psi));
    if (hc.real_time) return cmk<T>(-L.y + uimp * psi.y, L.x - uimp * psi.x);
    return vfma(-uimp, psi, L);
  }
  const T h = hc.h;
  C2<T> L = cmk<T>(lap.x * h - pot4 * psi.x, lap.y * h - pot4 * psi.y);
  if (hc.real_time) return cmk<T>(-L.y + uimp * psi.y, L.x - uimp * psi.x);
  return cmk<T>(L.x - uimp * psi.x, L.y - uimp * psi.y);
}

// <psi|H|psi> integrand from the H-apply output (Hpsi = -H or i*H).
template <class T>
EP_DEV double hexp(const Phys& ph, C2<T> psi, C2<T> H) {
  if (ph.time_mode == 1) return -(double)psi.x * H.y + (double)psi.y * H.x;
  return -((double)psi.x * H.x + (double)psi.y * H.y);
}

template <class T>
EP_DEV T hexp_t(const Phys& ph, C2<T> psi, C2<T> H) {
  if (ph.time_mode == 1) return -psi.x * H.y + psi.y * H.x;
  return -(psi.x * H.x + psi.y * H.y);
}

// ---------------------------------------------------------------------------
// X pass helpers (lines along x are contiguous; nl lines per CTA).
//
// Half-line transforms of N2 = nx/2 points.  N2 in {16, 32, 64, 128} (and
// in FP32 also 48, 80, 96) use
// xlines: P threads of one warp per line, E = N2/P points per thread, the
// two-factor decomposition of ep_rfft.cuh with the exchange done in place in
// the line's own shared-memory row (stride P+1 for the exchange), fenced by
// __syncwarp only.  The row stride x_row() makes the step-1 reads, the
// exchange and the step-2 reads conflict-free for 8- and 16-byte elements.
// N2 = 0 selects the general shared-memory Stockham engine.
template <int N2> struct XShape;
template <> struct XShape<16> { static constexpr int P = 4, E = 4; };
template <> struct XShape<32> { static constexpr int P = 4, E = 8; };
template <> struct XShape<64> { static constexpr int P = 8, E = 8; };
template <> struct XShape<128> { static constexpr int P = 8, E = 16; };
template <> struct XShape<48> { static constexpr int P = 4, E = 12; };
template <> struct XShape<80> { static constexpr int P = 4, E = 20; };
template <> struct XShape<96> { static constexpr int P = 4, E = 24; };

// the register transform length of half-lines of n2 points (0: the general
// engine); the mixed-radix lengths only in FP32, where the FP64 engine is
// bound by its arithmetic pipe either way
template <class T>
__host__ __device__ constexpr int x_reg_n2(int n2) {
  // double-float X passes run faster on the general engine (823 against 761
  // steps/s at 128^3): the register transforms' 4 lines per warp leave half of
  // a 16-line CTA waiting at its barriers
  return (!std::is_same<T, dfloat>::value && (n2 == 16 || n2 == 32 || n2 == 64 || n2 == 128)) ? n2
         : (sizeof(T) == 4 && (n2 == 48 || n2 == 80 || n2 == 96)) ? n2
                                                                    : 0;
}
// row stride (complex elements): >= n2 + 1 and >= E (P + 1), and congruent
// to P modulo 16 so that the lines sharing a half-warp fall on distinct banks
__host__ __device__ constexpr int x_row(int n2, int reg) {
  return !reg ? n2 + 1
              : (n2 == 16 ? 20 : n2 == 32 ? 52 : n2 == 48 ? 68 : n2 == 64 ? 72 : n2 == 80 ? 100 : n2 == 96 ? 132 : 152);
}
// shared memory of an X kernel: two line buffers, the twiddles exp(-2 pi i
// k/nx), the [ka][t] twiddle table of xlines, nreal real arrays
template <class T>
__host__ __device__ constexpr size_t x_smem_bytes(int nl, int nx, int nreal) {
  return 2 * (size_t)nl * x_row(nx / 2, x_reg_n2<T>(nx / 2)) * sizeof(C2<T>) + (size_t)nx * sizeof(C2<T>) +
         (size_t)(x_reg_n2<T>(nx / 2) ? nx / 2 : 0) * sizeof(C2<T>) + (size_t)nreal * nl * nx * sizeof(T);
}

template <class T, int N2, int DIR>
EP_DEV void xlines(C2<T>* A, int nl, int ld, const C2<T>* __restrict__ twt) {
  constexpr int P = XShape<N2>::P, E = XShape<N2>::E, LPW = 32 / P, Q = P + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int t = lane % P, lsub = lane / P;
  for (int base = warp * LPW; base < nl; base += nw * LPW) {
    const int l = base + lsub;
    const bool act = l < nl;
    C2<T>* row = A + (act ? l : 0) * ld;
    C2<T> v[E];
#pragma unroll
    for (int a = 0; a < E; ++a) v[a] = act ? row[t + P * a] : cmk<T>(T(0), T(0));
    epfft::dft<T, E, DIR>(v);
    if (t != 0) {
#pragma unroll
      for (int ka = 1; ka < E; ++ka) {
        const C2<T> w = twt[ka * P + t];
        v[ka] = DIR < 0 ? cmul(v[ka], w) : cmulc(v[ka], w);
      }
    }
    __syncwarp();
    if (act) {
#pragma unroll
      for (int ka = 0; ka < E; ++ka) row[ka * Q + t] = v[ka];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E / P; ++j) {
      C2<T> u[P];
#pragma unroll
      for (int tt = 0; tt < P; ++tt) u[tt] = row[(t + P * j) * Q + tt];
      epfft::dft<T, P, DIR>(u);
#pragma unroll
      for (int kt = 0; kt < P; ++kt) v[j + (E / P) * kt] = u[kt];
    }
    __syncwarp();
    if (act) {
#pragma unroll
      for (int m = 0; m < E; ++m) row[t + P * m] = v[m];
    }
  }
  __syncthreads();
}

// Transform nl lines held in A (B: scratch); returns the buffer with the result.
template <class T, int N2, int DIR>
EP_DEV const C2<T>* x_lines(C2<T>* A, C2<T>* B, int nl, int ld, const FftPlan& p2, const C2<T>* tw,
                            const C2<T>* twt) {
  if constexpr (N2 != 0) {
    xlines<T, N2, DIR>(A, nl, ld, twt);
    return A;
  } else {
    return epfft::lines<T, DIR>(A, B, nl, ld, p2, tw, 2);
  }
}

// Shared-memory carve-up of the X kernels.
template <class T>
struct XSmem {
  C2<T>* P;
  C2<T>* Q;
  C2<T>* tw;
  C2<T>* twt;  // [ka][t] twiddles of xlines
  T* R;        // nreal arrays of nl*nx
  int ld;
  EP_DEV XSmem(unsigned char* raw, int nl, int nx, int n2reg) {
    ld = x_row(nx / 2, n2reg);
    P = reinterpret_cast<C2<T>*>(raw);
    Q = P + nl * ld;
    tw = Q + nl * ld;
    twt = tw + nx;
    R = reinterpret_cast<T*>(twt + (n2reg ? nx / 2 : 0));
  }
  // tw and (for the register transforms) twt from the global table twx;
  // the caller synchronises before use
  template <int N2> EP_DEV void load_twiddles(const C2<T>* __restrict__ twx, int nx) {
    for (int i = threadIdx.x; i < nx; i += blockDim.x) tw[i] = twx[i];
    if constexpr (N2 != 0) {
      constexpr int P = XShape<N2>::P;
      for (int i = threadIdx.x; i < N2; i += blockDim.x) {
        const int ka = i / P, t = i - ka * P;
        twt[i] = twx[2 * t * ka];
      }
    }
  }
};

// Register-resident c2r of half-lines (N2 > 0): thread t of a line packs
// Z[k] = A + iB (c2r_pack's algebra) for its own k = t + P a straight from
// the spectrum in global memory, runs xlines' two steps and writes the real
// line (x = 2m, 2m+1) to Rout.
template <class T, int N2>
EP_DEV void x_inverse_reg(const C2<T>* __restrict__ spec, long long line0, int nlv, int nl, int nx, int nxh,
                          const XSmem<T>& S, T scale, T* Rout) {
  constexpr int P = XShape<N2>::P, E = XShape<N2>::E, LPW = 32 / P, Q = P + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int t = lane % P, lsub = lane / P;
  const C2<T>* tw = S.tw;
  for (int base = warp * LPW; base < nl; base += nw * LPW) {
    const int l = base + lsub;
    const bool act = l < nlv;
    const C2<T>* X = spec + (line0 + (act ? l : 0)) * nxh;
    C2<T> v[E];
#pragma unroll
    for (int a = 0; a < E; ++a) {
      const int k = t + P * a;
      const C2<T> xk = act ? X[k] : cmk<T>(T(0), T(0));
      const C2<T> xc = act ? conjg(X[N2 - k]) : cmk<T>(T(0), T(0));
      const C2<T> A = xk + xc;
      const C2<T> B = cmulc(xk - xc, tw[k]);
      v[a] = A + mul_i(B);
    }
    epfft::dft<T, E, +1>(v);
    if (t != 0) {
#pragma unroll
      for (int ka = 1; ka < E; ++ka) v[ka] = cmulc(v[ka], S.twt[ka * P + t]);
    }
    C2<T>* row = S.P + (l < nl ? l : 0) * S.ld;
    __syncwarp();
    if (l < nl) {
#pragma unroll
      for (int ka = 0; ka < E; ++ka) row[ka * Q + t] = v[ka];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E / P; ++j) {
      C2<T> u[P];
#pragma unroll
      for (int tt = 0; tt < P; ++tt) u[tt] = row[(t + P * j) * Q + tt];
      epfft::dft<T, P, +1>(u);
#pragma unroll
      for (int kt = 0; kt < P; ++kt) v[j + (E / P) * kt] = u[kt];
    }
    __syncwarp();
    if (l < nl) {
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int i = t + P * m;
        *reinterpret_cast<C2<T>*>(Rout + l * nx + 2 * i) = cmk<T>(v[m].x * scale, v[m].y * scale);
      }
    }
  }
  __syncthreads();
}

template <class T, int N2>
EP_DEV void x_inverse(const C2<T>* __restrict__ spec, long long line0, int nlv, int nl, int nx, int nxh,
                      const XSmem<T>& S, const FftPlan& p2, T scale, T* Rout) {
  if constexpr (N2 != 0) {
    x_inverse_reg<T, N2>(spec, line0, nlv, nl, nx, nxh, S, scale, Rout);
    return;
  }
  const int n2 = nx / 2, ld = S.ld;
  C2<T>* P = S.P;
  C2<T>* Q = S.Q;
  const float inv1 = 1.0f / (float)(n2 + 1), inv2 = 1.0f / (float)n2;
  for (int e = threadIdx.x; e < nl * (n2 + 1); e += blockDim.x) {
    int k;
    const int l = epfft::fdivmod(e, n2 + 1, inv1, k);
    P[l * ld + k] = l < nlv ? spec[(line0 + l) * nxh + k] : cmk<T>(T(0), T(0));
  }
  __syncthreads();
  epfft::c2r_pack<T>(P, ld, Q, ld, nl, n2, S.tw);
  __syncthreads();
  const C2<T>* z = x_lines<T, N2, +1>(Q, P, nl, ld, p2, S.tw, S.twt);
  for (int e = threadIdx.x; e < nl * n2; e += blockDim.x) {
    int m;
    const int l = epfft::fdivmod(e, n2, inv2, m);
    const C2<T> v = z[l * ld + m];
    Rout[l * nx + 2 * m] = v.x * scale;
    Rout[l * nx + 2 * m + 1] = v.y * scale;
  }
  __syncthreads();
}

// K consecutive values, moved as one 16-byte access when K * sizeof(T) == 16.
template <class T, int K> struct Pack {
  T v[K];
};
template <int K> struct KC {
  static constexpr int value = K;
};
template <class T, int K>
EP_DEV Pack<T, K> ldk(const T* p) {
  Pack<T, K> r;
  if constexpr (K == 1) {
    r.v[0] = *p;
  } else if constexpr (sizeof(T) == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    r.v[0] = q.x; r.v[1] = q.y; r.v[2] = q.z; r.v[3] = q.w;
  } else if constexpr (std::is_same<T, dfloat>::value) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    r.v[0] = dfloat(q.x, q.y); r.v[1] = dfloat(q.z, q.w);
  } else {
    const double2 q = *reinterpret_cast<const double2*>(p);
    r.v[0] = q.x; r.v[1] = q.y;
  }
  return r;
}
template <class T, int K>
EP_DEV void stk(T* p, const Pack<T, K>& r) {
  if constexpr (K == 1) {
    *p = r.v[0];
  } else if constexpr (sizeof(T) == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  } else if constexpr (std::is_same<T, dfloat>::value) {
    *reinterpret_cast<float4*>(p) = make_float4(r.v[0].hi, r.v[0].lo, r.v[1].hi, r.v[1].lo);
  } else {
    *reinterpret_cast<double2*>(p) = make_double2(r.v[0], r.v[1]);
  }
}
// Point-wise loop over the n contiguous points of an X-pass CTA:
// body(e, KC<K>) handles points e .. e+K-1, K = 16 / sizeof(T) when vec (the
// range and every array start 16-byte aligned: nx a multiple of K), else 1.
template <class T, class F>
EP_DEV void pointwise(int n, bool vec, F&& body) {
  constexpr int K = 16 / (int)sizeof(T);
  if (vec) {
    for (int e = threadIdx.x * K; e < n; e += blockDim.x * K) body(e, KC<K>());
  } else {
    for (int e = threadIdx.x; e < n; e += blockDim.x) body(e, KC<1>());
  }
}

// The pair (f[i], f[i+1]) of a line at an even index i, as one 8- or 16-byte
// load (rows of even length start aligned).
template <class T>
EP_DEV C2<T> ld2(const T* p) {
  return *reinterpret_cast<const C2<T>*>(p);
}

// Register-resident r2c of half-lines (N2 > 0): thread t packs its own
// z[m] = val(2m) + i val(2m+1) = pair(l, m), m = t + P a (one vector load
// per element from the caller's arrays, all issued before the transform),
// runs xlines' two steps, fetches
// the partner Z[N2 - k] of each of its outputs with a warp shuffle (lane
// P - t, register E - 1 - m; thread 0 holds its own partners) and writes
// r2c_unpack's X[k] straight to global memory (thread 0 also X[N2]).
template <class T, int N2, class F>
EP_DEV void x_forward_reg(F pair, C2<T>* __restrict__ out, long long line0, int nlv, int nl, int nxh,
                          const XSmem<T>& S) {
  constexpr int P = XShape<N2>::P, E = XShape<N2>::E, LPW = 32 / P, Q = P + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int t = lane % P, lsub = lane / P;
  const int plane = lane - t + (P - t) % P;
  const C2<T>* tw = S.tw;
  for (int base = warp * LPW; base < nl; base += nw * LPW) {
    const int l = base + lsub;
    const bool act = l < nlv;
    C2<T> v[E];
#pragma unroll
    for (int a = 0; a < E; ++a) {
      const int m = t + P * a;
      v[a] = act ? pair(l, m) : cmk<T>(T(0), T(0));
    }
    epfft::dft<T, E, -1>(v);
    if (t != 0) {
#pragma unroll
      for (int ka = 1; ka < E; ++ka) v[ka] = cmul(v[ka], S.twt[ka * P + t]);
    }
    C2<T>* row = S.P + (l < nl ? l : 0) * S.ld;
    __syncwarp();
    if (l < nl) {
#pragma unroll
      for (int ka = 0; ka < E; ++ka) row[ka * Q + t] = v[ka];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E / P; ++j) {
      C2<T> u[P];
#pragma unroll
      for (int tt = 0; tt < P; ++tt) u[tt] = row[(t + P * j) * Q + tt];
      epfft::dft<T, P, -1>(u);
#pragma unroll
      for (int kt = 0; kt < P; ++kt) v[j + (E / P) * kt] = u[kt];
    }
    __syncwarp();
    // v[m] = Z[t + P m]; w[m] = Z[(N2 - t - P m) mod N2]
    C2<T> w[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
      C2<T> u;
      u.x = __shfl_sync(0xffffffffu, v[j].x, plane);
      u.y = __shfl_sync(0xffffffffu, v[j].y, plane);
      w[E - 1 - j] = u;
    }
    if (t == 0) {
#pragma unroll
      for (int m = 0; m < E; ++m) w[m] = v[(E - m) % E];
    }
    if (act) {
      C2<T>* o = out + (line0 + l) * nxh;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int k = t + P * m;
        const C2<T> zk = v[m], zc = conjg(w[m]);
        const C2<T> e = epfft::K<T>::half * (zk + zc);
        const C2<T> od = epfft::K<T>::half * mul_mi(zk - zc);
        o[k] = e + cmul(tw[k], od);
      }
      if (t == 0) {
        const C2<T> zk = v[0], zc = conjg(v[0]);
        const C2<T> e = epfft::K<T>::half * (zk + zc);
        const C2<T> od = epfft::K<T>::half * mul_mi(zk - zc);
        o[N2] = e + cmul(tw[N2], od);
      }
    }
  }
  __syncthreads();
}

// Forward r2c of nl x-lines whose values are pair(l, m) = (val(l, 2m),
// val(l, 2m+1)).
template <class T, int N2, class F>
EP_DEV void x_forward(F pair, C2<T>* __restrict__ out, long long line0, int nlv, int nl, int nx, int nxh,
                      const XSmem<T>& S, const FftPlan& p2) {
  if constexpr (N2 != 0) {
    x_forward_reg<T, N2>(pair, out, line0, nlv, nl, nxh, S);
    return;
  }
  const int n2 = nx / 2, ld = S.ld;
  C2<T>* P = S.P;
  const float inv2 = 1.0f / (float)n2;
  for (int e = threadIdx.x; e < nl * n2; e += blockDim.x) {
    int m;
    const int l = epfft::fdivmod(e, n2, inv2, m);
    P[l * ld + m] = l < nlv ? pair(l, m) : cmk<T>(T(0), T(0));
  }
  __syncthreads();
  const C2<T>* Z = x_lines<T, N2, -1>(P, S.Q, nl, ld, p2, S.tw, S.twt);
  epfft::r2c_unpack<T>(Z, nl, ld, n2, S.tw, [&](int l, int k, C2<T> v) {
    if (l < nlv) out[(line0 + l) * nxh + k] = v;
  });
  __syncthreads();
}

// X1: den -> r2c along x (-> out).  grad den is k_d1march<MODE 0>.
template <class T, int N2>
__global__ void k_x1(Geo g, const T* __restrict__ den, C2<T>* __restrict__ out, const __grid_constant__ FftPlan p2,
                     const C2<T>* __restrict__ twx, int nl) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = g.nx;
  XSmem<T> S(smraw, nl, nx, N2);
  const long long nlines = (long long)g.ny * g.nz;
  const long long line0 = (long long)blockIdx.x * nl;
  const int nlv = (int)min((long long)nl, nlines - line0);
  S.template load_twiddles<N2>(twx, nx);
  __syncthreads();
  x_forward<T, N2>([&](int l, int m) { return ld2(den + (line0 + l) * nx + 2 * m); }, out, line0, nlv, nl, nx,
                   g.nxh, S, p2);
}

// X2: c2r of the three products of fden -> dencg, delj4 (and denalf for
// OTC); pot4 partial = delj4 + dencg^2 (a0 + a1 dencg) (poten.f90:34-92);
// forward r2c of den*dencg*(cp4 + cpp4*dencg) (poten.f90:62-67) and, for
// OTC, of f*grad(den), f = 1 - denalf/den0s (term_alfa.f90:157-170).
template <class T, int N2>
__global__ void k_x2(Geo g, Phys ph, const C2<T>* __restrict__ B0, const C2<T>* __restrict__ B1,
                     const C2<T>* __restrict__ B2, const T* __restrict__ den, const T* __restrict__ dxd,
                     const T* __restrict__ dyd, const T* __restrict__ dzd, T* __restrict__ dencg,
                     T* __restrict__ delj4, T* __restrict__ pot4, T* __restrict__ falfs, C2<T>* C0, C2<T>* C1,
                     C2<T>* C2o, C2<T>* C3, const __grid_constant__ FftPlan p2, const C2<T>* __restrict__ twx, int nl) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = g.nx, nxh = g.nxh;
  XSmem<T> S(smraw, nl, nx, N2);
  const bool otc = (ph.core == 1);
  const long long nlines = (long long)g.ny * g.nz;
  const long long line0 = (long long)blockIdx.x * nl;
  const int nlv = (int)min((long long)nl, nlines - line0);
  S.template load_twiddles<N2>(twx, nx);
  __syncthreads();
  T* Rcg = S.R;
  T* Rlj = S.R + nl * nx;
  T* Ral = S.R + 2 * nl * nx;
  const PConst<T> kc(ph);
  const T rn = kc.renor;
  x_inverse<T, N2>(B0, line0, nlv, nl, nx, nxh, S, p2, rn, Rcg);
  x_inverse<T, N2>(B1, line0, nlv, nl, nx, nxh, S, p2, rn, Rlj);
  if (otc) x_inverse<T, N2>(B2, line0, nlv, nl, nx, nxh, S, p2, rn, Ral);
  const T a0 = kc.a0, a1 = kc.a1, rden0s = kc.rden0s, cp4 = kc.cp4, cpp4 = kc.cpp4;
  const bool vec = nx % (16 / (int)sizeof(T)) == 0;
  pointwise<T>(nlv * nx, vec, [&](int e, auto kc) {
    constexpr int K = decltype(kc)::value;
    const long long p = line0 * nx + e;
    const Pack<T, K> cg = ldk<T, K>(Rcg + e), lj = ldk<T, K>(Rlj + e);
    Pack<T, K> pt;
#pragma unroll
    for (int k = 0; k < K; ++k) pt.v[k] = lj.v[k] + cg.v[k] * cg.v[k] * (a0 + a1 * cg.v[k]);
    stk<T, K>(dencg + p, cg);
    stk<T, K>(delj4 + p, lj);
    stk<T, K>(pot4 + p, pt);
    if (otc) {
      Pack<T, K> f = ldk<T, K>(Ral + e);
#pragma unroll
      for (int k = 0; k < K; ++k) f.v[k] = T(1) - f.v[k] * rden0s;
      stk<T, K>(falfs + p, f);
      stk<T, K>(Ral + e, f);  // the f * grad(den) transforms below reuse it
    }
  });
  __syncthreads();
  x_forward<T, N2>(
      [&](int l, int m) {
        const C2<T> cg = ld2(Rcg + l * nx + 2 * m), d = ld2(den + (line0 + l) * nx + 2 * m);
        return cmk<T>(d.x * cg.x * (cp4 + cpp4 * cg.x), d.y * cg.y * (cp4 + cpp4 * cg.y));
      },
      C0, line0, nlv, nl, nx, nxh, S, p2);
  if (otc) {
    // f * grad(den), one gradient component per transform
    const T* grad[3] = {dxd, dyd, dzd};
    C2<T>* outs[3] = {C1, C2o, C3};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T* gc = grad[c];
      x_forward<T, N2>(
          [&](int l, int m) {
            const C2<T> f = ld2(Ral + l * nx + 2 * m), d = ld2(gc + (line0 + l) * nx + 2 * m);
            return cmk<T>(f.x * d.x, f.y * d.y);
          },
          outs[c], line0, nlv, nl, nx, nxh, S, p2);
    }
  }
}

// X3: c2r of the correlation convolution -> pot4 (+ penalty for OT,
// poten.f90:74,88-92,122-126).  OTC: c2r of the three alpha_s integrals
// (term_alfa.f90:172-181), the x-derivative of f*I_x, f*I_y and f*I_z for
// the divergence (:216-225), and forward r2c of grad(den).I (:194-201).
template <class T, int N2>
__global__ void k_x3(Geo g, Phys ph, const __grid_constant__ FdW<T> fd, const C2<T>* __restrict__ D0, const C2<T>* __restrict__ D1,
                     const C2<T>* __restrict__ D2, const C2<T>* __restrict__ D3, const T* __restrict__ den,
                     const T* __restrict__ dxd, const T* __restrict__ dyd, const T* __restrict__ dzd,
                     const T* __restrict__ falfs, T* __restrict__ pot4, T* __restrict__ intx, T* __restrict__ inty,
                     T* __restrict__ intz, T* __restrict__ gy, T* __restrict__ gz, T* __restrict__ dgx,
                     C2<T>* E0, const __grid_constant__ FftPlan p2, const C2<T>* __restrict__ twx, int nl) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = g.nx, nxh = g.nxh;
  XSmem<T> S(smraw, nl, nx, N2);
  const bool otc = (ph.core == 1);
  const long long nlines = (long long)g.ny * g.nz;
  const long long line0 = (long long)blockIdx.x * nl;
  const int nlv = (int)min((long long)nl, nlines - line0);
  S.template load_twiddles<N2>(twx, nx);
  __syncthreads();
  const T rn = PConst<T>(ph).renor;
  T* Rc = S.R;
  x_inverse<T, N2>(D0, line0, nlv, nl, nx, nxh, S, p2, rn, Rc);
  if (!otc) {
    const Pen<T> pn(ph);
    pointwise<T>(nlv * nx, nx % (16 / (int)sizeof(T)) == 0, [&](int e, auto kc) {
      constexpr int K = decltype(kc)::value;
      const long long p = line0 * nx + e;
      Pack<T, K> pt = ldk<T, K>(pot4 + p);
      const Pack<T, K> rc = ldk<T, K>(Rc + e), dn = ldk<T, K>(den + p);
#pragma unroll
      for (int k = 0; k < K; ++k) pt.v[k] = (pt.v[k] + rc.v[k]) + penalty_of(pn, dn.v[k]);
      stk<T, K>(pot4 + p, pt);
    });
    return;
  }
  T* Rx = S.R + nl * nx;
  T* Ry = S.R + 2 * nl * nx;
  T* Rz = S.R + 3 * nl * nx;
  x_inverse<T, N2>(D1, line0, nlv, nl, nx, nxh, S, p2, rn, Rx);
  x_inverse<T, N2>(D2, line0, nlv, nl, nx, nxh, S, p2, rn, Ry);
  x_inverse<T, N2>(D3, line0, nlv, nl, nx, nxh, S, p2, rn, Rz);
  pointwise<T>(nlv * nx, nx % (16 / (int)sizeof(T)) == 0, [&](int e, auto kc) {
    constexpr int K = decltype(kc)::value;
    const long long p = line0 * nx + e;
    Pack<T, K> pt = ldk<T, K>(pot4 + p), rc = ldk<T, K>(Rc + e);
    const Pack<T, K> f = ldk<T, K>(falfs + p), rx = ldk<T, K>(Rx + e), ry = ldk<T, K>(Ry + e),
                     rz = ldk<T, K>(Rz + e);
    Pack<T, K> fy, fz;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      pt.v[k] = pt.v[k] + rc.v[k];
      fy.v[k] = f.v[k] * ry.v[k];
      fz.v[k] = f.v[k] * rz.v[k];
      rc.v[k] = f.v[k] * rx.v[k];
    }
    stk<T, K>(pot4 + p, pt);
    stk<T, K>(intx + p, rx);
    stk<T, K>(inty + p, ry);
    stk<T, K>(intz + p, rz);
    stk<T, K>(gy + p, fy);
    stk<T, K>(gz + p, fz);
    stk<T, K>(Rc + e, rc);
  });
  __syncthreads();
  for (int e = threadIdx.x; e < nlv * nx; e += blockDim.x) {
    int i;
      const int l = epfft::fdivmod(e, nx, 1.0f / (float)nx, i);
    dgx[line0 * nx + e] = d1_line(Rc + l * nx, i, nx, fd.w1[0], fd.R, fd.periodic);
  }
  x_forward<T, N2>(
      [&](int l, int m) {
        const int e = l * nx + 2 * m;
        const long long p = line0 * nx + e;
        const C2<T> gx = ld2(dxd + p), gy_ = ld2(dyd + p), gz_ = ld2(dzd + p);
        const C2<T> ix = ld2(Rx + e), iy = ld2(Ry + e), iz = ld2(Rz + e);
        return cmk<T>((gx.x * ix.x) + (gy_.x * iy.x) + (gz_.x * iz.x), (gx.y * ix.y) + (gy_.y * iy.y) + (gz_.y * iz.y));
      },
      E0, line0, nlv, nl, nx, nxh, S, p2);
}

// X4 (OTC): c2r of kalfs*FFT(grad(den).I) -> U_alpha = (u/den0s + div(f I))
// * h2o2m4 * alphas (term_alfa.f90:203-236); pot4 += U_alpha + penalty.
template <class T, int N2>
__global__ void k_x4(Geo g, Phys ph, const C2<T>* __restrict__ F0, const T* __restrict__ den,
                     const T* __restrict__ dgx, const T* __restrict__ dyz, T* __restrict__ pot4,
                     T* __restrict__ ualphas, const __grid_constant__ FftPlan p2, const C2<T>* __restrict__ twx, int nl) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = g.nx, nxh = g.nxh;
  XSmem<T> S(smraw, nl, nx, N2);
  const long long nlines = (long long)g.ny * g.nz;
  const long long line0 = (long long)blockIdx.x * nl;
  const int nlv = (int)min((long long)nl, nlines - line0);
  S.template load_twiddles<N2>(twx, nx);
  __syncthreads();
  T* Ru = S.R;
  const PConst<T> kc(ph);
  x_inverse<T, N2>(F0, line0, nlv, nl, nx, nxh, S, p2, kc.renor, Ru);
  const T rden0s = kc.rden0s, h2 = kc.h2o2m4, al = kc.alphas;
  const Pen<T> pn(ph);
  pointwise<T>(nlv * nx, nx % (16 / (int)sizeof(T)) == 0, [&](int e, auto kc) {
    constexpr int K = decltype(kc)::value;
    const long long p = line0 * nx + e;
    const Pack<T, K> ru = ldk<T, K>(Ru + e), gx = ldk<T, K>(dgx + p), yz = ldk<T, K>(dyz + p),
                     dn = ldk<T, K>(den + p);
    Pack<T, K> pt = ldk<T, K>(pot4 + p), ua;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      ua.v[k] = ((ru.v[k] * rden0s + gx.v[k]) + yz.v[k]) * h2 * al;
      pt.v[k] = (pt.v[k] + ua.v[k]) + penalty_of(pn, dn.v[k]);
    }
    stk<T, K>(ualphas + p, ua);
    stk<T, K>(pot4 + p, pt);
  });
}

// ---------------------------------------------------------------------------
// Strided complex passes (Y and Z).
template <class T>
struct LSmem {
  C2<T>* A;
  C2<T>* B;
  C2<T>* S;
  C2<T>* tw;
  long long* base;
  int ld;
};

template <class T>
EP_DEV LSmem<T> lsmem(unsigned char* raw, int LT, int n, int nbuf) {
  LSmem<T> s;
  s.ld = n + 1;
  s.A = reinterpret_cast<C2<T>*>(raw);
  s.B = s.A + LT * s.ld;
  s.S = nbuf > 2 ? s.B + LT * s.ld : nullptr;
  s.tw = s.B + (nbuf - 1) * LT * s.ld;
  s.base = reinterpret_cast<long long*>(s.tw + n);
  return s;
}

// Line loads/stores of the strided passes: LT is a power of two; up to 8
// loads per thread are issued before their shared-memory stores (ILP).
template <class T>
EP_DEV void load_lines(const C2<T>* __restrict__ a, const LSmem<T>& s, int LT, int n, long long Sa,
                       C2<T>* __restrict__ dst) {
  const int total = LT * n;
  const int lg = __ffs(LT) - 1;
  for (int e0 = threadIdx.x; e0 < total; e0 += 8 * blockDim.x) {
    C2<T> v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = e0 + i * blockDim.x;
      v[i] = cmk<T>(T(0), T(0));
      if (e < total) {
        const int k = e >> lg, t = e & (LT - 1);
        const long long b = s.base[t];
        if (b >= 0) v[i] = a[b + k * Sa];
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = e0 + i * blockDim.x;
      if (e < total) {
        const int k = e >> lg, t = e & (LT - 1);
        dst[t * s.ld + k] = v[i];
      }
    }
  }
}

template <class T>
EP_DEV void store_lines(C2<T>* __restrict__ a, const LSmem<T>& s, int LT, int n, long long Sa,
                        const C2<T>* __restrict__ src) {
  const int total = LT * n;
  const int lg = __ffs(LT) - 1;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int k = e >> lg, t = e & (LT - 1);
    const long long b = s.base[t];
    if (b >= 0) a[b + k * Sa] = src[t * s.ld + k];
  }
}

template <class T, int DIR>
__global__ void k_c2c(const __grid_constant__ Arr8<T> arr, LineSet ls, const __grid_constant__ FftPlan p, const C2<T>* __restrict__ twg, int LT) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int n = p.n;
  LSmem<T> s = lsmem<T>(smraw, LT, n, 2);
  C2<T>* a = arr.a[blockIdx.y];
  const long long L0 = (long long)blockIdx.x * LT;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.tw[i] = twg[i];
  for (int t = threadIdx.x; t < LT; t += blockDim.x) {
    const long long L = L0 + t;
    s.base[t] = L < ls.nlines ? (L % ls.Mi) + (L / ls.Mi) * ls.So : -1;
  }
  __syncthreads();
  load_lines<T>(a, s, LT, n, ls.Sa, s.A);
  __syncthreads();
  const C2<T>* r = epfft::lines<T, DIR>(s.A, s.B, LT, s.ld, p, s.tw, 1);
  store_lines<T>(a, s, LT, n, ls.Sa, r);
}

// Forward transform along the pass axis, then for each kernel table: multiply
// (the k-space product of poten.f90:34-36,46-48,69-71,95-97 and
// term_alfa.f90:172-176,203-205) and inverse transform.
template <class T>
__global__ void k_zconv(const __grid_constant__ ConvSpec<T> cs, LineSet ls, const __grid_constant__ FftPlan p, const C2<T>* __restrict__ twg, int LT) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int n = p.n;
  LSmem<T> s = lsmem<T>(smraw, LT, n, 3);
  const int which = blockIdx.y;
  const C2<T>* in = cs.in[which];
  const long long L0 = (long long)blockIdx.x * LT;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.tw[i] = twg[i];
  for (int t = threadIdx.x; t < LT; t += blockDim.x) {
    const long long L = L0 + t;
    s.base[t] = L < ls.nlines ? (L % ls.Mi) + (L / ls.Mi) * ls.So : -1;
  }
  __syncthreads();
  load_lines<T>(in, s, LT, n, ls.Sa, s.A);
  __syncthreads();
  C2<T>* r = epfft::lines<T, -1>(s.A, s.B, LT, s.ld, p, s.tw, 1);
  C2<T>* o1 = (r == s.A) ? s.B : s.A;
  C2<T>* o2 = s.S;
  for (int j = 0; j < cs.nout[which]; ++j) {
    const T* ker = cs.ker[which][j];
    const int lg = __ffs(LT) - 1;
    for (int e0 = threadIdx.x; e0 < LT * n; e0 += 8 * blockDim.x) {
      T kv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = e0 + i * blockDim.x;
        kv[i] = T(0);
        if (e < LT * n) {
          const long long b = s.base[e & (LT - 1)];
          if (b >= 0) kv[i] = ker[b + (e >> lg) * ls.Sa];
        }
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = e0 + i * blockDim.x;
        if (e < LT * n) {
          const int k = e >> lg, t = e & (LT - 1);
          const C2<T> v = r[t * s.ld + k];
          o1[t * s.ld + k] = cmk<T>(v.x * kv[i], v.y * kv[i]);
        }
      }
    }
    __syncthreads();
    const C2<T>* q = epfft::lines<T, +1>(o1, o2, LT, s.ld, p, s.tw, 1);
    store_lines<T>(cs.out[which][j], s, LT, n, ls.Sa, q);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// 2.5-D stencil march: a (TX x TY) tile of (x,y) columns walks z; the x/y
// neighbours of each plane come from a shared-memory tile with halo R, the
// z neighbours from a per-thread register queue.  The callback gets every
// grid point with lap = d2x + d2y + d2z (Deriv3D_pc,
// init_deriv_parallel.f90:923-1197, summed as steppc.f90:53).
#define EP_TX 32
#define EP_TY 8

// Shared memory of the pipelined march: two planes with halo, two z-queue
// slots, two copies of NC complex and NR real per-point inputs.
template <class T, int R, int NC, int NR>
constexpr size_t march_smem() {
  return (size_t)2 * (EP_TX + 2 * R) * (EP_TY + 2 * R) * sizeof(C2<T>) + (size_t)2 * EP_TX * EP_TY * sizeof(C2<T>) +
         (size_t)2 * NC * EP_TX * EP_TY * sizeof(C2<T>) + (size_t)2 * NR * EP_TX * EP_TY * sizeof(T) +
         (size_t)(EP_TX + 2 * R) * (EP_TY + 2 * R) * sizeof(int);
}

// The 2.5-D march, software-pipelined: while plane z is
// computed, cp.async brings plane z+1 (with halo), the z-queue element
// (x, y, z+1+R) and the NC complex / NR real per-point inputs of plane z+1
// into the other half of a double buffer.  f(p, psi, lap, ic, ir) gets the
// point's inputs as ic[i * NT] / ir[i * NT] in shared memory.  psi values
// are stored raw and multiplied by scale once (the Laplacian is linear).
// The (x, y) offsets of the halo plane (wrapped, or -1 outside a
// zero-boundary box) are tabulated once per CTA; each plane then costs one
// shared-memory read per element.
template <class T, int R, int NC, int NR, class F>
EP_DEV void lap_march_async(const Geo& g, const C2<T>* __restrict__ psi, const FdW<T>& fd, int zc,
                            unsigned char* smem, const C2<T>* const* cin, const T* const* rin, T scale, F&& f) {
  typedef C2<T> CT;
  constexpr int W = EP_TX + 2 * R, H = EP_TY + 2 * R, PL = W * H, NT = EP_TX * EP_TY;
  CT* sp = reinterpret_cast<CT*>(smem);
  CT* sq = sp + 2 * PL;
  CT* sc_ = sq + 2 * NT;
  T* sr = reinterpret_cast<T*>(sc_ + 2 * NC * NT);
  int* soff = reinterpret_cast<int*>(sr + 2 * NR * NT);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * EP_TX + tx;
  const int x = blockIdx.x * EP_TX + tx, y = blockIdx.y * EP_TY + ty;
  const int z0 = blockIdx.z * zc, z1 = min(z0 + zc, g.nz);
  const bool valid = (x < g.nx) && (y < g.ny);
  const int per = fd.periodic;
  const long long sxy = (long long)g.nx * g.ny;
  const long long xy = x + (long long)g.nx * y;
  auto addr = [&](int xx, int yy, int zz) -> long long {
    if (xx < 0 || xx >= g.nx || yy < 0 || yy >= g.ny || zz < 0 || zz >= g.nz) {
      if (!per) return -1;
      xx = wrapi(xx, g.nx);
      yy = wrapi(yy, g.ny);
      zz = wrapi(zz, g.nz);
    }
    return xx + (long long)g.nx * yy + sxy * zz;
  };
  // plane fetched in 16-byte chunks (two FP32 complex values) when the halo
  // and nx are chunk-aligned, else element by element
  constexpr int CH = 16 / (int)sizeof(CT);
  constexpr bool CHUNKED = CH > 1 && (R % CH) == 0 && (EP_TX % CH) == 0;
  const bool vec = CHUNKED && (g.nx % CH) == 0;
  const int ulen = vec ? CH : 1, uperrow = W / ulen, nunits = uperrow * H;
  for (int e = tid; e < nunits; e += NT) {
    const int r = e / uperrow, c = (e - r * uperrow) * ulen;
    int xx = blockIdx.x * EP_TX - R + c, yy = blockIdx.y * EP_TY - R + r;
    int o = -1;
    if (xx >= 0 && xx < g.nx && yy >= 0 && yy < g.ny) o = xx + g.nx * yy;
    else if (per) o = wrapi(xx, g.nx) + g.nx * wrapi(yy, g.ny);
    soff[e] = o;
  }
  __syncthreads();
  auto prefetch = [&](int z, int buf) {
    CT* P = sp + buf * PL;
    int zz = z;
    if (zz < 0 || zz >= g.nz) zz = per ? wrapi(zz, g.nz) : -1;
    const CT* pz = psi + sxy * (zz < 0 ? 0 : zz);
    if (CHUNKED && vec) {
      // chunks per row as a compile-time divisor (a multiply and a shift)
      constexpr int UPR = W / CH, NU = UPR * H;
      for (int e = tid; e < NU; e += NT) {
        const int r = e / UPR, c = (e - r * UPR) * CH;
        CT* dst = P + r * W + c;
        const int o = zz < 0 ? -1 : soff[e];
        if (o >= 0) {
          cp_async<16>(dst, pz + o);
        } else {
#pragma unroll
          for (int i = 0; i < CH; ++i) dst[i] = cmk<T>(T(0), T(0));
        }
      }
    } else {
      for (int e = tid; e < PL; e += NT) {
        const int o = zz < 0 ? -1 : soff[e];
        if (o >= 0) cp_async<sizeof(CT)>(P + e, pz + o);
        else P[e] = cmk<T>(T(0), T(0));
      }
    }
    if (valid) {
      // the z-queue element (x, y, z + R): only z can leave the box (z >= 0)
      int zq = z + R;
      const bool inq = zq < g.nz || per;
      if (zq >= g.nz) zq -= g.nz;
      if (inq) cp_async<sizeof(CT)>(sq + buf * NT + tid, psi + (xy + sxy * zq));
      else sq[buf * NT + tid] = cmk<T>(T(0), T(0));
      const long long p = xy + sxy * z;
#pragma unroll
      for (int i = 0; i < NC; ++i) cp_async<sizeof(CT)>(sc_ + (buf * NC + i) * NT + tid, cin[i] + p);
#pragma unroll
      for (int i = 0; i < NR; ++i) cp_async<sizeof(T)>(sr + (buf * NR + i) * NT + tid, rin[i] + p);
    }
    cp_commit();
  };
  CT q[2 * R + 1];
#pragma unroll
  for (int k = 0; k < 2 * R; ++k) {
    const long long a = valid ? addr(x, y, z0 - R + k) : -1;
    q[k] = a >= 0 ? psi[a] : cmk<T>(T(0), T(0));
  }
  prefetch(z0, 0);
  for (int z = z0; z < z1; ++z) {
    const int buf = (z - z0) & 1;
    // one barrier per plane: it publishes plane z and, as every thread has
    // finished plane z - 1, frees the other buffer for plane z + 1
    cp_wait<0>();
    __syncthreads();
    if (z + 1 < z1) prefetch(z + 1, buf ^ 1);
    if (valid) {
      q[2 * R] = sq[buf * NT + tid];
      const CT* row = sp + buf * PL + (ty + R) * W + (tx + R);
      const CT c = q[R];
      CT lap;
      if constexpr (std::is_same<T, dfloat>::value) {
#if defined(__CUDA_ARCH__)
        // unnormalised double-float accumulation, one sum per direction
        dd2_acc ax = dd2_start(fd.w2[0][0], c), ay = dd2_start(fd.w2[1][0], c), az = dd2_start(fd.w2[2][0], c);
        float2 ph, pl;
#pragma unroll
        for (int k = 1; k <= R; ++k) {
          dd2_wsum(fd.w2[0][k], row[-k], row[k], ph, pl);
          dd2_add(ax, ph, pl);
          dd2_wsum(fd.w2[1][k], row[-k * W], row[k * W], ph, pl);
          dd2_add(ay, ph, pl);
          dd2_wsum(fd.w2[2][k], q[R - k], q[R + k], ph, pl);
          dd2_add(az, ph, pl);
        }
        dd2_add(ax, ay.h, ay.l);
        dd2_add(ax, az.h, az.l);
        lap = dd2_value(ax);
#else
        lap = c;  // the host pass compiles no kernel body
#endif
      } else {
        CT lx = vmul(fd.w2[0][0], c), ly = vmul(fd.w2[1][0], c), lz = vmul(fd.w2[2][0], c);
#pragma unroll
        for (int k = 1; k <= R; ++k) {
          lx = vfma(fd.w2[0][k], vadd(row[-k], row[k]), lx);
          ly = vfma(fd.w2[1][k], vadd(row[-k * W], row[k * W]), ly);
          lz = vfma(fd.w2[2][k], vadd(q[R - k], q[R + k]), lz);
        }
        lap = vadd(vadd(lx, ly), lz);
      }
      f(xy + sxy * z, vmul(scale, c), vmul(scale, lap), sc_ + buf * NC * NT + tid, sr + buf * NR * NT + tid);
    }
#pragma unroll
    for (int k = 0; k < 2 * R; ++k) q[k] = q[k + 1];
  }
}

// The same march with two points per thread (FP32 fields, even R, even nx):
// thread (tx, ty) owns the x-neighbouring points 2 tx and 2 tx + 1 of a tile
// EP_PX = 2 EP_TX points wide.  Every plane element, z-queue element and
// complex input moves as a 16-byte pair of complex values (real inputs as
// 8-byte pairs), so a point costs half the shared-memory loads, copy and
// address instructions and barriers of the one-point form: the x-neighbours
// of a pair are R + 1 pairs of its row, the y-neighbours 2R pairs of its
// column.  Each point's Laplacian is summed in the one-point form's order,
// so both forms give the same bits.  f(p, psi, lap, ic, ir) gets the pair at
// the even index p, its inputs as ic[i * NT] / ir[i * NT].
#define EP_PX (2 * EP_TX)

template <int R, int NC, int NR>
constexpr size_t march_pair_smem() {
  return (size_t)2 * ((EP_PX + 2 * R) / 2) * (EP_TY + 2 * R) * sizeof(float4) +
         (size_t)2 * EP_TX * EP_TY * sizeof(float4) + (size_t)2 * NC * EP_TX * EP_TY * sizeof(float4) +
         (size_t)2 * NR * EP_TX * EP_TY * sizeof(float2) + (size_t)((EP_PX + 2 * R) / 2) * (EP_TY + 2 * R) * sizeof(int);
}

EP_DEV float2 lo2(float4 v) { return make_float2(v.x, v.y); }
EP_DEV float2 hi2(float4 v) { return make_float2(v.z, v.w); }
EP_DEV float4 cat2(float2 a, float2 b) { return make_float4(a.x, a.y, b.x, b.y); }

// The pair's Laplacian: e[] holds its row's elements x - R .. x + 1 + R,
// colp its column (rows R apart by pitch PITCH float4), q its z-queue.  Each
// point is summed in the order of the one-point march.
template <int R, int PITCH>
EP_DEV void pair_lap(const FdW<float>& fd, const float2* e, const float4* colp, const float4* q, float scale,
                     float4& c, float4& lap) {
  const float2 ca = lo2(q[R]), cb = hi2(q[R]);
  float2 lxa = vmul(fd.w2[0][0], ca), lya = vmul(fd.w2[1][0], ca), lza = vmul(fd.w2[2][0], ca);
  float2 lxb = vmul(fd.w2[0][0], cb), lyb = vmul(fd.w2[1][0], cb), lzb = vmul(fd.w2[2][0], cb);
#pragma unroll
  for (int k = 1; k <= R; ++k) {
    lxa = vfma(fd.w2[0][k], vadd(e[R - k], e[R + k]), lxa);
    lxb = vfma(fd.w2[0][k], vadd(e[R + 1 - k], e[R + 1 + k]), lxb);
    const float4 yn = colp[-k * PITCH], yp = colp[k * PITCH];
    lya = vfma(fd.w2[1][k], vadd(lo2(yn), lo2(yp)), lya);
    lyb = vfma(fd.w2[1][k], vadd(hi2(yn), hi2(yp)), lyb);
    const float4 zn = q[R - k], zp = q[R + k];
    lza = vfma(fd.w2[2][k], vadd(lo2(zn), lo2(zp)), lza);
    lzb = vfma(fd.w2[2][k], vadd(hi2(zn), hi2(zp)), lzb);
  }
  c = cat2(vmul(scale, ca), vmul(scale, cb));
  lap = cat2(vmul(scale, vadd(vadd(lxa, lya), lza)), vmul(scale, vadd(vadd(lxb, lyb), lzb)));
}

template <int R, int NC, int NR, class F>
EP_DEV void lap_march_pair(const Geo& g, const float2* __restrict__ psi, const FdW<float>& fd, int zc,
                           unsigned char* smem, const float2* const* cin, const float* const* rin, float scale,
                           F&& f) {
  static_assert(R % 2 == 0, "the pair march needs an even stencil radius");
  constexpr int W2 = (EP_PX + 2 * R) / 2, H = EP_TY + 2 * R, PL = W2 * H, NT = EP_TX * EP_TY, RH = R / 2;
  float4* sp = reinterpret_cast<float4*>(smem);
  float4* sq = sp + 2 * PL;
  float4* sc_ = sq + 2 * NT;
  float2* sr = reinterpret_cast<float2*>(sc_ + 2 * NC * NT);
  int* soff = reinterpret_cast<int*>(sr + 2 * NR * NT);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * EP_TX + tx;
  const int x = blockIdx.x * EP_PX + 2 * tx, y = blockIdx.y * EP_TY + ty;
  const int z0 = blockIdx.z * zc, z1 = min(z0 + zc, g.nz);
  const bool valid = (x < g.nx) && (y < g.ny);
  const int per = fd.periodic;
  const long long sxy = (long long)g.nx * g.ny;
  const long long xy = x + (long long)g.nx * y;
  // pair offsets of the halo plane (x even, so a pair never straddles the
  // wrap or the box edge); -1 outside a zero-boundary box
  for (int e = tid; e < PL; e += NT) {
    const int r = e / W2, c = e - r * W2;
    const int xx = blockIdx.x * EP_PX - R + 2 * c, yy = blockIdx.y * EP_TY - R + r;
    int o = -1;
    if (xx >= 0 && xx < g.nx && yy >= 0 && yy < g.ny) o = xx + g.nx * yy;
    else if (per) o = wrapi(xx, g.nx) + g.nx * wrapi(yy, g.ny);
    soff[e] = o;
  }
  __syncthreads();
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  auto zplane = [&](int zz) -> int {
    if (zz < 0 || zz >= g.nz) return per ? wrapi(zz, g.nz) : -1;
    return zz;
  };
  auto prefetch = [&](int z, int buf) {
    float4* P = sp + buf * PL;
    const int zz = zplane(z);
    const float2* pz = psi + sxy * (zz < 0 ? 0 : zz);
    for (int e = tid; e < PL; e += NT) {
      const int o = zz < 0 ? -1 : soff[e];
      if (o >= 0) cp_async<16>(P + e, pz + o);
      else P[e] = zero4;
    }
    if (valid) {
      const int zq = zplane(z + R);
      if (zq >= 0) cp_async<16>(sq + buf * NT + tid, psi + (xy + sxy * zq));
      else sq[buf * NT + tid] = zero4;
      const long long p = xy + sxy * z;
#pragma unroll
      for (int i = 0; i < NC; ++i) cp_async<16>(sc_ + (buf * NC + i) * NT + tid, cin[i] + p);
#pragma unroll
      for (int i = 0; i < NR; ++i) cp_async<8>(sr + (buf * NR + i) * NT + tid, rin[i] + p);
    }
    cp_commit();
  };
  float4 q[2 * R + 1];
#pragma unroll
  for (int k = 0; k < 2 * R; ++k) {
    const int zz = zplane(z0 - R + k);
    q[k] = (valid && zz >= 0) ? __ldg(reinterpret_cast<const float4*>(psi + (xy + sxy * zz))) : zero4;
  }
  prefetch(z0, 0);
  for (int z = z0; z < z1; ++z) {
    const int buf = (z - z0) & 1;
    // one barrier per plane: it publishes plane z and, as every thread has
    // finished plane z - 1, frees the other buffer for plane z + 1
    cp_wait<0>();
    __syncthreads();
    if (z + 1 < z1) prefetch(z + 1, buf ^ 1);
    if (valid) {
      q[2 * R] = sq[buf * NT + tid];
      // elements 2tx .. 2tx + 2R + 1 of the halo row (x - R .. x + 1 + R)
      const float4* rowp = sp + buf * PL + (ty + R) * W2 + tx;
      float2 e[2 * R + 2];
#pragma unroll
      for (int j = 0; j <= R; ++j) {
        const float4 v = rowp[j];
        e[2 * j] = lo2(v);
        e[2 * j + 1] = hi2(v);
      }
      float4 c, lap;
      pair_lap<R, W2>(fd, e, rowp + RH, q, scale, c, lap);
      f(xy + sxy * z, c, lap, sc_ + buf * NC * NT + tid, sr + buf * NR * NT + tid);
    }
#pragma unroll
    for (int k = 0; k < 2 * R; ++k) q[k] = q[k + 1];
  }
}

// Tensor maps of one TMA pair march (x in floats: a complex field is a
// float tensor of 2 nx x ny x nz): the marched field's boxes {128 x R},
// {128 x EP_TYT}, {16 x R} and {16 x EP_TYT} (floats x rows), a
// {128 x EP_TYT} box of each complex input and a {64 x EP_TYT} box of each
// real input.
// polls: the limit of each bounded mbarrier wait; no_copies: announce each
// plane's bytes but issue no copy (0; a failure-detection test sets it, so
// every wait runs out with nothing in flight).
struct MarchMaps {
  CUtensorMap halo[4];
  CUtensorMap cin[5];
  CUtensorMap rin[2];
  unsigned polls;
  unsigned no_copies;
};

// Kernel parameter of the predictor / corrector: the TMA form (PM = 2) takes
// its tensor maps, the other forms an empty placeholder.
struct NoMaps {
  int unused;
};
template <int PM> struct MapsOf { typedef NoMaps type; };
template <> struct MapsOf<2> { typedef MarchMaps type; };

// Polls of a bounded mbarrier wait (a few tens of milliseconds at least; a
// copy lands in microseconds).
#define EP_MBAR_POLLS (1u << 22)

// The TMA form's tile: EP_PX x EP_TYT points, 32 x EP_TYT threads (one CTA
// per SM), EP_MSTAGES plane buffers in flight.
#define EP_TYT 16
#define EP_MSTAGES 3

// Shared memory of the TMA pair march: per buffer the plane's centre columns
// (2R + EP_TYT rows of 64 points), its left and right columns (8 points
// each), the z-queue tile and the NC complex / NR real input tiles;
// EP_MSTAGES buffers, a 128-byte alignment pad and one mbarrier per buffer.
template <int R, int NC, int NR>
__host__ __device__ constexpr int march_tma_buf() {
  return (2 * R + EP_TYT) * EP_PX * 8 + 2 * (2 * R + EP_TYT) * 8 * 8 + (1 + NC) * EP_TX * EP_TYT * 16 +
         NR * EP_TX * EP_TYT * 8;
}
template <int R, int NC, int NR>
constexpr size_t march_tma_smem() {
  return 128 + EP_MSTAGES * (size_t)march_tma_buf<R, NC, NR>() + 8 * EP_MSTAGES;
}

// The pair march with every plane, z-queue tile and input tile brought in by
// TMA boxes that one thread issues (grids with nx a multiple of 64 and ny a
// multiple of EP_TYT): the plane's periodic halo is nine boxes -- left halo,
// centre and right halo columns by top halo, centre and bottom halo rows,
// each starting at its wrapped coordinate (in a zero-boundary box the boxes
// outside the tensor read zeros).  The row parts stack in shared memory; the
// left and right columns land in their own arrays and each thread keeps the
// shared-memory offsets of its R + 1 x-neighbour pairs.  Planes z + 1 and
// z + 2 are in flight while plane z is computed; one mbarrier per buffer
// counts the bytes, and a bounded wait that runs out raises EP_FLAG_TIMEOUT
// and ends the march of the block.
template <int R, int NC, int NR, class F>
EP_DEV void lap_march_pair_tma(const Geo& g, const float2* __restrict__ psi, const FdW<float>& fd, int zc,
                               unsigned char* smraw, const MarchMaps& mm, DevScalars* sc, float scale, F&& f) {
  static_assert(R % 2 == 0 && R <= 8, "the pair march needs an even stencil radius of at most 8");
  constexpr int TY = EP_TYT, NT = EP_TX * TY, RH = R / 2, HR = 2 * R + TY, S = EP_MSTAGES;
  constexpr int CB = HR * EP_PX * 8, LB = HR * 8 * 8, QB = NT * 16, IB = NT * 16, JB = NT * 8;
  constexpr int BUF = march_tma_buf<R, NC, NR>();
  unsigned char* smem =
      smraw + ((128u - (smem_u32(smraw) & 127u)) & 127u);  // 128-byte aligned TMA destinations
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * BUF);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * EP_TX + tx;
  const int bx = blockIdx.x * EP_PX, by = blockIdx.y * TY;
  const int x = bx + 2 * tx, y = by + ty;
  const int z0 = blockIdx.z * zc, z1 = min(z0 + zc, g.nz);
  const int per = fd.periodic;
  const long long sxy = (long long)g.nx * g.ny;
  const long long xy = x + (long long)g.nx * y;
  // float4 offsets (within a buffer) of the x-pairs tx .. tx + R of the
  // thread's extended row: left columns, centre columns, right columns
  int xo[R + 1];
  {
    const int r = ty + R;
#pragma unroll
    for (int i = 0; i <= R; ++i) {
      const int c = tx + i;
      xo[i] = c < RH ? HR * 32 + r * 4 + (4 - RH + c)
                     : (c < 32 + RH ? r * 32 + (c - RH) : HR * 36 + r * 4 + (c - 32 - RH));
    }
  }
  int xl = bx - 8, xr = bx + EP_PX, yt = by - R, yb = by + TY;
  if (per) {
    xl = wrapi(xl, g.nx);
    xr = wrapi(xr, g.nx);
    yt = wrapi(yt, g.ny);
    yb = wrapi(yb, g.ny);
  }
  auto issue = [&](int z, int b) {
    unsigned char* B = smem + b * BUF;
    uint64_t* bar = bars + b;
    fence_proxy_async();
    mbar_expect_tx(bar, (uint32_t)BUF);
    if (mm.no_copies) return;
    const int zq = per ? wrapi(z + R, g.nz) : z + R;  // beyond a zero-boundary box: zeros
    tma_load_3d(B, &mm.halo[0], 2 * bx, yt, z, bar);
    tma_load_3d(B + R * EP_PX * 8, &mm.halo[1], 2 * bx, by, z, bar);
    tma_load_3d(B + (R + TY) * EP_PX * 8, &mm.halo[0], 2 * bx, yb, z, bar);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      unsigned char* L = B + CB + s * LB;
      const int xs = 2 * (s ? xr : xl);
      tma_load_3d(L, &mm.halo[2], xs, yt, z, bar);
      tma_load_3d(L + R * 64, &mm.halo[3], xs, by, z, bar);
      tma_load_3d(L + (R + TY) * 64, &mm.halo[2], xs, yb, z, bar);
    }
    tma_load_3d(B + CB + 2 * LB, &mm.halo[1], 2 * bx, by, zq, bar);
#pragma unroll
    for (int i = 0; i < NC; ++i) tma_load_3d(B + CB + 2 * LB + QB + i * IB, &mm.cin[i], 2 * bx, by, z, bar);
#pragma unroll
    for (int i = 0; i < NR; ++i) tma_load_3d(B + CB + 2 * LB + QB + NC * IB + i * JB, &mm.rin[i], bx, by, z, bar);
  };
  if (tid == 0) {
#pragma unroll
    for (int b = 0; b < S; ++b) mbar_init(bars + b, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  constexpr int Q = 2 * R + 1;
  float4 q[Q];
#pragma unroll
  for (int k = 0; k < 2 * R; ++k) {
    int zz = z0 - R + k;
    if (zz < 0 || zz >= g.nz) zz = per ? wrapi(zz, g.nz) : -1;
    q[k] = zz >= 0 ? __ldg(reinterpret_cast<const float4*>(psi + (xy + sxy * zz))) : zero4;
  }
  if (tid == 0) {
#pragma unroll
    for (int b = 0; b < S - 1; ++b)
      if (z0 + b < z1) issue(z0 + b, b);
  }
  int b = 0;
  uint32_t par = 0;
  for (int z = z0; z < z1; ++z) {
    const bool ok = mbar_wait(bars + b, par, mm.polls);
    // one barrier per plane: every thread has finished plane z - 1, so its
    // buffer takes plane z + S - 1
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(&sc->flags, (unsigned)EP_FLAG_TIMEOUT);
        // the copies still in flight, once more each
        for (int k = 0; k < S - 1 && z + k < z1; ++k) {
          const int bk = (b + k) % S;
          mbar_wait(bars + bk, par ^ (bk < b ? 1u : 0u), mm.polls);
        }
      }
      break;
    }
    if (tid == 0 && z + S - 1 < z1) issue(z + S - 1, (b + S - 1) % S);
    const unsigned char* B = smem + b * BUF;
    const float4* B4 = reinterpret_cast<const float4*>(B);
    q[2 * R] = B4[(CB + 2 * LB) / 16 + tid];
    float2 e[2 * R + 2];
#pragma unroll
    for (int i = 0; i <= R; ++i) {
      const float4 v = B4[xo[i]];
      e[2 * i] = lo2(v);
      e[2 * i + 1] = hi2(v);
    }
    float4 c, lap;
    pair_lap<R, 32>(fd, e, B4 + (ty + R) * 32 + tx, q, scale, c, lap);
    f(xy + sxy * z, c, lap, reinterpret_cast<const float4*>(B + CB + 2 * LB + QB) + tid,
      reinterpret_cast<const float2*>(B + CB + 2 * LB + QB + NC * IB) + tid);
#pragma unroll
    for (int k = 0; k < 2 * R; ++k) q[k] = q[k + 1];
    if (++b == S) {
      b = 0;
      par ^= 1u;
    }
  }
}

// First derivatives of real fields by a 2.5-D march, software-pipelined like
// lap_march_async (13-point derivnd stencils, init_deriv_parallel.f90, with
// the boundary handling and summation order of d1_global):
//   MODE 0: o0, o1, o2 = d/dx, d/dy, d/dz of f   (derden, energy.f90:207-227)
//   MODE 1: o0 = d/dy f + d/dz f2                (term_alfa.f90:220-230)
// Each thread computes two x-neighbouring points (x even), so every
// neighbour in shared memory, the z-queue and every store move as pairs
// (8-byte FP32 / 16-byte FP64 accesses), and the y and z sums of the pair
// are paired FP32 instructions (each point summed in the scalar order).
#define EP_D1_TX (2 * EP_TX)  // x points of a CTA row
template <class T, int R, int MODE>
__global__ void __launch_bounds__(EP_TX* EP_TY) k_d1march(Geo g, const __grid_constant__ FdW<T> fd, int zc,
                                                         const T* __restrict__ f, const T* __restrict__ f2,
                                                         T* __restrict__ o0, T* __restrict__ o1,
                                                         T* __restrict__ o2) {
  typedef C2<T> PT;
  // The plane tile (x halo rounded up to whole 16-byte chunks) is fetched
  // chunk by chunk when nx is a multiple of the chunk; element by element
  // otherwise.  Offsets of chunks (or elements) are tabulated once per CTA.
  constexpr int CH = 16 / (int)sizeof(T);
  constexpr int HX = MODE == 0 ? ((R + CH - 1) / CH) * CH : 0;
  constexpr int W = EP_D1_TX + 2 * HX, H = EP_TY + 2 * R, PL = W * H, NT = EP_TX * EP_TY;
  constexpr int WC = W / CH, PC = WC * H, WP = W / 2;
  constexpr int JLO = -((R + 1) / 2), JHI = (R + 1) / 2, NE = 2 * (JHI - JLO + 1);
  static_assert(HX >= -2 * JLO || MODE != 0, "x halo");
  __shared__ __align__(16) T sp[2][PL];
  __shared__ __align__(16) PT sq[2][NT];
  __shared__ int soff[PL];
  const T* fq = MODE == 0 ? f : f2;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * EP_TX + tx;
  const int x = blockIdx.x * EP_D1_TX + 2 * tx, y = blockIdx.y * EP_TY + ty;
  const int z0 = blockIdx.z * zc, z1 = min(z0 + zc, g.nz);
  const bool valid = (x < g.nx) && (y < g.ny);  // nx is even: x + 1 < nx too
  const int per = fd.periodic;
  const bool vec = (g.nx % CH) == 0;
  const int nunits = vec ? PC : PL, ulen = vec ? CH : 1, uperrow = vec ? WC : W;
  const long long sxy = (long long)g.nx * g.ny;
  for (int e = tid; e < nunits; e += NT) {
    const int r = e / uperrow, c = (e - r * uperrow) * ulen;
    const int xx = blockIdx.x * EP_D1_TX - HX + c, yy = blockIdx.y * EP_TY - R + r;
    int o = -1;
    if (xx >= 0 && xx < g.nx && yy >= 0 && yy < g.ny) o = xx + g.nx * yy;
    else if (per) o = wrapi(xx, g.nx) + g.nx * wrapi(yy, g.ny);
    soff[e] = o;
  }
  auto zwrap = [&](int zz) -> int {
    if (zz < 0 || zz >= g.nz) return per ? wrapi(zz, g.nz) : -1;
    return zz;
  };
  const long long pxy = (long long)x + (long long)g.nx * y;
  PT q[2 * R + 1];
#pragma unroll
  for (int k = 0; k < 2 * R; ++k) {
    const int zz = zwrap(z0 - R + k);
    q[k] = (valid && zz >= 0) ? *reinterpret_cast<const PT*>(fq + pxy + sxy * zz) : cmk<T>(T(0), T(0));
  }
  __syncthreads();
  auto prefetch = [&](int z, int buf) {
    const int zz = zwrap(z);
    const T* pz = f + sxy * (zz < 0 ? 0 : zz);
    if (vec) {
      for (int e = tid; e < PC; e += NT) {
        const int r = e / WC, c = (e - r * WC) * CH;
        T* dst = &sp[buf][r * W + c];
        const int o = zz < 0 ? -1 : soff[e];
        if (o >= 0) {
          cp_async<16>(dst, pz + o);
        } else {
#pragma unroll
          for (int i = 0; i < CH; ++i) dst[i] = T(0);
        }
      }
    } else {
      for (int e = tid; e < PL; e += NT) {
        const int o = zz < 0 ? -1 : soff[e];
        if (o >= 0) cp_async<sizeof(T)>(&sp[buf][e], pz + o);
        else sp[buf][e] = T(0);
      }
    }
    if (valid) {
      const int zq = zwrap(z + R);
      if (zq >= 0) cp_async<sizeof(PT)>(&sq[buf][tid], fq + pxy + sxy * zq);
      else sq[buf][tid] = cmk<T>(T(0), T(0));
    }
    cp_commit();
  };
  prefetch(z0, 0);
  for (int z = z0; z < z1; ++z) {
    const int buf = (z - z0) & 1;
    cp_wait<0>();  // one barrier per plane, as in lap_march_async
    __syncthreads();
    if (z + 1 < z1) prefetch(z + 1, buf ^ 1);
    if (valid) {
      q[2 * R] = sq[buf][tid];
      // row element x of this thread (even offset: W, HX and 2 tx are even)
      const T* rowe = &sp[buf][(ty + R) * W + HX + 2 * tx];
      const PT* rowp = reinterpret_cast<const PT*>(rowe);
      const long long p = pxy + sxy * z;
      PT dy = cmk<T>(T(0), T(0)), dz = cmk<T>(T(0), T(0));
      if constexpr (std::is_same<T, dfloat>::value) {
#if defined(__CUDA_ARCH__)
        // unnormalised double-float accumulation of the pair's y and z sums
        dd2_acc ay, az;
        dd2_wdiff(fd.w1[1][1], rowp[WP], rowp[-WP], ay.h, ay.l);
        dd2_wdiff(fd.w1[2][1], q[R + 1], q[R - 1], az.h, az.l);
        float2 ph, pl;
#pragma unroll
        for (int k = 2; k <= R; ++k) {
          dd2_wdiff(fd.w1[1][k], rowp[k * WP], rowp[-k * WP], ph, pl);
          dd2_add(ay, ph, pl);
          dd2_wdiff(fd.w1[2][k], q[R + k], q[R - k], ph, pl);
          dd2_add(az, ph, pl);
        }
        dy = dd2_value(ay);
        dz = dd2_value(az);
#endif
      } else {
#pragma unroll
        for (int k = 1; k <= R; ++k) dy = vfma(fd.w1[1][k], vsub(rowp[k * WP], rowp[-k * WP]), dy);
#pragma unroll
        for (int k = 1; k <= R; ++k) dz = vfma(fd.w1[2][k], vsub(q[R + k], q[R - k]), dz);
      }
      if (MODE == 0) {
        // elements x + JLO*2 .. x + 2*JHI + 1 of the row, as pairs
        T e[NE];
#pragma unroll
        for (int j = JLO; j <= JHI; ++j) {
          const PT v = rowp[j];
          e[2 * (j - JLO)] = v.x;
          e[2 * (j - JLO) + 1] = v.y;
        }
        PT dx = cmk<T>(T(0), T(0));
#pragma unroll
        for (int k = 1; k <= R; ++k) {
          dx.x += fd.w1[0][k] * (e[k - 2 * JLO] - e[-k - 2 * JLO]);
          dx.y += fd.w1[0][k] * (e[1 + k - 2 * JLO] - e[1 - k - 2 * JLO]);
        }
        *reinterpret_cast<PT*>(o0 + p) = dx;
        *reinterpret_cast<PT*>(o1 + p) = dy;
        *reinterpret_cast<PT*>(o2 + p) = dz;
      } else {
        *reinterpret_cast<PT*>(o0 + p) = cmk<T>(dy.x + dz.x, dy.y + dz.y);
      }
    }
#pragma unroll
    for (int k = 0; k < 2 * R; ++k) q[k] = q[k + 1];
  }
}

// Scale slots of the buffers a stencil kernel touches (see DevScalars).
struct Slots {
  int psi, a, b, h1, h2, pc, out;
};

// Last block of a kernel (every other block has finished and counted):
// returns true in all threads of that block.
EP_DEV bool last_block(unsigned int* counter) {
  __shared__ bool last;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == nb - 1;
  }
  __syncthreads();
  return last;
}

// Predictor + modifier of steppc.f90:53-64.  The new psi is written over
// psiold(ioldp(3)) (read here point-wise), so the host swaps buffers instead
// of copying.
// PM: 0 one point per thread, 1 two points per thread staged by cp.async,
// 2 two points per thread staged by TMA boxes.
template <class T, int R, int PM>
__global__ void __launch_bounds__(PM == 2 ? EP_TX * EP_TYT : EP_TX * EP_TY, PM == 2 ? 1 : (PM ? 2 : (sizeof(T) == 4 ? 4 : 2))) k_predict(Geo g, FdW<T> fd, Phys ph, int zc,
                                                         const C2<T>* __restrict__ psi, const T* __restrict__ pot4,
                                                         const T* __restrict__ uimp, C2<T>* po3,
                                                         const C2<T>* __restrict__ h1, C2<T>* h2, C2<T>* pc,
                                                         T* __restrict__ den, T f, T c112, DevScalars* sc,
                                                         Slots sl, const __grid_constant__ typename MapsOf<PM>::type mm) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int NT = EP_TX * (PM == 2 ? EP_TYT : EP_TY);
  const HCoef<T> hc(ph);
  // buffer scales folded into the method's coefficients once per thread:
  // pp = s3 po3 + f (2 H - s1 h1 + 2 s2 h2), pn = pp - c112 sp pc
  const T s3 = bscale_of<T>(sc, sl.a), k2f = T(2) * f, kh1 = f * bscale_of<T>(sc, sl.h1),
          kh2 = (T(2) * f) * bscale_of<T>(sc, sl.h2), kpc = c112 * bscale_of<T>(sc, sl.pc);
  const C2<T>* cin[4] = {po3, h1, h2, pc};
  const T* rin[2] = {pot4, uimp};
  // one point: H psi, the predictor pp and the modified value pn, from psi,
  // its Laplacian, po3, h1, h2, pc, pot4 and uimp
  auto point = [&](C2<T> c, C2<T> lap, C2<T> a3, C2<T> b1, C2<T> b2, C2<T> opc, T v, T u, C2<T>& H, C2<T>& pp,
                   C2<T>& pn) {
    H = happly<T>(hc, lap, c, v, u);
    if constexpr (sizeof(T) == 4) {
      pp = vfma(kh2, b2, vfma(-kh1, b1, vfma(k2f, H, vmul(s3, a3))));
      pn = vfma(-kpc, opc, pp);
    } else {
      pp = ((s3 * a3 + k2f * H) - kh1 * b1) + kh2 * b2;
      pn = pp - kpc * opc;
    }
  };
  if constexpr (PM != 0) {
    auto pairf = [&](long long p, float4 c, float4 lap, const float4* ic, const float2* ir) {
      float2 Ha, ppa, pna, Hb, ppb, pnb;
      point(lo2(c), lo2(lap), lo2(ic[0]), lo2(ic[NT]), lo2(ic[2 * NT]), lo2(ic[3 * NT]), ir[0].x, ir[NT].x, Ha, ppa,
            pna);
      point(hi2(c), hi2(lap), hi2(ic[0]), hi2(ic[NT]), hi2(ic[2 * NT]), hi2(ic[3 * NT]), ir[0].y, ir[NT].y, Hb, ppb,
            pnb);
      *reinterpret_cast<float4*>(po3 + p) = cat2(pna, pnb);
      *reinterpret_cast<float4*>(pc + p) = cat2(ppa, ppb);
      *reinterpret_cast<float4*>(h2 + p) = cat2(Ha, Hb);
      *reinterpret_cast<float2*>(den + p) = make_float2(pna.x * pna.x + pna.y * pna.y, pnb.x * pnb.x + pnb.y * pnb.y);
    };
    if constexpr (PM == 2) lap_march_pair_tma<R, 4, 2>(g, psi, fd, zc, smraw, mm, sc, bscale_of<T>(sc, sl.psi), pairf);
    else lap_march_pair<R, 4, 2>(g, psi, fd, zc, smraw, cin, rin, bscale_of<T>(sc, sl.psi), pairf);
  } else {
    lap_march_async<T, R, 4, 2>(
        g, psi, fd, zc, smraw, cin, rin, bscale_of<T>(sc, sl.psi),
        [&](long long p, C2<T> c, C2<T> lap, const C2<T>* ic, const T* ir) {
          C2<T> H, pp, pn;
          point(c, lap, ic[0], ic[NT], ic[2 * NT], ic[3 * NT], ir[0], ir[NT], H, pp, pn);
          po3[p] = pn;
          pc[p] = pp;
          h2[p] = H;
          den[p] = pn.x * pn.x + pn.y * pn.y;
        });
  }
  if (last_block(&sc->counter2)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      sc->bscale[sl.a] = 1.0;
      sc->bscale[sl.h2] = 1.0;
      sc->bscale[sl.pc] = 1.0;
      sc->bscale_f[sl.a] = 1.0f;
      sc->bscale_f[sl.h2] = 1.0f;
      sc->bscale_f[sl.pc] = 1.0f;
      sc->den_scale = 1.0;
      sc->counter2 = 0u;
    }
  }
}

// Corrector + final value of steppc.f90:135-151 with fused reductions:
// sum |pc|, sum |psi|^2 (new), <psi|H|psi> and sum |psi|^2 of the modified
// psi (chemical potential).
template <class T, int R, bool STATS, int PM>
__global__ void __launch_bounds__(PM == 2 ? EP_TX * EP_TYT : EP_TX * EP_TY, PM == 2 ? 1 : (PM ? 2 : (sizeof(T) == 4 ? 3 : 2))) k_correct(Geo g, FdW<T> fd, Phys ph, int zc,
                                                         const C2<T>* __restrict__ psi, const T* __restrict__ pot4,
                                                         const T* __restrict__ uimp,
                                                         const C2<T>* __restrict__ po3,
                                                         const C2<T>* __restrict__ po2,
                                                         const C2<T>* __restrict__ h1,
                                                         const C2<T>* __restrict__ h2, C2<T>* pc,
                                                         C2<T>* __restrict__ out, T* __restrict__ den, T f3, T c9,
                                                         double* __restrict__ partials, DevScalars* sc, int renorm,
                                                         double n4, Slots sl,
                                                         const __grid_constant__ typename MapsOf<PM>::type mm) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int NT = EP_TX * (PM == 2 ? EP_TYT : EP_TY);
  const HCoef<T> hc(ph);
  Kahan<T> acc[4];
  // buffer scales folded into the method's coefficients once per thread:
  // p5 = (9 s3 po3 - s2o po2 + f3 (H + 2 s1 h1 - s2 h2)) / 8
  const T k3 = T(1.125) * bscale_of<T>(sc, sl.a), k2o = T(0.125) * bscale_of<T>(sc, sl.b), kH = T(0.125) * f3,
          k1 = (T(0.25) * f3) * bscale_of<T>(sc, sl.h1), k2 = (T(0.125) * f3) * bscale_of<T>(sc, sl.h2),
          sp_ = bscale_of<T>(sc, sl.pc);
  const C2<T>* cin[5] = {po3, po2, h1, h2, pc};
  const T* rin[2] = {pot4, uimp};
  // one point: the corrected pc and the final psi from psi, its Laplacian,
  // po3, po2, h1, h2, pc, pot4 and uimp; returns |psi|^2 and adds the point
  // to the reductions
  auto point = [&](C2<T> c, C2<T> lap, C2<T> a3, C2<T> a2, C2<T> b1, C2<T> b2, C2<T> opc, T v, T u, C2<T>& pcn,
                   C2<T>& po) -> T {
    const C2<T> H = happly<T>(hc, lap, c, v, u);
    C2<T> p5;
    if constexpr (sizeof(T) == 4) {
      p5 = vfma(-k2, b2, vfma(k1, b1, vfma(kH, H, vfma(-k2o, a2, vmul(k3, a3)))));
      pcn = vsub(vmul(sp_, opc), p5);
      po = vfma(c9, pcn, p5);
    } else {
      p5 = (((k3 * a3 - k2o * a2) + kH * H) + k1 * b1) - k2 * b2;
      pcn = sp_ * opc - p5;
      po = p5 + c9 * pcn;
    }
    const T dn = po.x * po.x + po.y * po.y;
    acc[1].add(dn);
    if (STATS) {  // errHe and mu are read only when the caller asks for them
      acc[0].add(sqrt(pcn.x * pcn.x + pcn.y * pcn.y));
      acc[2].add(hexp_t<T>(ph, c, H));
      acc[3].add(c.x * c.x + c.y * c.y);
    }
    return dn;
  };
  if constexpr (PM != 0) {
    auto pairf = [&](long long p, float4 c, float4 lap, const float4* ic, const float2* ir) {
      float2 pca, poa, pcb, pob;
      const float da = point(lo2(c), lo2(lap), lo2(ic[0]), lo2(ic[NT]), lo2(ic[2 * NT]), lo2(ic[3 * NT]),
                             lo2(ic[4 * NT]), ir[0].x, ir[NT].x, pca, poa);
      const float db = point(hi2(c), hi2(lap), hi2(ic[0]), hi2(ic[NT]), hi2(ic[2 * NT]), hi2(ic[3 * NT]),
                             hi2(ic[4 * NT]), ir[0].y, ir[NT].y, pcb, pob);
      *reinterpret_cast<float4*>(pc + p) = cat2(pca, pcb);
      *reinterpret_cast<float4*>(out + p) = cat2(poa, pob);
      *reinterpret_cast<float2*>(den + p) = make_float2(da, db);
    };
    if constexpr (PM == 2) lap_march_pair_tma<R, 5, 2>(g, psi, fd, zc, smraw, mm, sc, bscale_of<T>(sc, sl.psi), pairf);
    else lap_march_pair<R, 5, 2>(g, psi, fd, zc, smraw, cin, rin, bscale_of<T>(sc, sl.psi), pairf);
  } else {
    lap_march_async<T, R, 5, 2>(g, psi, fd, zc, smraw, cin, rin, bscale_of<T>(sc, sl.psi),
                                [&](long long p, C2<T> c, C2<T> lap, const C2<T>* ic, const T* ir) {
      C2<T> pcn, po;
      den[p] = point(c, lap, ic[0], ic[NT], ic[2 * NT], ic[3 * NT], ic[4 * NT], ir[0], ir[NT], pcn, po);
      pc[p] = pcn;
      out[p] = po;
    });
  }
  // without STATS only the norm (q = 1) is reduced and finalised
  constexpr unsigned QM = STATS ? 0xFu : 0x2u;
  block_reduce_store_acc<4, QM>(acc, partials);
  // The last block to finish sums all partials (no block waits for another).
  __shared__ bool last;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
  if (tid == 0) {
    __threadfence();
    last = atomicAdd(&sc->counter, 1u) == nb - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    finalize_block(partials, (int)nb, 4, sc, 0, 1, (double)g.N, ph.dxyz, n4, renorm, STATS ? 1 : 0, QM);
    if (tid == 0) {
      // renormalise lazily: every logical state value is multiplied by s;
      // the buffers written here restart their scale at s
      const double s = sc->scale;
      for (int k = 0; k < EP_NSLOTS; ++k) sc->bscale[k] *= s;
      sc->bscale[sl.pc] = s;
      sc->bscale[sl.out] = s;
      for (int k = 0; k < EP_NSLOTS; ++k) sc->bscale_f[k] = (float)sc->bscale[k];
      sc->den_scale = s * s;
      sc->counter = 0u;
    }
  }
}

// One Runge-Kutta-Gill stage of steprk.f90:71-89 (jrun-independent part) on
// the pipelined march (q, pot4 and uimp of the next plane arrive with its
// halo); the first stage also records H into hout (the history shift itself
// is done by rotating buffers).  den <= 0 raises a flag (steprk.f90:94-110).
// psi is materialised before steprk (no pending renormalisation scale).
template <class T, int R>
__global__ void __launch_bounds__(EP_TX* EP_TY, sizeof(T) == 4 ? 4 : 2) k_rkstage(Geo g, FdW<T> fd, Phys ph, int zc,
                                                         const C2<T>* __restrict__ psi, const T* __restrict__ pot4,
                                                         const T* __restrict__ uimp, C2<T>* q,
                                                         C2<T>* __restrict__ out, C2<T>* __restrict__ hout,
                                                         T* __restrict__ den, T a, T b, T cr, T dt,
                                                         DevScalars* sc) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int NT = EP_TX * EP_TY;
  const HCoef<T> hc(ph);
  bool bad = false;
  const C2<T>* cin[1] = {q};
  const T* rin[2] = {pot4, uimp};
  lap_march_async<T, R, 1, 2>(g, psi, fd, zc, smraw, cin, rin, T(1),
                              [&](long long p, C2<T> c, C2<T> lap, const C2<T>* ic, const T* ir) {
    const C2<T> H = happly<T>(hc, lap, c, ir[0], ir[NT]);
    const C2<T> qq = ic[0];
    const C2<T> aux2 = a * (H - b * qq);
    q[p] = (qq + T(3) * aux2) - cr * H;
    if (hout) hout[p] = H;
    const C2<T> pn = c + dt * aux2;
    out[p] = pn;
    const T dn = pn.x * pn.x + pn.y * pn.y;
    den[p] = dn;
    if (!(dn > T(0))) bad = true;
  });
  if (bad) atomicOr(&sc->flags, (unsigned)EP_FLAG_DEN_NONPOS);
}

// ---------------------------------------------------------------------------
// Point-wise kernels.
template <class T>
__global__ void k_psi_to_den(const C2<T>* __restrict__ psi, T* __restrict__ den, long long N) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const C2<T> v = psi[i];
    den[i] = v.x * v.x + v.y * v.y;
  }
}

// Imaginary-time renormalisation with the factor the finalize kernel left
// in sc->scale: psi and the whole multistep history (psiold x3, hpsiold x2,
// pc) are scaled together so they keep describing one trajectory.
template <class T>
struct HistPtrs { C2<T>* h[6]; };
template <class T>
__global__ void k_rescale(C2<T>* __restrict__ psi, T* __restrict__ den, HistPtrs<T> hist, long long N,
                          const DevScalars* __restrict__ sc) {
  const T s = (T)sc->scale;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    C2<T> v = psi[i];
    v.x *= s;
    v.y *= s;
    psi[i] = v;
    den[i] = v.x * v.x + v.y * v.y;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      C2<T> w = hist.h[k][i];
      w.x *= s;
      w.y *= s;
      hist.h[k][i] = w;
    }
  }
}

// Apply the pending scales to the state buffers and den (then the scales
// are reset by k_reset_scales, launched after this kernel).
template <class T>
struct SlotPtrs { C2<T>* b[EP_NSLOTS]; };
template <class T>
__global__ void k_materialize(SlotPtrs<T> bufs, T* __restrict__ den, long long N, const DevScalars* __restrict__ sc) {
  T f[EP_NSLOTS];
#pragma unroll
  for (int k = 0; k < EP_NSLOTS; ++k) f[k] = (T)sc->bscale[k];
  const T fd = (T)sc->den_scale;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < EP_NSLOTS; ++k) {
      if (f[k] != T(1)) {
        C2<T> v = bufs.b[k][i];
        v.x *= f[k];
        v.y *= f[k];
        bufs.b[k][i] = v;
      }
    }
    if (fd != T(1)) den[i] *= fd;
  }
}
__global__ void k_reset_scales(DevScalars* sc);

// Sum of partials (fixed order, compensated) -> sc->sums[out0 + q].
// mode 1: corrector epilogue (errHe, norm, mu, renormalisation factor).
// mode 2: norm only (renormalisation factor).
__global__ void k_finalize(const double* __restrict__ partials, int nblocks, int nq, DevScalars* sc, int out0,
                           int mode, double N, double dxyz, double n4, int renorm);

// Impurity field: updatepoten + potenimp P state (potenimp.f90:1-46,184-186,
// 515-632).  Tables are FP64 (0..npot+1).
template <class T>
__global__ void k_potenimp(Geo g, double xmax, double ymax, double zmax, double hx, double hy, double hz,
                           double r0, double r1, double r2, const double* __restrict__ potpi,
                           const double* __restrict__ potdel, int npot, double rmax, double umax_sigma,
                           double2 iv0, double2 iv1, double2 iv2, double2 iv3, double2 iv4, double2 iv5,
                           T* __restrict__ vpi, T* __restrict__ delta, T* __restrict__ uimp);

// D state (potenimp.f90:47-182, 545-566): Delta = V_Delta(r),
// Pi_Del = (V_Pi - V_Delta)(r)/r^4, Sig_Del = (V_Sigma - V_Delta)(r)/r^4 and
// uimp = sum_ij M_ij Re G_ij, M = Delta 1 + Pi_Del d d^T + Sig_Del P(x).
// G holds Re G_ij = Re(conj(iv_2i) iv_2j + conj(iv_2i+1) iv_2j+1) over the
// upper triangle (1,1),(1,2),..,(1,5),(2,2),..,(5,5), off-diagonal doubled.
struct DGram {
  double g[15];
};
template <class T>
__global__ void k_potenimp_d(Geo g, double xmax, double ymax, double zmax, double hx, double hy, double hz,
                             double r0, double r1, double r2, const double* __restrict__ potdel,
                             const double* __restrict__ potpidel, const double* __restrict__ potsigdel, int npot,
                             double rmax, double umax_pi, double umax_sigma, const __grid_constant__ DGram G,
                             T* __restrict__ delta, T* __restrict__ pidel, T* __restrict__ sigdel,
                             T* __restrict__ uimp);

// Energy integrals of energy.f90:47-165 (8 sums, see the launcher).
struct PotDev {
  int kind;
  double r_cutoff, umax, par[4];
  ep_series s;  // EP_POT_SERIES
};
template <class T>
__global__ void k_energy(Geo g, FdW<T> fd, Phys ph, const C2<T>* __restrict__ psi, const T* __restrict__ den,
                         const T* __restrict__ dencg, const T* __restrict__ delj4, const T* __restrict__ falfs,
                         const T* __restrict__ dxd, const T* __restrict__ dyd, const T* __restrict__ dzd,
                         const T* __restrict__ ix, const T* __restrict__ iy, const T* __restrict__ iz,
                         const T* __restrict__ uimp, double xmax, double ymax, double zmax, double hx, double hy,
                         double hz, double r0, double r1, double r2, double zexc, const __grid_constant__ PotDev vplus,
                         int impurity, double* __restrict__ partials);

// forceimp / potinvar moments (potenimp.f90:193-258, 298-317); the F_z sum
// runs over the planes izlo <= iz < izhi (the exciplex filter, :211-248).
template <class T>
__global__ void k_impmoments(Geo g, const T* __restrict__ den, const T* __restrict__ dxd,
                             const T* __restrict__ dyd, const T* __restrict__ dzd, const T* __restrict__ uimp,
                             const T* __restrict__ vpi, const T* __restrict__ delta, double xmax, double ymax,
                             double zmax, double hx, double hy, double hz, double r0, double r1, double r2,
                             int izlo, int izhi, double* __restrict__ partials);

// forceimp sums + the D-state matrix (potenimp.f90:331-405): 3 + 15 sums,
// the matrix's upper triangle in DGram's order.
template <class T>
__global__ void k_impmoments_d(Geo g, const T* __restrict__ den, const T* __restrict__ dxd,
                               const T* __restrict__ dyd, const T* __restrict__ dzd, const T* __restrict__ uimp,
                               const T* __restrict__ delta, const T* __restrict__ pidel,
                               const T* __restrict__ sigdel, double xmax, double ymax, double zmax, double hx,
                               double hy, double hz, double r0, double r1, double r2, int izlo, int izhi,
                               double* __restrict__ partials);

// Form factors on the device (fforma.f90:11-60, initcg.f90:314-331,
// DFT4He3d.f90:396-400), FP64 evaluation, stored in T.
template <class T>
__global__ void k_formfactors(Geo g, const double* __restrict__ px, const double* __restrict__ py,
                              const double* __restrict__ pz, int core, double h4, double eps, double sigma,
                              double bforce, double l, T* __restrict__ fvlj, T* __restrict__ wcgk,
                              T* __restrict__ kalfs);

// Precision conversion of a state array.
template <class B, class A> EP_HD B conv(A a) { return (B)a; }
template <> EP_HD float2 conv<float2, double2>(double2 a) { return make_float2((float)a.x, (float)a.y); }
template <> EP_HD double2 conv<double2, float2>(float2 a) { return make_double2(a.x, a.y); }
template <> EP_HD double2 conv<double2, double2>(double2 a) { return a; }
template <> EP_HD float2 conv<float2, float2>(float2 a) { return a; }
template <> EP_HD dfloat2 conv<dfloat2, double2>(double2 a) { return dfloat2{dfloat(a.x), dfloat(a.y)}; }
template <> EP_HD double2 conv<double2, dfloat2>(dfloat2 a) { return make_double2((double)a.x, (double)a.y); }
template <> EP_HD dfloat2 conv<dfloat2, float2>(float2 a) { return dfloat2{dfloat(a.x), dfloat(a.y)}; }
template <> EP_HD float2 conv<float2, dfloat2>(dfloat2 a) { return make_float2((float)a.x, (float)a.y); }
template <> EP_HD dfloat2 conv<dfloat2, dfloat2>(dfloat2 a) { return a; }
template <class A, class B>
__global__ void k_convert(const A* __restrict__ in, B* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = conv<B, A>(in[i]);
}
