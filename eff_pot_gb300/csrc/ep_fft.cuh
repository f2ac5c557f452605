// ep_fft.cuh - shared-memory FFT engine for batched 3-D real transforms.
//
// A 3-D r2c transform of an (nx,ny,nz) column-major array is three passes:
//  X: each x-line (contiguous) is packed as nx/2 complex numbers, transformed
//     with a half-length complex FFT and unpacked to nx/2+1 outputs;
//  Y, Z: complex transforms of strided lines of the half spectrum.
// A CTA stages a group of lines in shared memory (coalesced global access:
// consecutive threads touch consecutive addresses), runs a self-sorting
// (Stockham) mixed-radix FFT over them with butterflies of radix 8/4/2/3/5,
// and writes them back.  The convolution kernels fuse the point-wise k-space
// multiply between the forward and inverse Z transforms, and the X kernels
// fuse the real-space arithmetic of poten/term_alfa around the transforms.
//
// Conventions match the reference's FFTW use (fft.f90:233-371): forward is
// unnormalised with exp(-2 pi i k n / N); backward uses exp(+...) and the
// caller applies 1/N.
#pragma once
#include "ep_common.cuh"

namespace epfft {

template <class T> struct K;
template <> struct K<double> {
  static constexpr double half = 0.5;
  static constexpr double s3 = 0.86602540378443864676372317075294;   // sin(2pi/3)
  static constexpr double c51 = 0.30901699437494742410229341718282;  // cos(2pi/5)
  static constexpr double c52 = -0.80901699437494742410229341718282; // cos(4pi/5)
  static constexpr double s51 = 0.95105651629515357211643933337938;  // sin(2pi/5)
  static constexpr double s52 = 0.58778525229247312916870595463907;  // sin(4pi/5)
  static constexpr double r2 = 0.70710678118654752440084436210485;   // 1/sqrt(2)
};
template <> struct K<dfloat> {
  static constexpr dfloat half = dfloat(0.5);
  static constexpr dfloat s3 = dfloat(0.86602540378443864676372317075294);
  static constexpr dfloat c51 = dfloat(0.30901699437494742410229341718282);
  static constexpr dfloat c52 = dfloat(-0.80901699437494742410229341718282);
  static constexpr dfloat s51 = dfloat(0.95105651629515357211643933337938);
  static constexpr dfloat s52 = dfloat(0.58778525229247312916870595463907);
  static constexpr dfloat r2 = dfloat(0.70710678118654752440084436210485);
};
template <> struct K<float> {
  static constexpr float half = 0.5f;
  static constexpr float s3 = 0.86602540378443864676372317075294f;
  static constexpr float c51 = 0.30901699437494742410229341718282f;
  static constexpr float c52 = -0.80901699437494742410229341718282f;
  static constexpr float s51 = 0.95105651629515357211643933337938f;
  static constexpr float s52 = 0.58778525229247312916870595463907f;
  static constexpr float r2 = 0.70710678118654752440084436210485f;
};

// w*z with w = DIR*i  (DIR = -1 forward, +1 backward)
template <int DIR, class T2> EP_DEV T2 rot(T2 z) { return DIR < 0 ? mul_mi(z) : mul_i(z); }

template <class T, int DIR> EP_DEV void dft2(C2<T>* v) {
  C2<T> a = v[0], b = v[1];
  v[0] = a + b; v[1] = a - b;
}

template <class T, int DIR> EP_DEV void dft3(C2<T>* v) {
  C2<T> a = v[0], b = v[1], c = v[2];
  C2<T> s = b + c, d = b - c;
  C2<T> t = a - K<T>::half * s;
  C2<T> u = rot<DIR>(K<T>::s3 * d);
  v[0] = a + s; v[1] = t + u; v[2] = t - u;
}

template <class T, int DIR> EP_DEV void dft4(C2<T>* v) {
  C2<T> a = v[0], b = v[1], c = v[2], d = v[3];
  C2<T> s0 = a + c, d0 = a - c, s1 = b + d, d1 = rot<DIR>(b - d);
  v[0] = s0 + s1; v[2] = s0 - s1; v[1] = d0 + d1; v[3] = d0 - d1;
}

template <class T, int DIR> EP_DEV void dft5(C2<T>* v) {
  C2<T> a = v[0];
  C2<T> s1 = v[1] + v[4], d1 = v[1] - v[4], s2 = v[2] + v[3], d2 = v[2] - v[3];
  C2<T> t1 = a + K<T>::c51 * s1 + K<T>::c52 * s2;
  C2<T> t2 = a + K<T>::c52 * s1 + K<T>::c51 * s2;
  C2<T> u1 = rot<DIR>(K<T>::s51 * d1 + K<T>::s52 * d2);
  C2<T> u2 = rot<DIR>(K<T>::s52 * d1 - K<T>::s51 * d2);
  v[0] = a + s1 + s2;
  v[1] = t1 + u1; v[4] = t1 - u1;
  v[2] = t2 + u2; v[3] = t2 - u2;
}

template <class T, int DIR> EP_DEV void dft8(C2<T>* v) {
  C2<T> e[4] = {v[0], v[2], v[4], v[6]};
  C2<T> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T, DIR>(e);
  dft4<T, DIR>(o);
  // o[k] *= w8^k, w8 = (1 + DIR i)/sqrt(2)
  {
    C2<T> z = o[1];
    C2<T> r = cmk<T>(z.x - DIR * z.y, z.y + DIR * z.x);
    o[1] = K<T>::r2 * r;
  }
  o[2] = rot<DIR>(o[2]);
  {
    C2<T> z = o[3];
    C2<T> r = cmk<T>(-z.x - DIR * z.y, -z.y + DIR * z.x);
    o[3] = K<T>::r2 * r;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) { v[k] = e[k] + o[k]; v[k + 4] = e[k] - o[k]; }
}

template <class T, int R, int DIR> EP_DEV void dftR(C2<T>* v) {
  if (R == 2) dft2<T, DIR>(v);
  else if (R == 3) dft3<T, DIR>(v);
  else if (R == 4) dft4<T, DIR>(v);
  else if (R == 5) dft5<T, DIR>(v);
  else dft8<T, DIR>(v);
}

template <class T> struct K16;
template <> struct K16<double> {
  static constexpr double c = 0.92387953251128675612818318939678829;  // cos(pi/8)
  static constexpr double s = 0.38268343236508977172845998403039887;  // sin(pi/8)
  static constexpr double r = 0.70710678118654752440084436210484904;  // 1/sqrt(2)
};
template <> struct K16<dfloat> {
  static constexpr dfloat c = dfloat(0.92387953251128675612818318939678829);
  static constexpr dfloat s = dfloat(0.38268343236508977172845998403039887);
  static constexpr dfloat r = dfloat(0.70710678118654752440084436210484904);
};
template <> struct K16<float> {
  static constexpr float c = 0.92387953251128675612818318939678829f;
  static constexpr float s = 0.38268343236508977172845998403039887f;
  static constexpr float r = 0.70710678118654752440084436210484904f;
};

// z * (a + DIR b i)
template <class T, int DIR> EP_DEV C2<T> rotc(C2<T> z, T a, T b) {
  const T bb = DIR < 0 ? -b : b;
  return cmk<T>(z.x * a - z.y * bb, z.x * bb + z.y * a);
}

// 16-point DFT as 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2.
template <class T, int DIR> EP_DEV void dft16(C2<T>* v) {
  C2<T> y[16];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    C2<T> a[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
    dft4<T, DIR>(a);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) y[4 * n2 + k1] = a[k1];
  }
  // w16^(n2 k1) for n2, k1 in 1..3: exponents 1 2 3 / 2 4 6 / 3 6 9
  const T c = K16<T>::c, s = K16<T>::s, r = K16<T>::r;
  y[5] = rotc<T, DIR>(y[5], c, s);
  y[6] = rotc<T, DIR>(y[6], r, r);
  y[7] = rotc<T, DIR>(y[7], s, c);
  y[9] = rotc<T, DIR>(y[9], r, r);
  y[10] = rot<DIR>(y[10]);
  y[11] = rotc<T, DIR>(y[11], -r, r);
  y[13] = rotc<T, DIR>(y[13], s, c);
  y[14] = rotc<T, DIR>(y[14], -r, r);
  y[15] = rotc<T, DIR>(y[15], -c, -s);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    C2<T> b[4] = {y[k1], y[4 + k1], y[8 + k1], y[12 + k1]};
    dft4<T, DIR>(b);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = b[k2];
  }
}

// cos(2 pi m / n) (c = 0) and sin(2 pi m / n) (c = 1) as compile-time
// constants: the angle is reduced by its quadrant to q pi/2 + phi with
// phi in [0, pi/2), phi above pi/4 is taken as the complement, and the
// Taylor series of sin and cos are summed at |x| <= pi/4 (terms to x^29,
// far below double rounding there).
namespace ctw {
constexpr double kPi = 3.14159265358979323846264338327950288;
__host__ __device__ constexpr double sin_t(double x) {
  double t = x, s = x;
  for (int i = 1; i < 15; ++i) {
    t *= -x * x / ((2.0 * i) * (2.0 * i + 1.0));
    s += t;
  }
  return s;
}
__host__ __device__ constexpr double cos_t(double x) {
  double t = 1.0, s = 1.0;
  for (int i = 1; i < 15; ++i) {
    t *= -x * x / ((2.0 * i - 1.0) * (2.0 * i));
    s += t;
  }
  return s;
}
__host__ __device__ constexpr double cs2pi(int m, int n, int c) {
  const int mm = ((m % n) + n) % n;
  const int q = (4 * mm) / n, r = 4 * mm - q * n;  // angle = q pi/2 + (pi/2) r/n
  double co = 0.0, si = 0.0;
  if (2 * r <= n) {
    const double x = 0.5 * kPi * r / n;
    co = cos_t(x);
    si = sin_t(x);
  } else {
    const double x = 0.5 * kPi * (n - r) / n;
    co = sin_t(x);
    si = cos_t(x);
  }
  const double C[4] = {co, -si, -co, si}, S[4] = {si, co, -si, -co};
  return c == 0 ? C[q] : S[q];
}
}  // namespace ctw

// y[I] *= w_N^(DIR (I / A)(I % A)) for I = I0 .. N-1, w_N = exp(2 pi i / N):
// the inner twiddles of dft_ab, as constants (multiples of pi/2 as swaps)
template <class T, int N, int A, int DIR, int I>
EP_DEV void tw_ab(C2<T>* y) {
  if constexpr (I < N) {
    constexpr int e = (I / A) * (I % A) % N;
    if constexpr (e != 0) {
      if constexpr ((4 * e) % N == 0) {
        constexpr int q = 4 * e / N;
        if constexpr (q == 1) y[I] = rot<DIR>(y[I]);
        else if constexpr (q == 2) y[I] = cmk<T>(-y[I].x, -y[I].y);
        else y[I] = rot<-DIR>(y[I]);
      } else {
        constexpr double c = ctw::cs2pi(e, N, 0), s = ctw::cs2pi(e, N, 1);
        y[I] = rotc<T, DIR>(y[I], T(c), T(s));
      }
    }
    tw_ab<T, N, A, DIR, I + 1>(y);
  }
}

// N = A B point DFT (A, B in {2, 3, 4, 5, 8}) in registers:
//   n = B n1 + n2, k = k1 + A k2,
//   X[k1 + A k2] = sum_n2 w_B^(n2 k2) w_N^(n2 k1) sum_n1 x[B n1 + n2] w_A^(n1 k1)
template <class T, int A, int B, int DIR> EP_DEV void dft_ab(C2<T>* v) {
  constexpr int N = A * B;
  C2<T> y[N];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    C2<T> a[A];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) a[n1] = v[B * n1 + n2];
    dftR<T, A, DIR>(a);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) y[A * n2 + k1] = a[k1];
  }
  tw_ab<T, N, A, DIR, 0>(y);
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) {
    C2<T> b[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) b[n2] = y[A * n2 + k1];
    dftR<T, B, DIR>(b);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = b[k2];
  }
}

// Register DFT of R points, R in {2, 4, 8, 12, 16, 20, 24}.
template <class T, int R, int DIR> EP_DEV void dft(C2<T>* v) {
  if constexpr (R == 16) dft16<T, DIR>(v);
  else if constexpr (R == 8) dft8<T, DIR>(v);
  else if constexpr (R == 4) dft4<T, DIR>(v);
  else if constexpr (R == 12) dft_ab<T, 4, 3, DIR>(v);
  else if constexpr (R == 20) dft_ab<T, 4, 5, DIR>(v);
  else if constexpr (R == 24) dft_ab<T, 8, 3, DIR>(v);
  else {
    static_assert(R == 2, "register DFT length");
    dft2<T, DIR>(v);
  }
}

// q = a / d, r = a - q d for 0 <= a < 2^22 through a float reciprocal
// (one correction step makes it exact); far cheaper than integer division.
EP_DEV int fdivmod(int a, int d, float inv_d, int& r) {
  int q = __float2int_rz(__fmul_rz((float)a, inv_d));
  r = a - q * d;
  if (r >= d) { ++q; r -= d; }
  if (r < 0) { --q; r += d; }
  return q;
}

// One Stockham stage of radix R over nl lines (line stride ld) of length n.
// tw: roots exp(-2 pi i k / (n*tws)), accessed with stride tws.
template <class T, int R, int DIR>
EP_DEV void stage(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst, int nl, int n, int ld,
                  int Ns, const C2<T>* __restrict__ tw, int tws) {
  const int m = n / R;
  const int total = nl * m;
  const int tstep = (n / (Ns * R)) * tws;
  const float inv_nl = 1.0f / (float)nl, inv_ns = 1.0f / (float)Ns;
  // consecutive threads take the same butterfly of consecutive lines: the
  // line stride ld is odd, so every access of a warp hits distinct banks
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    int line, k;
    const int j = fdivmod(b, nl, inv_nl, line);
    fdivmod(j, Ns, inv_ns, k);
    const C2<T>* s = src + line * ld;
    C2<T>* d = dst + line * ld;
    C2<T> v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = s[j + t * m];
    if (k != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) {
        C2<T> w = tw[t * k * tstep];
        v[t] = DIR < 0 ? cmul(v[t], w) : cmulc(v[t], w);
      }
    }
    dftR<T, R, DIR>(v);
    const int idxD = (j - k) * R + k;
#pragma unroll
    for (int u = 0; u < R; ++u) d[idxD + u * Ns] = v[u];
  }
}

// Full FFT over nl lines held in a (ping) with b as scratch; returns the
// buffer that holds the result.  Caller synchronises before the call; the
// result is visible to all threads on return.
template <class T, int DIR>
EP_DEV C2<T>* lines(C2<T>* a, C2<T>* b, int nl, int ld, const FftPlan& p,
                    const C2<T>* __restrict__ tw, int tws) {
  int Ns = 1;
  for (int s = 0; s < p.nst; ++s) {
    const int R = p.rad[s];
    switch (R) {
      case 8: stage<T, 8, DIR>(a, b, nl, p.n, ld, Ns, tw, tws); break;
      case 4: stage<T, 4, DIR>(a, b, nl, p.n, ld, Ns, tw, tws); break;
      case 2: stage<T, 2, DIR>(a, b, nl, p.n, ld, Ns, tw, tws); break;
      case 3: stage<T, 3, DIR>(a, b, nl, p.n, ld, Ns, tw, tws); break;
      default: stage<T, 5, DIR>(a, b, nl, p.n, ld, Ns, tw, tws); break;
    }
    __syncthreads();
    C2<T>* t = a; a = b; b = t;
    Ns *= R;
  }
  return a;
}

// r2c unpack: Z (n2 = nx/2 complex per line, the FFT of the packed line)
// -> X[k], k = 0..n2, written through the functor out(line, k, X).
// twx: exp(-2 pi i k / nx), k = 0..nx-1.
template <class T, class Out>
EP_DEV void r2c_unpack(const C2<T>* Z, int nl, int ld, int n2, const C2<T>* __restrict__ twx, Out out) {
  const int per = n2 + 1;
  const float inv = 1.0f / (float)per;
  for (int b = threadIdx.x; b < nl * per; b += blockDim.x) {
    int k;
    const int line = fdivmod(b, per, inv, k);
    const C2<T>* z = Z + line * ld;
    const C2<T> zk = z[k == n2 ? 0 : k];
    const C2<T> zc = conjg(z[k == 0 ? 0 : n2 - k]);
    const C2<T> e = K<T>::half * (zk + zc);
    const C2<T> o = K<T>::half * mul_mi(zk - zc);
    out(line, k, e + cmul(twx[k], o));
  }
}

// c2r pack: X[k] (k = 0..n2, line stride ldx) -> Z[k] = A + iB, k < n2,
// A = X[k] + conj(X[n2-k]), B = (X[k] - conj(X[n2-k])) * exp(+2 pi i k/nx).
template <class T>
EP_DEV void c2r_pack(const C2<T>* X, int ldx, C2<T>* Z, int ldz, int nl, int n2,
                     const C2<T>* __restrict__ twx) {
  const float inv = 1.0f / (float)n2;
  for (int b = threadIdx.x; b < nl * n2; b += blockDim.x) {
    int k;
    const int line = fdivmod(b, n2, inv, k);
    const C2<T> xk = X[line * ldx + k];
    const C2<T> xc = conjg(X[line * ldx + n2 - k]);
    const C2<T> A = xk + xc;
    const C2<T> B = cmulc(xk - xc, twx[k]);
    Z[line * ldz + k] = A + mul_i(B);
  }
}

}  // namespace epfft
