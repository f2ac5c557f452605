// oracle.cpp - CPU FP64 restatement of the reference hot path.
//
// TEST INFRASTRUCTURE ONLY: the parity checker of the CUDA library and the
// timed CPU baseline ("port") of bench.py.  The product never links it.
//
// Each routine cites the reference routine it restates (paths relative to
// the reference project root).  Arrays are column-major (x fastest) as in
// the Fortran modules; complex arrays are std::complex<double>.
//
// Departures from the reference, all deliberate and shared with the CUDA
// library (the two implement the same definitions):
//  * The FFT is this file's own FP64 mixed-radix transform (the reference
//    calls FFTW through MKL, fft.f90:233-371): unnormalised forward r2c,
//    backward c2r scaled by 1/N, half spectrum along x.
//  * Sums use compensated (Neumaier) accumulation.
//  * eHeX / uplus are zeroed before accumulation (energy.f90:146-165 never
//    zeroes them).
//  * The impurity term of the H-apply is -uimp*psi in imaginary time and
//    -i*uimp*psi in real time (steppc.f90:53 hard-wires the latter).
//  * STOP -> status codes.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

namespace {

const double kPi = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// Compensated summation (per thread, combined in a fixed order).
struct Neu {
  double s = 0.0, c = 0.0;
  void add(double v) {
    double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) c += (s - t) + v; else c += (v - t) + s;
    s = t;
  }
  double get() const { return s + c; }
};

template <class F>
double par_sum(size_t n, F f) {
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  std::vector<Neu> acc(nt);
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    Neu a;
#pragma omp for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) a.add(f((size_t)i));
    acc[t] = a;
  }
  Neu tot;
  for (auto& a : acc) { tot.add(a.s); tot.add(a.c); }
  return tot.get();
}

// ---------------------------------------------------------------------------
// 1-D complex FFT: iterative self-sorting (Stockham) mixed radix 4,2,3,5.
// Roots of unity are rounded once from long double.
struct Plan1D {
  int n = 0;
  std::vector<int> rad;
  std::vector<cd> w;  // exp(-2 pi i k / n)
};

static bool factor235(int n, std::vector<int>& rad) {
  rad.clear();
  int m = n;
  while (m % 4 == 0) { rad.push_back(4); m /= 4; }
  while (m % 2 == 0) { rad.push_back(2); m /= 2; }
  while (m % 3 == 0) { rad.push_back(3); m /= 3; }
  while (m % 5 == 0) { rad.push_back(5); m /= 5; }
  return m == 1;
}

static Plan1D make_plan(int n) {
  Plan1D p;
  p.n = n;
  factor235(n, p.rad);
  p.w.resize(n);
  for (int k = 0; k < n; ++k) {
    long double a = -2.0L * 3.141592653589793238462643383279502884L * k / n;
    p.w[k] = cd((double)cosl(a), (double)sinl(a));
  }
  return p;
}

// sign = -1 forward, +1 backward (unnormalised).  work has n entries.
static void fft1d(const Plan1D& p, cd* a, cd* work, int sign) {
  const int n = p.n;
  if (n == 1) return;
  cd* x = a;
  cd* y = work;
  int Ns = 1;
  auto W = [&](long long e) {
    cd v = p.w[(size_t)(e % n)];
    return sign < 0 ? v : std::conj(v);
  };
  for (int r : p.rad) {
    const int m = n / r;
    for (int j = 0; j < m; ++j) {
      const int k = j % Ns;
      cd v[5];
      for (int t = 0; t < r; ++t) {
        cd tw = W((long long)t * k * (n / (Ns * r)));
        v[t] = x[j + t * m] * tw;
      }
      const int idxD = (j / Ns) * Ns * r + k;
      for (int u = 0; u < r; ++u) {
        cd s = v[0];
        for (int t = 1; t < r; ++t) s += v[t] * W((long long)((t * u) % r) * (n / r));
        y[idxD + u * Ns] = s;
      }
    }
    std::swap(x, y);
    Ns *= r;
  }
  if (x != a) std::copy(x, x + n, a);
}

// 3-D real-to-complex, unnormalised.  out: (nx/2+1, ny, nz).
static void rfft3(int nx, int ny, int nz, const double* in, cd* out) {
  const int nxh = nx / 2 + 1;
  Plan1D px = make_plan(nx), py = make_plan(ny), pz = make_plan(nz);
#pragma omp parallel
  {
    std::vector<cd> b(std::max(nx, std::max(ny, nz))), w(b.size());
#pragma omp for schedule(static)
    for (long long l = 0; l < (long long)ny * nz; ++l) {
      const double* src = in + (size_t)l * nx;
      for (int i = 0; i < nx; ++i) b[i] = cd(src[i], 0.0);
      fft1d(px, b.data(), w.data(), -1);
      cd* dst = out + (size_t)l * nxh;
      for (int i = 0; i < nxh; ++i) dst[i] = b[i];
    }
#pragma omp for schedule(static)
    for (long long l = 0; l < (long long)nxh * nz; ++l) {
      const int ix = (int)(l % nxh), iz = (int)(l / nxh);
      cd* base = out + ix + (size_t)nxh * ny * iz;
      for (int j = 0; j < ny; ++j) b[j] = base[(size_t)j * nxh];
      fft1d(py, b.data(), w.data(), -1);
      for (int j = 0; j < ny; ++j) base[(size_t)j * nxh] = b[j];
    }
#pragma omp for schedule(static)
    for (long long l = 0; l < (long long)nxh * ny; ++l) {
      cd* base = out + l;
      const size_t st = (size_t)nxh * ny;
      for (int k = 0; k < nz; ++k) b[k] = base[k * st];
      fft1d(pz, b.data(), w.data(), -1);
      for (int k = 0; k < nz; ++k) base[k * st] = b[k];
    }
  }
}

// 3-D complex-to-real, unnormalised (the caller scales by 1/N as the
// reference's fftbk_* wrappers do, fft.f90:321-371).  Imaginary parts of the
// x = 0 and x = nx/2 planes are ignored, as FFTW's c2r does.
static void irfft3(int nx, int ny, int nz, const cd* in, double* out) {
  const int nxh = nx / 2 + 1;
  std::vector<cd> t(in, in + (size_t)nxh * ny * nz);
  Plan1D px = make_plan(nx), py = make_plan(ny), pz = make_plan(nz);
#pragma omp parallel
  {
    std::vector<cd> b(std::max(nx, std::max(ny, nz))), w(b.size());
#pragma omp for schedule(static)
    for (long long l = 0; l < (long long)nxh * ny; ++l) {
      cd* base = t.data() + l;
      const size_t st = (size_t)nxh * ny;
      for (int k = 0; k < nz; ++k) b[k] = base[k * st];
      fft1d(pz, b.data(), w.data(), +1);
      for (int k = 0; k < nz; ++k) base[k * st] = b[k];
    }
#pragma omp for schedule(static)
    for (long long l = 0; l < (long long)nxh * nz; ++l) {
      const int ix = (int)(l % nxh), iz = (int)(l / nxh);
      cd* base = t.data() + ix + (size_t)nxh * ny * iz;
      for (int j = 0; j < ny; ++j) b[j] = base[(size_t)j * nxh];
      fft1d(py, b.data(), w.data(), +1);
      for (int j = 0; j < ny; ++j) base[(size_t)j * nxh] = b[j];
    }
#pragma omp for schedule(static)
    for (long long l = 0; l < (long long)ny * nz; ++l) {
      const cd* src = t.data() + (size_t)l * nxh;
      for (int i = 0; i < nxh; ++i) b[i] = src[i];
      for (int i = nxh; i < nx; ++i) b[i] = std::conj(src[nx - i]);
      fft1d(px, b.data(), w.data(), +1);
      double* dst = out + (size_t)l * nx;
      for (int i = 0; i < nx; ++i) dst[i] = b[i].real();
    }
  }
}

// ---------------------------------------------------------------------------
// Central-row finite-difference weights of an M = 2R+1 point stencil, the
// rows NEWDER(ICON=1) unpacks from the Bickley table (newder.f:95-127,
// mates.f BLKDS).  Closed forms from Lagrange interpolation:
//   d/dx  : w_k = (-1)^(k+1) (R!)^2 / (k (R-k)! (R+k)!),  w_-k = -w_k
//   d2/dx2: w_k = 2 (-1)^(k+1) (R!)^2 / (k^2 (R-k)! (R+k)!),
//           w_0 = -2 sum_k 1/k^2
static void fd_central(int npd, int id, double* w) {
  const int R = npd / 2;
  long double lf[64];
  lf[0] = 0.0L;
  for (int i = 1; i < 64; ++i) lf[i] = lf[i - 1] + logl((long double)i);
  for (int j = 0; j < npd; ++j) w[j] = 0.0;
  long double w0 = 0.0L;
  for (int k = 1; k <= R; ++k) {
    long double mag = expl(2.0L * lf[R] - lf[R - k] - lf[R + k]);
    long double sgn = (k % 2 == 1) ? 1.0L : -1.0L;
    if (id == 1) {
      long double v = sgn * mag / k;
      w[R + k] = (double)v;
      w[R - k] = (double)(-v);
    } else {
      long double v = 2.0L * sgn * mag / ((long double)k * k);
      w[R + k] = (double)v;
      w[R - k] = (double)v;
      w0 -= 2.0L / ((long double)k * k);
    }
  }
  if (id == 2) w[R] = (double)w0;
}

// ---------------------------------------------------------------------------
// Si(x): power series for |x| <= 4, else the continued fraction of E1(ix)
// evaluated by the modified Lentz method (Numerical Recipes 6.9).  The
// reference uses NAG's Chebyshev expansions (s13adf.f90); both are accurate
// to a few ulp.
static double sinint_si(double x) {
  const double ax = std::fabs(x);
  double r;
  if (ax <= 4.0) {
    double term = ax, sum = ax;
    const double x2 = ax * ax;
    for (int k = 1; k < 60; ++k) {
      term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
      double t = term / (2.0 * k + 1.0);
      sum += t;
      if (std::fabs(t) < 1e-19 * std::fabs(sum)) break;
    }
    r = sum;
  } else {
    std::complex<long double> b(1.0L, (long double)ax), c(1e300L, 0.0L);
    std::complex<long double> d = 1.0L / b, h = d;
    for (int i = 2; i < 10000; ++i) {
      long double a = -(long double)(i - 1) * (i - 1);
      b += 2.0L;
      d = 1.0L / (a * d + b);
      c = b + a / c;
      std::complex<long double> del = c * d;
      h *= del;
      if (std::abs(del - 1.0L) < 1e-19L) break;
    }
    h *= std::complex<long double>(cosl(ax), -sinl(ax));
    r = (double)(1.5707963267948966192313216916397514L + h.imag());
  }
  return x < 0 ? -r : r;
}

// fforma.f90:143-196: integral of sin(a t)/t from x to infinity.
static double fsinint(double a, double x) {
  const double halfpi = kPi * 0.5;
  double res = sinint_si(a * x);
  return a > 0.0 ? halfpi - res : halfpi + res;
}

// fforma.f90:73-102: integral of sin(a t)/t^11 from x to infinity.
static double sinx11(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double b[5] = {40320.0, -720.0, 24.0, -2.0, 1.0};
  const double c[5] = {362880.0, -5040.0, 120.0, -6.0, 1.0};
  const double d[5] = {1.0, y2, y2 * y2, y2 * y2 * y2, y2 * y2 * y2 * y2};
  double bd = 0.0, cdd = 0.0;
  for (int i = 0; i < 5; ++i) bd += b[i] * d[i];
  for (int i = 0; i < 5; ++i) cdd += c[i] * d[i];
  const double x9 = std::pow(x, 9);
  const double res1 = (a * bd * std::cos(y) + cdd * std::sin(y) / x) / (3628800.0 * x9);
  const double res2 = -(std::pow(a, 10) * fsinint(a, x)) / 3628800.0;
  return res1 + res2;
}

// fforma.f90:108-137: integral of sin(a t)/t^5 from x to infinity.
static double sinx5(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double bd = -2.0 * 1.0 + 1.0 * y2;
  const double cdd = -6.0 * 1.0 + 1.0 * y2;
  const double res1 = -(a * bd * std::cos(y) + cdd * std::sin(y) / x) / (24.0 * x * x * x);
  const double res2 = (std::pow(a, 4) * fsinint(a, x)) / 24.0;
  return res1 + res2;
}

// fforma.f90:221-245: Orsay-Paris core integral.
static double intcore(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double b[3] = {-120.0, 20.0, -1.0}, c[3] = {120.0, -60.0, 5.0};
  double d[3], e[3];
  d[0] = x / std::pow(a, 5); e[0] = 1.0 / std::pow(a, 6);
  d[1] = d[0] * y2; e[1] = e[0] * y2;
  d[2] = d[1] * y2; e[2] = e[1] * y2;
  double bd = 0, ce = 0;
  for (int i = 0; i < 3; ++i) bd += b[i] * d[i];
  for (int i = 0; i < 3; ++i) ce += c[i] * e[i];
  return bd * std::cos(y) + ce * std::sin(y);
}

// fforma.f90:256-280: the p = 0 value (volume integral of the LJ potential).
static double bforce_(int core, double eps, double sigma, double hc) {
  const double pi4 = 4.0 * kPi, eps4 = 4.0 * eps;
  const double xx = std::pow(sigma / hc, 6);
  const double v0 = xx * (xx - 1.0) / std::pow(hc, 4);
  const double s6 = std::pow(sigma, 6), s12 = s6 * s6;
  const double bb2 = pi4 * eps4 * s12 / (9.0 * std::pow(hc, 9));
  const double bb3 = -pi4 * eps4 * s6 / (3.0 * std::pow(hc, 3));
  if (core == EP_CORE_OP) return pi4 * eps4 * (v0 * std::pow(hc, 7)) / 7.0 + bb2 + bb3;
  return bb2 + bb3;
}

// Pair potentials: Select_Pot subset (V_impur.f90:87-932) + Morse.
// V_Koutselos_{Na,K,Rb,Cs}_plus_gs (V_impur.f90:1704-1883), xx in A, result in K.
static double v_koutselos(int ion, double xx) {
  struct Ion { double v_0, rho, R_m, C4, C6, C8; };
  static const Ion ions[4] = {{0.2063, 0.7640, 4.55, 0.0, 1.424, 13.17},   // Na+ :1771-1772
                              {0.2690, 0.8589, 5.49, 0.0, 5.83, 72.05},    // K+  :1861-1862
                              {0.3474, 0.8868, 5.85, 0.0, 8.8, 126.2},     // Rb+ :1817-1818
                              {0.5092, 0.9241, 6.38, 0.0, 13.69, 236.4}};  // Cs+ :1727-1728
  const Ion& p = ions[std::min(std::max(ion, 0), 3)];
  const double a_bohr = 0.529177, Hartree = 27.2114, eV_K = 11604.448;
  const double A = 146.98, a_a = 1.5024, B = 70.198, b_b = 1.4041;
  const double a_d = 1.3831, a_q = 2.4434, a_o = 10.614;
  const double CC4 = p.C4 + a_d / 2.0, CC6 = p.C6 + a_q / 2.0, CC8 = p.C8 + a_o / 2.0;
  const double x = xx / a_bohr;
  const double Rs = x / p.rho;
  const double V_ex = p.v_0 * (A * std::exp(-a_a * Rs) - B * std::exp(-b_b * Rs));
  const double Aux = p.R_m * 1.28;
  double h_r;
  if (x >= Aux) {
    h_r = 1.0;
  } else {
    h_r = 0.0;
    if (x != 0.0) h_r = std::exp(-std::pow(Aux / x - 1.0, 2));
  }
  double Sto = V_ex;
  if (x != 0.0) {
    const double x2 = x * x, x4 = x2 * x2, x6 = x4 * x2, x8 = x6 * x2;
    Sto = Sto + (-CC4 / x4 - CC6 / x6 - CC8 / x8) * h_r;
  }
  return Sto * Hartree * eV_K;
}

// V_alka (V_impur.f90:1097-1192): Patil's alkali-He potential; atom 0..4 =
// LI, NA, K, RB, CS (the order of celem).
static double v_alka(int atom, double dist) {
  static const double av[5] = {1.588, 1.627, 1.771, 1.805, 1.869};          // :1127
  static const double c6v[5] = {22.5, 24.7, 38.9, 44.6, 51.2};              // :1129
  static const double c8v[5] = {1.06e3, 1.29e3, 2.66e3, 3.18e3, 4.34e3};    // :1130
  static const double agranv[5] = {0.0519, 0.0450, 0.0259, 0.0226, 0.0173};  // :1134
  const int ie = std::min(std::max(atom, 0), 4);
  const double evk = 11604.448, bohr = 0.529177249, hartree = 27.211608, factor = evk * hartree;
  const double a = av[ie], b = 0.744, c6 = c6v[ie], c8 = c8v[ie], agran = agranv[ie];
  const double r2 = 2.37, r4 = 7.78, r6 = 50.5;
  const double d = dist / bohr;
  const double pi = 4.0 * std::atan(1.0);
  const double abar = (a + b) / 4.0, u = a - 1.0, v = -0.5 * std::pow(a, 2) * u;
  const double roa = agran * std::pow(d, 2.0 * u) * std::pow(1.0 + v / d, 2) * std::exp(-2.0 * d / a);
  double f[2];
  for (int l = 1; l <= 2; ++l) {
    double sum = 0.0;
    const int l7 = 2 * l + 7;
    for (int n = 0; n <= l7; ++n) {
      double fac = 1.0;
      for (int i = 2; i <= n; ++i) fac *= i;
      sum += std::pow(d / abar, n) / fac;
    }
    f[l - 1] = 1.0 - sum * std::exp(-d / abar);
  }
  const double vimp = 4.0 * pi / 3.0 * roa * (r2 + 37.0 / 90.0 * r4 / std::pow(a, 2) + 28.0 / 525.0 * r6 / std::pow(a, 4)) -
                      c6 * f[0] / std::pow(d, 6) - c8 * f[1] / std::pow(d, 8);
  return vimp * factor;
}

// V_Aziz_He (V_impur.f90:970-990).
static double v_aziz_he(double rr) {
  const double Eps = 10.948, A = 1.8443101e5, alpha = 10.43329537, beta = -2.27965105, D = 1.4826;
  const double C6 = 1.36745214, C8 = 0.42123807, C10 = 0.17473318, rm = 2.963;
  double ff = 1.0;
  const double r = rr / rm;
  if (r <= D) ff = std::exp(-std::pow(D / r - 1.0, 2));
  if (r == 0.0) return A * Eps;
  return (A * std::exp(-alpha * r + beta * std::pow(r, 2)) -
          ff * (C6 / std::pow(r, 6) + C8 / std::pow(r, 8) + C10 / std::pow(r, 10))) *
         Eps;
}

// V_Ar_He / V_Xe_He (V_impur.f90:2681-2782), atom 0 = Ar, 1 = Xe.
static double v_tang_toennies(int atom, double r) {
  const double AA = atom ? 74.9002 : 75.8953, BB = atom ? 1.8175 : 2.0589;
  const double C6 = atom ? 21.5674 : 9.7697, C8 = atom ? 430.148 : 152.8468, C10 = atom ? 10610.21 : 3249.728;
  const double rbohr = 0.5292, Hartree_to_K = 27.21 * 11604.0;
  double B[19], C[8], S[19];  // 1-based as the reference
  B[1] = BB;
  for (int i = 2; i <= 18; ++i) B[i] = B[i - 1] * BB / (double)i;
  C[1] = C6;
  C[2] = C8;
  C[3] = C10;
  for (int i = 4; i <= 7; ++i) C[i] = std::pow(C[i - 1] / C[i - 2], 3) * C[i - 3];
  const double rr = r / rbohr;
  const double Stoe = std::exp(-BB * rr);
  double Stor = rr;
  S[1] = B[1] * Stor;
  for (int i = 2; i <= 18; ++i) {
    Stor = Stor * rr;
    S[i] = S[i - 1] + B[i] * Stor;
  }
  double Aux = AA * Stoe;
  const double Sto1 = 1.0 / std::pow(rr, 2);
  Stor = std::pow(Sto1, 3);
  for (int i = 1; i <= 7; ++i) {
    const int kmax = 2 * i + 4;
    Aux = Aux + ((S[kmax] + 1.0) * Stoe - 1.0) * C[i] * Stor;
    Stor = Stor * Sto1;
  }
  return Aux * Hartree_to_K;
}

// V_Ag_gs / V_Ag_Pi / V_Ag_Sig (V_impur.f90:1038-1096); the literals the
// reference writes without exponent letter are default REAL (binary32).
static double v_ag(int which, double r) {
  struct Ag { double A, alpha, beta, D, C6, C8, C10, C12; };
  static const Ag t[3] = {
      {78741.3877f, 0.65299f, 0.36367f, 12.093f, 137042.07, 189386.217, 111358462.0, 1.17670377e10},      // :1040-1047
      {0.7095092e6, 1.9928f, 0.45500f, 4.0562f, 0.21661134e6, 123454.7952f, 0.307155024e6, 0.740464032e-10},  // :1060-1067
      {40005.2f, 0.41529f, 0.14888f, 25.730f, 1.97443e-9, 3.37393e-6, 0.00788363f, 7.52624e12}};          // :1080-1087
  const Ag& p = t[std::min(std::max(which, 0), 2)];
  double ff = 1.0;
  if (r <= p.D) ff = std::exp(-std::pow(p.D / r - 1.0, 2));
  if (r == 0.0) return p.A;
  return p.A * std::exp(-p.alpha * r - p.beta * std::pow(r, 2)) -
         ff * (p.C6 / std::pow(r, 6) + p.C8 / std::pow(r, 8) + p.C10 / std::pow(r, 10) + p.C12 / std::pow(r, 12));
}

// V_Ba_gs (V_impur.f90:1197-1210).
static double v_ba_gs(double x) {
  if (x <= 3.7) return 1297.1;
  return -6.146426949008034e14 / std::pow(x, 18) + 1.6797251118695925e14 / std::pow(x, 16) -
         1.6513058293510484e13 / std::pow(x, 14) + 7.015334514979032e11 / std::pow(x, 12) -
         1.1066880774828484e10 / std::pow(x, 10) + 4.900282758445466e7 / std::pow(x, 8) -
         450294.6878721156 / std::pow(x, 6);
}

// V_CH3I_l with radpot(l, r) (V_impur.f90:3079-3243).
static double v_ch3i(int l, double r) {
  static const double r_cutoff[5] = {3.6, 3.6f, 3.6, 3.6, 3.6f};
  static const double umax[5] = {3.1648655845e3, -5.1115736616e3, 5.5581502684e3, -2.7398540818e3, 2.4025334047e3};
  static const double d[5] = {0.000185445f, -4.51657e-05f, 2.53688e-05f, -6.51825e-06f, 1.5032e-06f};
  static const double b[5] = {0.782913f, 0.837569f, 0.849398f, 0.779254f, 0.787553f};
  static const double c[5] = {9.5243f, 10.3772f, 10.6988f, 11.454f, 12.236f};
  const int k = std::min(std::max(l, 0), 4);
  const double a_bohr = 0.529177, Hartree = 27.2114, eV_K = 11604.448;
  if (r <= r_cutoff[k]) return umax[k];
  const double r_au = r / a_bohr;
  const double radpot = d[k] * std::pow(1.0 - std::exp(-b[k] * (r_au - c[k])), 2) - d[k];
  return radpot * Hartree * eV_K;
}

// The surface and adatom potentials (V_grafeno, V_grafeno_sin_dispersion,
// V_TiO2, V_Au, V_Au_TiO2, V_dAu_TiO2, Ag_Graphene, dz_Ag_Graphene,
// Au_Graphene, dz_Au_Graphene; V_impur.f90:939-965,2417-2554,3013-3030).
static double v_surface(int which, double z) {
  const double C_meV_to_K = 11.604448;
  if (which == 0) {
    const double A = 554811.0, alpha = 3.21193, C4 = 1531.83, C6 = 22259.0;
    return (A * std::exp(-alpha * z) - C4 / std::pow(z, 4) - C6 / std::pow(z, 6)) * C_meV_to_K;
  }
  if (which == 1) {
    const double D = 0.493191, alpha = 1.54605, Ze = 4.34871;
    return (D * std::pow(1.0 - std::exp(-alpha * (z - Ze)), 2) - D) * C_meV_to_K;
  }
  if (which == 2) {
    const double cmm1toK = 1.4387770, de = 95.9583, alpha = 1.47089, ze = 4.22534, z0 = 4.77765, c3 = 8.85163,
                 aa = 1.06161;
    const double vz = de * std::pow(1.0 - std::exp(-alpha * (z - ze)), 2) - de;
    const double vzd = -0.5 * (1.0 + std::tanh((z - z0) / aa) * c3 * std::pow(c3 / z, 3));
    return (vz + vzd) * cmm1toK;
  }
  if (which == 3) {
    const double a[10] = {0.0, 1.6417, -0.6164, 0.3770, -0.0549, 0.0018, 0.0046, -0.0010, 0.0001, 2.7e-6};
    const double Re = 4.124, De = 20.301143, r = z - Re;
    double h = a[9];
    for (int k = 8; k >= 1; --k) h = a[k] + r * h;
    return -De * (1.0 + r * h) * std::exp(-a[1] * r);
  }
  if (which == 4 || which == 5) {
    const double C6 = -4.18518e6, C8 = 6.54459e7, C10 = -3.73112e8, C12 = 9.44942e8, C14 = -8.97265e8;
    if (!(z > 2.0)) return (which == 4 ? 1821.44287109375 : -5415.35400390625) * C_meV_to_K;
    const double Aux = 1.0 / z, Aux2 = std::pow(Aux, 2);
    if (which == 4) return (((((C14 * Aux2 + C12) * Aux2 + C10) * Aux2 + C8) * Aux2 + C6) * std::pow(Aux2, 3)) * C_meV_to_K;
    return (((((-14.0 * C14 * Aux2 - 12.0 * C12) * Aux2 - 10.0 * C10) * Aux2 - 8.0 * C8) * Aux2 - 6.0 * C6) *
            (std::pow(Aux2, 3) * Aux)) *
           C_meV_to_K;
  }
  const bool ag = which == 6 || which == 7, deriv = which == 7 || which == 9;
  const double A = ag ? 11557.3 : 448058.0, beta = ag ? 2.33671 : 2.12336, C4 = ag ? 1143.0 : 83077.3;
  const double unit = ag ? 5.03216592455e2 : C_meV_to_K;
  if (!deriv) return (A * std::exp(-beta * z) - C4 / std::pow(z, 4)) * unit;
  return (-A * beta * std::exp(-beta * z) + 4.0 * C4 / std::pow(z, 5)) * unit;
}

// The inverse-power fits with a parabolic core (e.g. V_Fausto_Rb_gs,
// V_impur.f90:2206-2250: Sto = sum_k Pg(k) Aux, Aux = xq**(k0+1) times xq
// per term, xq = 1/x, all in Real*16).  The Real*16 arithmetic is restated
// as an unevaluated sum of two doubles: hi + lo with |lo| <= ulp(hi)/2.
namespace qd {
struct Q {
  double hi, lo;
};
static Q renorm(double a, double b) {
  const double s = a + b;
  return Q{s, b - (s - a)};
}
static Q plus(Q a, Q b) {
  double s = a.hi + b.hi, v = s - a.hi;
  double e = (a.hi - (s - v)) + (b.hi - v);
  double t = a.lo + b.lo, w = t - a.lo;
  double f = (a.lo - (t - w)) + (b.lo - w);
  Q r = renorm(s, e + t);
  return renorm(r.hi, r.lo + f);
}
static Q times(Q a, Q b) {
  const double p = a.hi * b.hi;
  return renorm(p, std::fma(a.hi, b.hi, -p) + a.hi * b.lo + a.lo * b.hi);
}
static Q inverse(double x) {
  const double q = 1.0 / x;
  return renorm(q, std::fma(-q, x, 1.0) / x);
}
}  // namespace qd

static double v_series(const ep_series& s, double x) {
  if (x <= s.r_core) return s.f_core;
  if (x <= s.r0) return std::fabs(s.aa * std::pow(x, 2) + s.bb * x + s.cc);
  if (!s.quad) {  // Real*8 Pg, Sto, xq (V_LJ_OT, :1021-1036)
    const double xq = 1.0 / x;
    double Sto = 0.0;
    for (int k = 1; k <= s.n; ++k) Sto = Sto + s.c_hi[k - 1] * std::pow(xq, k + s.k0);
    return Sto;
  }
  const qd::Q xq = qd::inverse(x);
  qd::Q Aux{1.0, 0.0};
  for (int i = 0; i < s.k0 + 1; ++i) Aux = qd::times(Aux, xq);
  qd::Q Sto{0.0, 0.0};
  for (int k = 1; k <= s.n; ++k) {
    Sto = qd::plus(Sto, qd::times(qd::Q{s.c_hi[k - 1], s.c_lo[k - 1]}, Aux));
    Aux = qd::times(Aux, xq);
  }
  return Sto.hi + Sto.lo;
}

// Func_Ba_plus_gs (V_impur.f90:1479-1497), behind 'Ba_plus_old_gs'.
static double v_evenpow(const ep_series& s, double x) {
  if (x <= s.r0) return s.aa * std::pow(x, 2) + s.bb * x + s.cc;
  double Sto = 0.0;
  for (int k = 1; k <= s.n; ++k) Sto = Sto + s.c_hi[k - 1] / std::pow(x, 2 * (k - 1) + 6);
  return Sto;
}

// V_Cs_7s (V_impur.f90:1682-1702): Pg in c_hi, Ps in c_lo, x0 in r_core.
static double v_expfit(const ep_series& s, double xx) {
  const double x = xx < s.r_core ? s.r_core : xx;
  if (x <= s.r0) return s.aa * std::pow(x, 2) + s.bb * x + s.cc;
  double Sto = s.c_hi[0] * std::exp(-s.c_lo[0] * x) / x;
  for (int k = 2; k <= s.n; ++k) Sto = Sto + s.c_hi[k - 1] * std::pow(x, k - 1) * std::exp(-s.c_lo[k - 1] * x);
  return Sto;
}

static double select_pot(const ep_potential& p, double r) {
  if (p.kind == EP_POT_NULL) return 0.0;
  if (r < p.r_cutoff) return p.umax;
  if (p.kind == EP_POT_MORSE) {
    const double De = p.par[0], re = p.par[1], al = p.par[2];
    const double e = std::exp(-al * (r - re));
    return De * (e * e - 2.0 * e);
  }
  if (p.kind == EP_POT_KOUTSELOS) return v_koutselos((int)p.par[0], r);
  if (p.kind == EP_POT_PATIL) return v_alka((int)p.par[0], r);
  if (p.kind == EP_POT_AZIZ) return v_aziz_he(r);
  if (p.kind == EP_POT_TANG_TOENNIES) return v_tang_toennies((int)p.par[0], r);
  if (p.kind == EP_POT_SERIES && p.series) return v_series(*p.series, r);
  if (p.kind == EP_POT_AG) return v_ag((int)p.par[0], r);
  if (p.kind == EP_POT_BA_GS) return v_ba_gs(r);
  if (p.kind == EP_POT_CH3I) return v_ch3i((int)p.par[0], r);
  if (p.kind == EP_POT_SURFACE) return v_surface((int)p.par[0], r);
  if (p.kind == EP_POT_EVENPOW && p.series) return v_evenpow(*p.series, r);
  if (p.kind == EP_POT_EXPFIT && p.series) return v_expfit(*p.series, r);
  return 0.0;
}

// The potential and its fit, kept beyond the call that passed them.
struct KeptPot {
  ep_potential p{};
  ep_series s{};
  void keep(const ep_potential& q) {
    p = q;
    p.series = nullptr;
    if ((q.kind == EP_POT_SERIES || q.kind == EP_POT_EVENPOW || q.kind == EP_POT_EXPFIT) && q.series) {
      s = *q.series;
      p.series = &s;
    }
  }
};

// potenimp.f90:588-632 (update): parabolic interpolation in f(0:nint+1).
static double update_interp(double r, int nint, double rmax, const double* f) {
  const double h = rmax / (nint - 1);
  const double c1oh = 1.0 / h;
  const double c1o2h2 = c1oh * c1oh * 0.5;
  const int i0 = (int)(1.5 + r / h);
  const double r0 = (i0 - 1) * h;
  const double f0 = f[i0];
  int i1, i2;
  if (r < r0) { i1 = i0 - 1; i2 = i0 + 1; } else { i1 = i0 + 1; i2 = i0 - 1; }
  const double f1 = f[i1], f2 = f[i2];
  const double aa = (f2 - 2.0 * f0 + f1) * c1o2h2;
  double bb;
  if (r < r0) bb = (f2 - f0) * c1oh - aa * (2.0 * r0 + h);
  else bb = (f1 - f0) * c1oh - aa * (2.0 * r0 + h);
  const double cc = f0 - r0 * (bb + r0 * aa);
  return r * (aa * r + bb) + cc;
}

}  // namespace

// ===========================================================================
struct oc_ctx {
  ep_config cfg;
  int nx, ny, nz, nxh;
  size_t N, Nh;
  double hx, hy, hz, dxyz, renor;
  std::vector<double> x, y, z;
  std::vector<double> fvlj4, wcgk, kalfs;
  double wd1[3][32], wd2[3][32];  // central rows scaled by 1/h^id per axis
  int R;
  // fields (modules rho, field, classicimp, lenard4, alphasterm, deriva)
  std::vector<cd> psi, psiold[3], hpsiold[2], pc, q;
  std::vector<double> den, pot4, uimp, dencg, delj4, dxden, dyden, dzden;
  std::vector<double> denalf, falfs, intx, inty, intz, ualphas, penalty;
  std::vector<double> vpi, delta, sigdel;  // D state: vpi = Pi_Del, delta = V_Delta, sigdel = Sig_Del
  std::vector<cd> fden, wk1, wk2, wk3;
  std::vector<double> sto1, sto2, sto3, sto4, sto5, sto6;
  std::vector<cd> lap;  // sum of the three second derivatives
  int ioldp[3], ioldh[2];
  bool have_field = false;
  // impurity (module classicimp, steppc/steprk variables)
  double rimp[3] = {0, 0, 0}, vimp[3] = {0, 0, 0}, aimp[3] = {0, 0, 0};
  cd invar[10], hinvar[10];
  double qr[3] = {0, 0, 0}, qv[3] = {0, 0, 0};
  double rimpold[3][3] = {}, vimpold[3][3] = {}, aimpold[3][2] = {};
  int ioldr[3], ioldv[3], iolda[2], ioldiv[3], ioldhiv[2];
  double pcr[3] = {0, 0, 0}, pcv[3] = {0, 0, 0};
  cd qiv[10], invarold[10][3], hinvarold[10][2], pciv[10];
  // interpolation tables (module interpol)
  int npot = 0;
  double delinter = 0, umax_sigma = 9.674836e3, umax_pi = 0.0;
  std::vector<double> potpi, potdel;  // D state: potpi = potpidel, potdel = V_Delta
  std::vector<double> potsigdel;      // D state only
  KeptPot plus;
  bool have_tables = false;
  double last_mu = 0, last_norm = 0;
  std::string err;
};

static int fail(oc_ctx* c, int code, const char* msg) {
  if (c) c->err = msg;
  return code;
}

static bool even235(int n) {
  std::vector<int> r;
  return n >= 2 && n % 2 == 0 && factor235(n, r);
}

// Column-major neighbour access helpers.
static inline size_t IDX(const oc_ctx* c, int i, int j, int k) {
  return (size_t)i + (size_t)c->nx * ((size_t)j + (size_t)c->ny * k);
}

// derivnd -> Deriv3D_p / Deriv3D_pc (init_deriv_parallel.f90:368-642,
// 923-1197), central-row form: periodic (icon 8: wrap; the reference splits
// the wrapped sum, :527-639) or zero outside the grid (icon 13: REDEF shifts
// the central row, redef.f:151-169, which equals zero padding).
template <class T>
static void deriv(const oc_ctx* c, int id, int axis, const T* f, T* df) {
  const double* w = (id == 1) ? c->wd1[axis] : c->wd2[axis];
  const int R = c->R;
  const int n = axis == 0 ? c->nx : axis == 1 ? c->ny : c->nz;
  const bool periodic = (c->cfg.icon == EP_ICON_PERIODIC);
  const long long total = (long long)c->N;
  const size_t stride = axis == 0 ? 1 : axis == 1 ? (size_t)c->nx : (size_t)c->nx * c->ny;
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < total; ++p) {
    const int ix = (int)(p % c->nx);
    const int iy = (int)((p / c->nx) % c->ny);
    const int iz = (int)(p / ((long long)c->nx * c->ny));
    const int i = axis == 0 ? ix : axis == 1 ? iy : iz;
    const size_t base = (size_t)p - (size_t)i * stride;
    T s = T(0);
    if (i >= R && i < n - R) {
      for (int j = 0; j < 2 * R + 1; ++j) s += w[j] * f[base + (size_t)(i - R + j) * stride];
    } else if (periodic) {
      T a = T(0), b = T(0);
      for (int j = 0; j < 2 * R + 1; ++j) {
        int ii = i - R + j;
        if (ii < 0) a += w[j] * f[base + (size_t)(ii + n) * stride];
        else if (ii >= n) b += w[j] * f[base + (size_t)(ii - n) * stride];
        else s += w[j] * f[base + (size_t)ii * stride];
      }
      s = (i < R) ? (a + s) : (s + b);
    } else {
      for (int j = 0; j < 2 * R + 1; ++j) {
        int ii = i - R + j;
        if (ii >= 0 && ii < n) s += w[j] * f[base + (size_t)ii * stride];
      }
    }
    df[p] = s;
  }
}

extern "C" {

int oc_potential_values(const ep_potential* p, const double* r, double* v, int n) {
  if (!p || n < 0 || (n > 0 && (!r || !v))) return EP_ERR_INVALID_ARG;
  if ((p->kind == EP_POT_SERIES || p->kind == EP_POT_EVENPOW || p->kind == EP_POT_EXPFIT) &&
      (!p->series || p->series->n < 1 || p->series->n > EP_SERIES_MAX))
    return EP_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i) v[i] = select_pot(*p, r[i]);
  return EP_OK;
}

int oc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int oc_fd_weights(int npd, int id, double* w) {
  if (npd < 3 || npd > 25 || npd % 2 == 0 || (id != 1 && id != 2) || !w) return EP_ERR_INVALID_ARG;
  fd_central(npd, id, w);
  return EP_OK;
}

double oc_sinint(double x) { return sinint_si(x); }
double oc_bforce(int core, double eps, double sigma, double hc) { return bforce_(core, eps, sigma, hc); }

int oc_rfft3(int nx, int ny, int nz, const double* in, double* out_c) {
  if (!even235(nx) || nx < 2 || ny < 1 || nz < 1) return EP_ERR_BAD_GRID;
  std::vector<int> r;
  if (!factor235(ny, r) || !factor235(nz, r)) return EP_ERR_BAD_GRID;
  rfft3(nx, ny, nz, in, reinterpret_cast<cd*>(out_c));
  return EP_OK;
}

int oc_irfft3(int nx, int ny, int nz, const double* in_c, double* out) {
  if (!even235(nx)) return EP_ERR_BAD_GRID;
  std::vector<int> r;
  if (!factor235(ny, r) || !factor235(nz, r)) return EP_ERR_BAD_GRID;
  irfft3(nx, ny, nz, reinterpret_cast<const cd*>(in_c), out);
  return EP_OK;
}

// DFT4He3d.f90:205-300 (grids), :385-400 (form factors), initcg.f90:5-51,
// Init_deriv_p (init_deriv_parallel.f90:51-82), dimen.f90:8-148.
int oc_create(const ep_config* cfg, oc_ctx** out) {
  if (!cfg || !out) return EP_ERR_INVALID_ARG;
  *out = nullptr;
  if (!even235(cfg->nx) || !even235(cfg->ny) || !even235(cfg->nz)) return EP_ERR_BAD_GRID;
  if (cfg->npd < 3 || cfg->npd > 25 || cfg->npd % 2 == 0) return EP_ERR_INVALID_ARG;
  if (cfg->icon != EP_ICON_PERIODIC && cfg->icon != EP_ICON_ZERO_OUTSIDE) return EP_ERR_UNSUPPORTED;
  if (cfg->nx < cfg->npd || cfg->ny < cfg->npd || cfg->nz < cfg->npd) return EP_ERR_BAD_GRID;
  oc_ctx* c = new oc_ctx();
  c->cfg = *cfg;
  const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
  c->nx = nx; c->ny = ny; c->nz = nz; c->nxh = nx / 2 + 1;
  c->N = (size_t)nx * ny * nz;
  c->Nh = (size_t)c->nxh * ny * nz;
  c->hx = 2.0 * std::fabs(cfg->xmax) / nx;
  c->hy = 2.0 * std::fabs(cfg->ymax) / ny;
  c->hz = 2.0 * std::fabs(cfg->zmax) / nz;
  c->dxyz = c->hx * c->hy * c->hz;
  c->renor = 1.0 / ((double)nx * ny * nz);
  c->x.resize(nx); c->y.resize(ny); c->z.resize(nz);
  for (int i = 0; i < nx; ++i) c->x[i] = -cfg->xmax + c->hx * i;
  for (int i = 0; i < ny; ++i) c->y[i] = -cfg->ymax + c->hy * i;
  for (int i = 0; i < nz; ++i) c->z[i] = -cfg->zmax + c->hz * i;
  // FFT-ordered momentum grid (DFT4He3d.f90:213-219,266-300).
  const double hpx = 1.0 / (nx * c->hx), hpy = 1.0 / (ny * c->hy), hpz = 1.0 / (nz * c->hz);
  const double pmaxx = 1.0 / (2.0 * c->hx), pmaxy = 1.0 / (2.0 * c->hy), pmaxz = 1.0 / (2.0 * c->hz);
  std::vector<double> px(nx), py(ny), pz(nz);
  for (int i = 1; i <= nx / 2 + 1; ++i) px[i - 1] = hpx * (i - 1);
  for (int i = nx / 2 + 2; i <= nx; ++i) px[i - 1] = -pmaxx + hpx * (i - (nx / 2 + 1));
  for (int i = 1; i <= ny / 2 + 1; ++i) py[i - 1] = hpy * (i - 1);
  for (int i = ny / 2 + 2; i <= ny; ++i) py[i - 1] = -pmaxy + hpy * (i - (ny / 2 + 1));
  for (int i = 1; i <= nz / 2 + 1; ++i) pz[i - 1] = hpz * (i - 1);
  for (int i = nz / 2 + 2; i <= nz; ++i) pz[i - 1] = -pmaxz + hpz * (i - (nz / 2 + 1));
  c->fvlj4.resize(c->Nh); c->wcgk.resize(c->Nh); c->kalfs.resize(c->Nh);
  const double h4 = (cfg->core == EP_CORE_OP) ? cfg->h4op : cfg->h4ot;
  const double eps = cfg->eps4, sigma = cfg->sigma4;
  const double sigma6 = std::pow(sigma, 6), aux1 = 8.0 * eps, aux3 = sigma6 / std::pow(h4, 6);
  const double bf = bforce_(cfg->core, eps, sigma, h4);
  const double twopi = 2.0 * kPi;
  const int nxh = c->nxh;
#pragma omp parallel for schedule(static)
  for (long long l = 0; l < (long long)c->Nh; ++l) {
    const int ipx = (int)(l % nxh), ipy = (int)((l / nxh) % ny), ipz = (int)(l / ((long long)nxh * ny));
    const double p = std::sqrt(px[ipx] * px[ipx] + py[ipy] * py[ipy] + pz[ipz] * pz[ipz]);
    // fforma.f90:40-60
    double fv;
    if (std::fabs(p) < 1e-10) {
      fv = bf;
    } else {
      const double a2 = twopi * p;
      const double t1 = sinx11(a2, h4), t2 = sinx5(a2, h4);
      if (cfg->core == EP_CORE_OP) {
        const double v0 = aux1 * aux3 * (aux3 - 1.0) / std::pow(h4, 4);
        const double t3 = intcore(a2, h4);
        fv = (aux1 * sigma6 * (sigma6 * t1 - t2) + v0 * t3) / p;
      } else {
        fv = (aux1 * sigma6 * (sigma6 * t1 - t2)) / p;
      }
    }
    c->fvlj4[l] = fv;
    // initcg.f90:314-331
    double wc = 1.0;
    if (p > 0.0) {
      const double arg = twopi * p * h4;
      const double aux = std::sin(arg) - arg * std::cos(arg);
      wc = (std::fabs(aux) < 1e-10) ? 1.0 : 3.0 * aux / (arg * arg * arg);
    }
    c->wcgk[l] = wc;
    // DFT4He3d.f90:396-400
    const double t = kPi * cfg->l * p;
    c->kalfs[l] = std::exp(-(t * t));
  }
  // FD weights (Init_deriv_p + Deriv3D_p scaling Sto = 1/h**id).
  c->R = cfg->npd / 2;
  double w1[32], w2[32];
  fd_central(cfg->npd, 1, w1);
  fd_central(cfg->npd, 2, w2);
  const double hh[3] = {c->hx, c->hy, c->hz};
  for (int a = 0; a < 3; ++a) {
    const double s1 = 1.0 / hh[a], s2 = 1.0 / (hh[a] * hh[a]);
    for (int j = 0; j < cfg->npd; ++j) { c->wd1[a][j] = w1[j] * s1; c->wd2[a][j] = w2[j] * s2; }
  }
  const size_t N = c->N, Nh = c->Nh;
  c->psi.assign(N, cd(0)); c->pc.assign(N, cd(0)); c->q.assign(N, cd(0));
  for (auto& v : c->psiold) v.assign(N, cd(0));
  for (auto& v : c->hpsiold) v.assign(N, cd(0));
  for (auto* v : {&c->den, &c->pot4, &c->uimp, &c->dencg, &c->delj4, &c->dxden, &c->dyden, &c->dzden,
                  &c->denalf, &c->falfs, &c->intx, &c->inty, &c->intz, &c->ualphas, &c->penalty,
                  &c->vpi, &c->delta, &c->sto1, &c->sto2, &c->sto3, &c->sto4, &c->sto5, &c->sto6})
    v->assign(N, 0.0);
  if (cfg->state == EP_STATE_D) c->sigdel.assign(N, 0.0);
  c->lap.assign(N, cd(0));
  c->fden.assign(Nh, cd(0)); c->wk1.assign(Nh, cd(0)); c->wk2.assign(Nh, cd(0)); c->wk3.assign(Nh, cd(0));
  for (int i = 0; i < 3; ++i) { c->ioldp[i] = i; c->ioldr[i] = i; c->ioldv[i] = i; c->ioldiv[i] = i; }
  for (int i = 0; i < 2; ++i) { c->ioldh[i] = i; c->iolda[i] = i; c->ioldhiv[i] = i; }
  for (int i = 0; i < 10; ++i) {
    c->invar[i] = c->hinvar[i] = c->qiv[i] = c->pciv[i] = cd(0);
    for (int j = 0; j < 3; ++j) c->invarold[i][j] = cd(0);
    for (int j = 0; j < 2; ++j) c->hinvarold[i][j] = cd(0);
  }
  c->plus.p.kind = EP_POT_NULL;
  *out = c;
  return EP_OK;
}

int oc_destroy(oc_ctx* c) {
  delete c;
  return EP_OK;
}

const char* oc_last_error(const oc_ctx* c) { return c ? c->err.c_str() : "null context"; }

int oc_form_factors(oc_ctx* c, double* fv, double* wc, double* ka) {
  if (!c) return EP_ERR_INVALID_ARG;
  if (fv) std::copy(c->fvlj4.begin(), c->fvlj4.end(), fv);
  if (wc) std::copy(c->wcgk.begin(), c->wcgk.end(), wc);
  if (ka) std::copy(c->kalfs.begin(), c->kalfs.end(), ka);
  return EP_OK;
}

int oc_deriv(const oc_ctx* c, int id, int axis, int is_complex, const double* f, double* df) {
  if (!c || !f || !df || axis < 0 || axis > 2 || (id != 1 && id != 2)) return EP_ERR_INVALID_ARG;
  if (is_complex) deriv(c, id, axis, reinterpret_cast<const cd*>(f), reinterpret_cast<cd*>(df));
  else deriv(c, id, axis, f, df);
  return EP_OK;
}

// potenimpini.f90:1-72 (P state).
int oc_set_impurity_potentials(oc_ctx* c, const ep_potential* pi, const ep_potential* sigma,
                               const ep_potential* plus) {
  if (!c || !pi || !sigma) return EP_ERR_INVALID_ARG;
  const ep_config& g = c->cfg;
  const int npot = 100 * std::max(g.nx, std::max(g.ny, g.nz)) + 1;
  const double rmax = 4.0 * std::max(g.xmax, std::max(g.ymax, g.zmax));
  const double del = rmax / (double)(npot - 1);
  std::vector<double> tp(npot + 2), td(npot + 2);
  for (int i = 1; i <= npot; ++i) {
    const double r = (double)(i - 1) * del;
    const double a = select_pot(*pi, r);
    tp[i] = a;
    td[i] = select_pot(*sigma, r) - a;
  }
  td[0] = td[1]; td[npot + 1] = td[npot];
  tp[0] = tp[1]; tp[npot + 1] = tp[npot];
  if (plus) c->plus.keep(*plus);
  return oc_set_impurity_tables(c, tp.data(), td.data(), npot, del, sigma->umax);
}

int oc_set_impurity_tables(oc_ctx* c, const double* potpi, const double* potdel, int npot,
                           double delinter, double umax_sigma) {
  if (!c || !potpi || !potdel || npot < 3 || !(delinter > 0)) return EP_ERR_INVALID_ARG;
  if (c->cfg.state != EP_STATE_P) return fail(c, EP_ERR_STATE, "P-state tables need state = EP_STATE_P");
  c->npot = npot;
  c->delinter = delinter;
  c->umax_sigma = umax_sigma;
  c->potpi.assign(potpi, potpi + npot + 2);
  c->potdel.assign(potdel, potdel + npot + 2);
  c->have_tables = true;
  return EP_OK;
}

// potenimpini.f90:28-50, D state: potdel = V_Delta, potpidel = V_Pi - V_Delta,
// potsigdel = V_Sigma - V_Delta, end points repeated.
int oc_set_impurity_potentials_d(oc_ctx* c, const ep_potential* pi, const ep_potential* sigma,
                                 const ep_potential* delta, const ep_potential* plus) {
  if (!c || !pi || !sigma || !delta) return EP_ERR_INVALID_ARG;
  const ep_config& g = c->cfg;
  const int npot = 100 * std::max(g.nx, std::max(g.ny, g.nz)) + 1;
  const double rmax = 4.0 * std::max(g.xmax, std::max(g.ymax, g.zmax));
  const double del = rmax / (double)(npot - 1);
  std::vector<double> td(npot + 2), tpd(npot + 2), tsd(npot + 2);
  for (int i = 1; i <= npot; ++i) {
    const double r = (double)(i - 1) * del;
    const double aux = select_pot(*delta, r);
    td[i] = aux;
    tpd[i] = select_pot(*pi, r) - aux;
    tsd[i] = select_pot(*sigma, r) - aux;
  }
  td[0] = td[1]; td[npot + 1] = td[npot];
  tpd[0] = tpd[1]; tpd[npot + 1] = tpd[npot];
  tsd[0] = tsd[1]; tsd[npot + 1] = tsd[npot];
  if (plus) c->plus.keep(*plus);
  return oc_set_impurity_tables_d(c, td.data(), tpd.data(), tsd.data(), npot, del, pi->umax, sigma->umax);
}

int oc_set_impurity_tables_d(oc_ctx* c, const double* potdel, const double* potpidel, const double* potsigdel,
                             int npot, double delinter, double umax_pi, double umax_sigma) {
  if (!c || !potdel || !potpidel || !potsigdel || npot < 3 || !(delinter > 0)) return EP_ERR_INVALID_ARG;
  if (c->cfg.state != EP_STATE_D) return fail(c, EP_ERR_STATE, "D-state tables need state = EP_STATE_D");
  c->npot = npot;
  c->delinter = delinter;
  c->umax_pi = umax_pi;
  c->umax_sigma = umax_sigma;
  c->potdel.assign(potdel, potdel + npot + 2);
  c->potpi.assign(potpidel, potpidel + npot + 2);
  c->potsigdel.assign(potsigdel, potsigdel + npot + 2);
  c->have_tables = true;
  return EP_OK;
}

int oc_get_impurity_tables(oc_ctx* c, double* potpi, double* potdel, int* npot, double* delinter) {
  if (!c || !c->have_tables) return EP_ERR_STATE;
  if (npot) *npot = c->npot;
  if (delinter) *delinter = c->delinter;
  if (potpi) std::copy(c->potpi.begin(), c->potpi.end(), potpi);
  if (potdel) std::copy(c->potdel.begin(), c->potdel.end(), potdel);
  return EP_OK;
}

int oc_set_impurity_state(oc_ctx* c, const double* rimp, const double* vimp, const double* invar) {
  if (!c) return EP_ERR_INVALID_ARG;
  for (int i = 0; i < 3; ++i) {
    if (rimp) c->rimp[i] = rimp[i];
    if (vimp) c->vimp[i] = vimp[i];
  }
  if (invar)
    for (int i = 0; i < 10; ++i) c->invar[i] = cd(invar[2 * i], invar[2 * i + 1]);
  return EP_OK;
}

int oc_get_impurity_state(oc_ctx* c, double* rimp, double* vimp, double* aimp, double* invar) {
  if (!c) return EP_ERR_INVALID_ARG;
  for (int i = 0; i < 3; ++i) {
    if (rimp) rimp[i] = c->rimp[i];
    if (vimp) vimp[i] = c->vimp[i];
    if (aimp) aimp[i] = c->aimp[i];
  }
  if (invar)
    for (int i = 0; i < 10; ++i) { invar[2 * i] = c->invar[i].real(); invar[2 * i + 1] = c->invar[i].imag(); }
  return EP_OK;
}

int oc_upload_psi(oc_ctx* c, const double* psi) {
  if (!c || !psi) return EP_ERR_INVALID_ARG;
  const cd* p = reinterpret_cast<const cd*>(psi);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)c->N; ++i) {
    c->psi[i] = p[i];
    c->den[i] = std::norm(p[i]);
  }
  return EP_OK;
}

int oc_download_psi(oc_ctx* c, double* psi) {
  if (!c || !psi) return EP_ERR_INVALID_ARG;
  std::copy(c->psi.begin(), c->psi.end(), reinterpret_cast<cd*>(psi));
  return EP_OK;
}

int oc_download_cfield(oc_ctx* c, int which, double* out) {
  if (!c || !out) return EP_ERR_INVALID_ARG;
  const std::vector<cd>* v = nullptr;
  switch (which) {
    case EP_CFIELD_PSI: v = &c->psi; break;
    case EP_CFIELD_PSIOLD1: v = &c->psiold[0]; break;
    case EP_CFIELD_PSIOLD2: v = &c->psiold[1]; break;
    case EP_CFIELD_PSIOLD3: v = &c->psiold[2]; break;
    case EP_CFIELD_HPSIOLD1: v = &c->hpsiold[0]; break;
    case EP_CFIELD_HPSIOLD2: v = &c->hpsiold[1]; break;
    case EP_CFIELD_PC: v = &c->pc; break;
    case EP_CFIELD_Q: v = &c->q; break;
    default: return EP_ERR_INVALID_ARG;
  }
  std::copy(v->begin(), v->end(), reinterpret_cast<cd*>(out));
  return EP_OK;
}

int oc_download_field(oc_ctx* c, int which, double* out) {
  if (!c || !out) return EP_ERR_INVALID_ARG;
  const std::vector<double>* v = nullptr;
  switch (which) {
    case EP_FIELD_DEN: v = &c->den; break;
    case EP_FIELD_POT4: v = &c->pot4; break;
    case EP_FIELD_UIMP: v = &c->uimp; break;
    case EP_FIELD_DENCG: v = &c->dencg; break;
    case EP_FIELD_DELJ4: v = &c->delj4; break;
    case EP_FIELD_DXDEN: v = &c->dxden; break;
    case EP_FIELD_DYDEN: v = &c->dyden; break;
    case EP_FIELD_DZDEN: v = &c->dzden; break;
    case EP_FIELD_FALFS: v = &c->falfs; break;
    case EP_FIELD_INTXALF: v = &c->intx; break;
    case EP_FIELD_INTYALF: v = &c->inty; break;
    case EP_FIELD_INTZALF: v = &c->intz; break;
    case EP_FIELD_UALPHAS: v = &c->ualphas; break;
    case EP_FIELD_VPI: v = &c->vpi; break;
    case EP_FIELD_DELTA: v = &c->delta; break;
    case EP_FIELD_SIGDEL:
      if (c->cfg.state != EP_STATE_D) return EP_ERR_INVALID_ARG;
      v = &c->sigdel;
      break;
    default: return EP_ERR_INVALID_ARG;
  }
  std::copy(v->begin(), v->end(), out);
  return EP_OK;
}

// D-state angular factors at x = r - rimp (potenimp.f90:68-117, the same
// algebra in potinvar :346-390 and instates.f90:478-527): the d harmonics
// armonicd = (d1..d5, d0) and the symmetric matrix P whose upper triangle
// the reference writes out (MP before the factor dV2).
static void d_factors(double xx, double yy, double zz, double arm[6], double P[5][5]) {
  const double sqr3 = std::sqrt(3.0), sqr3o2 = std::sqrt(3.0) / 2.0, insqr3 = 1.0 / std::sqrt(3.0), in3 = 1.0 / 3.0;
  const double d0 = xx * xx + yy * yy + zz * zz;
  const double d1 = sqr3 * xx * yy;
  const double d2 = sqr3 * yy * zz;
  const double d3 = (-xx * xx - yy * yy + 2 * zz * zz) / 2;
  const double d4 = sqr3 * xx * zz;
  const double d5 = sqr3o2 * (xx * xx - yy * yy);
  arm[0] = d1; arm[1] = d2; arm[2] = d3; arm[3] = d4; arm[4] = d5; arm[5] = d0;
  const double sd1 = d1 * d1, sd2 = d2 * d2, sd4 = d4 * d4, sd5 = d5 * d5;
  const double sumd3d5 = d3 + insqr3 * d5, difd3d5 = d3 - insqr3 * d5;
  P[0][0] = in3 * (sd2 + sd4 + 4.0 * sd5);
  P[1][1] = in3 * (sd1 + sd4) + sumd3d5 * sumd3d5;
  P[2][2] = sd4 + sd2;
  P[3][3] = in3 * (sd1 + sd2) + difd3d5 * difd3d5;
  P[4][4] = in3 * (sd2 + sd4 + 4.0 * sd1);
  P[0][1] = -4.0 * in3 * d1 * d2 + insqr3 * d4 * d0;
  P[0][2] = -2.0 * insqr3 * d2 * d4;
  P[0][3] = -4.0 * in3 * d1 * d4 + insqr3 * d2 * d0;
  P[0][4] = -4.0 * in3 * d1 * d5;
  P[1][2] = insqr3 * d1 * d4 - d2 * sumd3d5;
  P[1][3] = -4.0 * in3 * d2 * d4 + insqr3 * d1 * d0;
  P[1][4] = -d1 * d4 - insqr3 * d2 * sumd3d5;
  P[2][3] = insqr3 * d1 * d2 - d4 * difd3d5;
  P[2][4] = insqr3 * (sd2 - sd4);
  P[3][4] = d1 * d2 + insqr3 * d4 * difd3d5;
  for (int i = 0; i < 5; ++i)
    for (int j = i + 1; j < 5; ++j) P[j][i] = P[i][j];
}

// Spin-orbit matrix SOD of the D state (potenimp.f90:429-451,
// instates.f90:549-571): upper triangle, then SOD(j,i) = conj(SOD(i,j)).
static void sod_matrix(cd S[10][10]) {
  const cd uim(0.0, 1.0);
  const double sqr3 = std::sqrt(3.0);
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) S[i][j] = cd(0);
  S[0][3] = 1.0;  S[0][7] = -uim;  S[0][8] = 2.0 * uim;
  S[1][2] = -1.0; S[1][6] = -uim;  S[1][9] = -2.0 * uim;
  S[2][5] = -uim * sqr3; S[2][6] = uim; S[2][9] = -uim;
  S[3][4] = -uim * sqr3; S[3][7] = -uim; S[3][8] = -uim;
  S[4][7] = -sqr3; S[5][6] = sqr3; S[6][9] = -1.0; S[7][8] = 1.0;
  for (int i = 0; i < 10; ++i)
    for (int j = i; j < 10; ++j) S[j][i] = std::conj(S[i][j]);
}

// updatepoten D branch (potenimp.f90:545-566) + potenimp D state (:47-182).
static void potenimp_d(oc_ctx* c) {
  const double rmax = (c->npot - 1) * c->delinter;
  const double zeror = 1e-3;
  const int nx = c->nx, ny = c->ny;
  const double* rr = c->rimp;
  const cd* iv = c->invar;
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < (long long)c->N; ++p) {
    const int ix = (int)(p % nx), iy = (int)((p / nx) % ny), iz = (int)(p / ((long long)nx * ny));
    const double zt = (c->z[iz] - rr[2]) * (c->z[iz] - rr[2]);
    const double yt = (c->y[iy] - rr[1]) * (c->y[iy] - rr[1]) + zt;
    const double r2 = (c->x[ix] - rr[0]) * (c->x[ix] - rr[0]) + yt;
    const double r4 = r2 * r2;
    const double r = std::sqrt(r2);
    c->delta[p] = update_interp(r, c->npot, rmax, c->potdel.data());
    if (r > zeror) {
      c->vpi[p] = update_interp(r, c->npot, rmax, c->potpi.data()) / r4;
      c->sigdel[p] = update_interp(r, c->npot, rmax, c->potsigdel.data()) / r4;
    } else {
      c->vpi[p] = c->umax_pi;
      c->sigdel[p] = c->umax_sigma;
    }
    const double xx = c->x[ix] - rr[0], yy = c->y[iy] - rr[1], zz = c->z[iz] - rr[2];
    const double dVdel = c->delta[p], dV1 = c->vpi[p], dV2 = c->sigdel[p];
    double arm[6], P[5][5], MP[5][5];
    d_factors(xx, yy, zz, arm, P);
    // MP = sumVdel + MS + MP (the reference's names: MS = armonicd (x)
    // armonicd * dV1, MP = P * dV2)
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) MP[i][j] = (i == j ? dVdel : 0.0) + arm[i] * arm[j] * dV1 + P[i][j] * dV2;
    // MatD = MP (x) 1_2; Aux = sum_i (MatD iv)_i conj(iv_i), real part
    double aux = 0.0;
    for (int i = 0; i < 10; ++i) {
      cd ivs(0);
      for (int j = 0; j < 10; ++j)
        if ((i & 1) == (j & 1)) ivs += MP[i / 2][j / 2] * iv[j];
      aux += (ivs * std::conj(iv[i])).real();
    }
    c->uimp[p] = std::min(aux, 1000.0);
  }
}

// updatepoten (potenimp.f90:515-585) + potenimp (:1-189, cap :184-186).
int oc_potenimp(oc_ctx* c) {
  if (!c) return EP_ERR_INVALID_ARG;
  if (c->cfg.impurity == EP_IMPURITY_NONE) {
    std::fill(c->uimp.begin(), c->uimp.end(), 0.0);
    return EP_OK;
  }
  if (!c->have_tables) return fail(c, EP_ERR_STATE, "impurity tables not set");
  if (c->cfg.state == EP_STATE_D) {
    potenimp_d(c);
    return EP_OK;
  }
  const double rmax = (c->npot - 1) * c->delinter;
  const double zeror = 1e-3;
  const int nx = c->nx, ny = c->ny;
  const double* rr = c->rimp;
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < (long long)c->N; ++p) {
    const int ix = (int)(p % nx), iy = (int)((p / nx) % ny), iz = (int)(p / ((long long)nx * ny));
    const double zt = (c->z[iz] - rr[2]) * (c->z[iz] - rr[2]);
    const double yt = (c->y[iy] - rr[1]) * (c->y[iy] - rr[1]) + zt;
    const double r2 = (c->x[ix] - rr[0]) * (c->x[ix] - rr[0]) + yt;
    const double r = std::sqrt(r2);
    const double vp = update_interp(r, c->npot, rmax, c->potpi.data());
    const double dl = (r > zeror) ? update_interp(r, c->npot, rmax, c->potdel.data()) / r2 : c->umax_sigma;
    c->vpi[p] = vp;
    c->delta[p] = dl;
    const double xx = c->x[ix] - rr[0], yy = c->y[iy] - rr[1], zz = c->z[iz] - rr[2];
    const cd* iv = c->invar;
    const cd odd = iv[0] * xx + iv[2] * yy + iv[4] * zz;
    const cd even = iv[1] * xx + iv[3] * yy + iv[5] * zz;
    double u = vp + dl * (std::norm(odd) + std::norm(even));
    c->uimp[p] = std::min(u, 1000.0);
  }
  return EP_OK;
}

// derden (energy.f90:207-227 in poten.f90's file order).
static void derden(oc_ctx* c) {
  deriv(c, 1, 0, c->den.data(), c->dxden.data());
  deriv(c, 1, 1, c->den.data(), c->dyden.data());
  deriv(c, 1, 2, c->den.data(), c->dzden.data());
}

static void kmul(const std::vector<cd>& a, const std::vector<double>& k, std::vector<cd>& o) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)a.size(); ++i) o[i] = a[i] * k[i];
}
static void kmul_inplace(std::vector<cd>& a, const std::vector<double>& k) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)a.size(); ++i) a[i] *= k[i];
}
static void bk(oc_ctx* c, const std::vector<cd>& in, std::vector<double>& out) {
  irfft3(c->nx, c->ny, c->nz, in.data(), out.data());
  const double s = c->renor;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)c->N; ++i) out[i] *= s;
}
static void fw(oc_ctx* c, const std::vector<double>& in, std::vector<cd>& out) {
  rfft3(c->nx, c->ny, c->nz, in.data(), out.data());
}

// term_alfa (term_alfa.f90:5-109).
static void term_alfa(oc_ctx* c) {
  const long long N = (long long)c->N;
  const double den0s = c->cfg.den0s;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i) {
    c->falfs[i] = 1.0 - c->denalf[i] / den0s;
    c->sto1[i] = c->falfs[i] * c->dxden[i];
    c->sto2[i] = c->falfs[i] * c->dyden[i];
    c->sto3[i] = c->falfs[i] * c->dzden[i];
  }
  fw(c, c->sto1, c->wk1); fw(c, c->sto2, c->wk2); fw(c, c->sto3, c->wk3);
  kmul_inplace(c->wk1, c->kalfs); kmul_inplace(c->wk2, c->kalfs); kmul_inplace(c->wk3, c->kalfs);
  bk(c, c->wk1, c->intx); bk(c, c->wk2, c->inty); bk(c, c->wk3, c->intz);
  if (c->cfg.core != EP_CORE_OTC) return;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i)
    c->sto1[i] = (c->dxden[i] * c->intx[i]) + (c->dyden[i] * c->inty[i]) + (c->dzden[i] * c->intz[i]);
  fw(c, c->sto1, c->wk1);
  kmul_inplace(c->wk1, c->kalfs);
  bk(c, c->wk1, c->ualphas);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i) {
    c->ualphas[i] = c->ualphas[i] / den0s;
    c->sto1[i] = c->falfs[i] * c->intx[i];
    c->sto2[i] = c->falfs[i] * c->inty[i];
    c->sto3[i] = c->falfs[i] * c->intz[i];
  }
  deriv(c, 1, 0, c->sto1.data(), c->sto4.data());
  deriv(c, 1, 1, c->sto2.data(), c->sto5.data());
  deriv(c, 1, 2, c->sto3.data(), c->sto6.data());
  const double f = c->cfg.h2o2m4 * c->cfg.alphas;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i)
    c->ualphas[i] = (c->ualphas[i] + c->sto4[i] + c->sto5[i] + c->sto6[i]) * c->cfg.h2o2m4 * c->cfg.alphas;
  (void)f;
}

// poten (poten.f90:5-131).
int oc_poten(oc_ctx* c) {
  if (!c) return EP_ERR_INVALID_ARG;
  const long long N = (long long)c->N;
  const ep_config& g = c->cfg;
  fw(c, c->den, c->fden);
  kmul(c->fden, c->wcgk, c->wk1);
  bk(c, c->wk1, c->dencg);
  derden(c);
  kmul(c->fden, c->fvlj4, c->wk1);
  bk(c, c->wk1, c->delj4);
  const double a0 = g.cp4 / 2.0, a1 = g.cpp4 / 3.0;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i) c->sto1[i] = c->den[i] * c->dencg[i] * (g.cp4 + g.cpp4 * c->dencg[i]);
  fw(c, c->sto1, c->wk1);
  kmul_inplace(c->wk1, c->wcgk);
  bk(c, c->wk1, c->sto1);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i) {
    const double t = std::tanh(g.beta * (c->den[i] - g.den_m));
    c->penalty[i] = g.C * (1.0 + t + g.beta * c->den[i] * (1.0 - t * t));
    c->pot4[i] = c->delj4[i] + c->dencg[i] * c->dencg[i] * (a0 + a1 * c->dencg[i]) + c->sto1[i];
  }
  if (g.core == EP_CORE_OTC) {
    kmul(c->fden, c->kalfs, c->wk1);
    bk(c, c->wk1, c->denalf);
    term_alfa(c);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < N; ++i) c->pot4[i] = c->pot4[i] + c->ualphas[i];
  }
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i) c->pot4[i] = c->pot4[i] + c->penalty[i];
  c->have_field = true;
  return EP_OK;
}

// energy (energy.f90:12-202), P-state spin-orbit term.
int oc_energy(oc_ctx* c, ep_energies* e) {
  if (!c || !e) return EP_ERR_INVALID_ARG;
  const ep_config& g = c->cfg;
  std::vector<cd> d1(c->N), d2(c->N), d3(c->N);
  deriv(c, 1, 0, c->psi.data(), d1.data());
  deriv(c, 1, 1, c->psi.data(), d2.data());
  deriv(c, 1, 2, c->psi.data(), d3.data());
  const double aux1 = 0.5 * g.cp4, aux2 = (1.0 / 3.0) * g.cpp4;
  const size_t N = c->N;
  double ekin4 = par_sum(N, [&](size_t i) { return std::norm(d1[i]) + std::norm(d2[i]) + std::norm(d3[i]); });
  double elj4 = par_sum(N, [&](size_t i) { return c->delj4[i] * c->den[i]; });
  double ecor4 = par_sum(N, [&](size_t i) {
    const double a3 = c->den[i], a4 = c->dencg[i];
    return a3 * (a4 * a4) * (aux1 + aux2 * a4);
  });
  double ealphas = 0.0;
  if (g.core == EP_CORE_OTC) {
    ealphas = par_sum(N, [&](size_t i) {
      return c->falfs[i] * (c->dxden[i] * c->intx[i] + c->dyden[i] * c->inty[i] + c->dzden[i] * c->intz[i]);
    });
    ealphas = -g.h2o2m4 * 0.5 * g.alphas * ealphas * c->dxyz;
  }
  double esolid = g.C * par_sum(N, [&](size_t i) {
    return c->den[i] * (1.0 + std::tanh(g.beta * (c->den[i] - g.den_m)));
  }) * c->dxyz;
  ekin4 = g.h2o2m4 * ekin4 * c->dxyz;
  elj4 = 0.5 * elj4 * c->dxyz;
  ecor4 = ecor4 * c->dxyz;
  double etot4 = ekin4 + elj4 + ecor4;
  if (g.core == EP_CORE_OTC) etot4 = etot4 + ealphas;
  const double mAg_u = g.mimpur * 0.0207569277;
  const double ekinx = 0.5 * mAg_u * (c->vimp[0] * c->vimp[0] + c->vimp[1] * c->vimp[1] + c->vimp[2] * c->vimp[2]);
  double eHeX = 0.0, uplus = 0.0;
  if (g.impurity != EP_IMPURITY_NONE) {
    const int nx = c->nx, ny = c->ny;
    auto rof = [&](size_t p) {
      const int ix = (int)(p % nx), iy = (int)((p / nx) % ny), iz = (int)(p / ((size_t)nx * ny));
      const double a = c->rimp[0] - c->x[ix], b = c->rimp[1] - c->y[iy], d = c->rimp[2] - c->z[iz];
      return std::sqrt(a * a + b * b + d * d);
    };
    eHeX = par_sum(N, [&](size_t p) { return rof(p) >= g.z_exciplex_exclusion ? c->den[p] * c->uimp[p] : 0.0; }) * c->dxyz;
    uplus = par_sum(N, [&](size_t p) {
      const double r = rof(p);
      return r >= g.z_exciplex_exclusion ? c->den[p] * select_pot(c->plus.p, r) : 0.0;
    }) * c->dxyz;
  }
  const cd* iv = c->invar;
  cd ivs[10];
  for (int i = 0; i < 10; ++i) ivs[i] = std::conj(iv[i]);
  double eso;
  if (g.state == EP_STATE_D) {
    // energy.f90:176-190: eso = Als_D * 0.5 * sum_i (SOD iv)_i conj(iv_i), real part
    cd S[10][10];
    sod_matrix(S);
    cd vls(0);
    for (int i = 0; i < 10; ++i) {
      cd t(0);
      for (int j = 0; j < 10; ++j) t += S[i][j] * iv[j];
      vls += t * std::conj(iv[i]);
    }
    vls *= 0.5;
    eso = (vls * g.als_d).real();
  } else {
    const double Also2 = 0.5 * g.als_p;
    eso = Also2 * (2.0 * (ivs[0] * iv[5] - ivs[1] * iv[4]).real() +
                   2.0 * (ivs[0] * iv[2] + ivs[3] * iv[1] + ivs[2] * iv[5] + ivs[3] * iv[4]).imag());
  }
  e->ekin4 = ekin4; e->elj4 = elj4; e->ecor4 = ecor4; e->ealphas = ealphas; e->esolid = esolid;
  e->etot4 = etot4; e->ekinx = ekinx; e->eHeX = eHeX; e->uplus = uplus; e->eso = eso;
  e->eimpu = ekinx + eHeX + eso;
  e->etot = etot4 + e->eimpu;
  e->n4 = par_sum(N, [&](size_t i) { return c->den[i]; }) * c->dxyz;
  return EP_OK;
}

// forceimp (potenimp.f90:193-258).  With Lfilter_exciplex_force the z
// component sums the planes iz0..nz (impurity below z = 0) or 1..nz0
// (:211-248); aux2, the He-He correction, is commented out there.
int oc_forceimp(oc_ctx* c, double* F) {
  if (!c || !F) return EP_ERR_INVALID_ARG;
  const size_t N = c->N;
  const ep_config& g = c->cfg;
  F[0] = -par_sum(N, [&](size_t i) { return c->dxden[i] * c->uimp[i]; }) * c->dxyz;
  F[1] = -par_sum(N, [&](size_t i) { return c->dyden[i] * c->uimp[i]; }) * c->dxyz;
  if (g.filter_exciplex_force) {
    int izfirst = 1, izlast = c->nz;  // 1-based, inclusive
    if (c->rimp[2] < 0.0) {
      int iz0 = (int)((c->rimp[2] - c->z[0] + g.z_exciplex_exclusion) / c->hz + 1.5);
      izfirst = std::max(1, iz0);
    } else {
      int nz0 = (int)((c->rimp[2] - c->z[0] - g.z_exciplex_exclusion) / c->hz + 1.5);
      izlast = std::min(c->nz, nz0);
    }
    const size_t nxy = (size_t)c->nx * c->ny;
    double aux1 = par_sum(N, [&](size_t i) {
      const int iz = (int)(i / nxy) + 1;
      return (iz >= izfirst && iz <= izlast) ? c->dzden[i] * c->uimp[i] : 0.0;
    });
    const double aux2 = 0.0;
    F[2] = -aux1 * c->dxyz + -aux2 * c->dxyz;
  } else {
    F[2] = -par_sum(N, [&](size_t i) { return c->dzden[i] * c->uimp[i]; }) * c->dxyz;
  }
  // the callers' aimp = F / mAg_u (DFT4He3d.f90:454-455, steppc.f90:114-115)
  if (c->cfg.impurity == EP_IMPURITY_MOVING)
    for (int i = 0; i < 3; ++i) c->aimp[i] = F[i] / (c->cfg.mimpur * 0.0207569277);
  return EP_OK;
}

// The density-weighted D-state matrix MP + MS + sumVdel, times dxyz
// (potenimp.f90:331-405; instates.f90:457-534), summed as the reference
// does: the three matrices separately, then added.
static void dmatrix(oc_ctx* c, double M[5][5]) {
  const int nx = c->nx, ny = c->ny;
  const double* rr = c->rimp;
  const size_t N = c->N;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  // per thread: MP, MS upper triangles and sumVdel, compensated
  std::vector<std::vector<Neu>> acc(nt, std::vector<Neu>(31));
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    std::vector<Neu>& a = acc[t];
#pragma omp for schedule(static)
    for (long long p = 0; p < (long long)N; ++p) {
      const int ix = (int)(p % nx), iy = (int)((p / nx) % ny), iz = (int)(p / ((long long)nx * ny));
      const double xx = c->x[ix] - rr[0], yy = c->y[iy] - rr[1], zz = c->z[iz] - rr[2];
      const double aux = c->den[p];
      const double dVdel = c->delta[p] * aux, dV1 = c->vpi[p] * aux, dV2 = c->sigdel[p] * aux;
      double arm[6], P[5][5];
      d_factors(xx, yy, zz, arm, P);
      int k = 0;
      for (int i = 0; i < 5; ++i)
        for (int j = i; j < 5; ++j, ++k) {
          a[k].add(P[i][j] * dV2);
          a[15 + k].add(arm[i] * arm[j] * dV1);
        }
      a[30].add(dVdel);
    }
  }
  double tot[31];
  for (int q = 0; q < 31; ++q) {
    Neu s;
    for (int t = 0; t < nt; ++t) s.add(acc[t][q].get());
    tot[q] = s.get();
  }
  int k = 0;
  for (int i = 0; i < 5; ++i)
    for (int j = i; j < 5; ++j, ++k) {
      const double v = tot[k] * c->dxyz + tot[15 + k] * c->dxyz + (i == j ? tot[30] * c->dxyz : 0.0);
      M[i][j] = M[j][i] = v;
    }
}

int oc_impurity_matrix_d(oc_ctx* c, double* m25) {
  if (!c || !m25) return EP_ERR_INVALID_ARG;
  if (c->cfg.state != EP_STATE_D) return fail(c, EP_ERR_STATE, "the D-state matrix needs state = EP_STATE_D");
  double M[5][5];
  dmatrix(c, M);
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) m25[5 * i + j] = M[i][j];
  return EP_OK;
}

// potinvar, D state (potenimp.f90:331-475, :487-492): Hiv = (MatD + Als_D/2
// SOD) iv with MatD = M (x) 1_2, then -i (Hiv - Ev0 iv).
static void potinvar_d(oc_ctx* c, cd* Hiv) {
  const ep_config& g = c->cfg;
  double M[5][5];
  dmatrix(c, M);
  cd S[10][10];
  sod_matrix(S);
  const cd uim(0.0, 1.0);
  const double Also2 = g.als_d / 2.0;
  const cd* iv = c->invar;
  for (int i = 0; i < 10; ++i) {
    cd h(0);
    for (int j = 0; j < 10; ++j) {
      const double md = ((i & 1) == (j & 1)) ? M[i / 2][j / 2] : 0.0;
      h += (md + Also2 * S[i][j]) * iv[j];
    }
    Hiv[i] = h;
  }
  for (int i = 0; i < 10; ++i) Hiv[i] = -uim * (Hiv[i] - g.ev0 * iv[i]);
}

// potinvar, P state (potenimp.f90:261-330, :487-492).
static void potinvar_(oc_ctx* c, cd* Hiv) {
  const ep_config& g = c->cfg;
  if (g.state == EP_STATE_D) {
    potinvar_d(c, Hiv);
    return;
  }
  const int nx = c->nx, ny = c->ny;
  const double* rr = c->rimp;
  auto X = [&](size_t p) { return c->x[(int)(p % nx)] - rr[0]; };
  auto Y = [&](size_t p) { return c->y[(int)((p / nx) % ny)] - rr[1]; };
  auto Z = [&](size_t p) { return c->z[(int)(p / ((size_t)nx * ny))] - rr[2]; };
  const size_t N = c->N;
  const double uxx = par_sum(N, [&](size_t p) { double xx = X(p); return c->den[p] * (c->delta[p] * xx * xx + c->vpi[p]); });
  const double uxy = par_sum(N, [&](size_t p) { return c->den[p] * c->delta[p] * X(p) * Y(p); });
  const double uxz = par_sum(N, [&](size_t p) { return c->den[p] * c->delta[p] * X(p) * Z(p); });
  const double uyy = par_sum(N, [&](size_t p) { double yy = Y(p); return c->den[p] * (c->delta[p] * yy * yy + c->vpi[p]); });
  const double uyz = par_sum(N, [&](size_t p) { return c->den[p] * c->delta[p] * Y(p) * Z(p); });
  const double uzz = par_sum(N, [&](size_t p) { double zz = Z(p); return c->den[p] * (c->delta[p] * zz * zz + c->vpi[p]); });
  const cd* iv = c->invar;
  const cd uim(0.0, 1.0);
  const double Also2 = g.als_p / 2.0, dxyz = c->dxyz;
  Hiv[0] = (uxx * iv[0] + uxy * iv[2] + uxz * iv[4]) * dxyz + Also2 * (-uim * iv[2] + iv[5]);
  Hiv[1] = (uxx * iv[1] + uxy * iv[3] + uxz * iv[5]) * dxyz + Also2 * (uim * iv[3] - iv[4]);
  Hiv[2] = (uxy * iv[0] + uyy * iv[2] + uyz * iv[4]) * dxyz + Also2 * (uim * iv[0] - uim * iv[5]);
  Hiv[3] = (uxy * iv[1] + uyy * iv[3] + uyz * iv[5]) * dxyz + Also2 * (-uim * iv[1] - uim * iv[4]);
  Hiv[4] = (uxz * iv[0] + uyz * iv[2] + uzz * iv[4]) * dxyz + Also2 * (-iv[1] + uim * iv[3]);
  Hiv[5] = (uxz * iv[1] + uyz * iv[3] + uzz * iv[5]) * dxyz + Also2 * (iv[0] + uim * iv[2]);
  for (int i = 6; i < 10; ++i) Hiv[i] = cd(0);
  for (int i = 0; i < 10; ++i) Hiv[i] = -uim * (Hiv[i] - g.ev0 * iv[i]);
}

// (Vx, Vy, Vz, Vxy, Vxz, Vyz) of instates.f90:123-147.
int oc_impurity_moments(oc_ctx* c, double* v6) {
  if (!c || !v6) return EP_ERR_INVALID_ARG;
  const int nx = c->nx, ny = c->ny;
  const double* rr = c->rimp;
  auto X = [&](size_t p) { return c->x[(int)(p % nx)] - rr[0]; };
  auto Y = [&](size_t p) { return c->y[(int)((p / nx) % ny)] - rr[1]; };
  auto Z = [&](size_t p) { return c->z[(int)(p / ((size_t)nx * ny))] - rr[2]; };
  const size_t N = c->N;
  v6[0] = par_sum(N, [&](size_t p) { double xx = X(p); return c->den[p] * (c->delta[p] * xx * xx + c->vpi[p]); });
  v6[1] = par_sum(N, [&](size_t p) { double yy = Y(p); return c->den[p] * (c->delta[p] * yy * yy + c->vpi[p]); });
  v6[2] = par_sum(N, [&](size_t p) { double zz = Z(p); return c->den[p] * (c->delta[p] * zz * zz + c->vpi[p]); });
  v6[3] = par_sum(N, [&](size_t p) { return c->den[p] * c->delta[p] * X(p) * Y(p); });
  v6[4] = par_sum(N, [&](size_t p) { return c->den[p] * c->delta[p] * X(p) * Z(p); });
  v6[5] = par_sum(N, [&](size_t p) { return c->den[p] * c->delta[p] * Y(p) * Z(p); });
  for (int k = 0; k < 6; ++k) v6[k] *= c->dxyz;
  return EP_OK;
}

int oc_potinvar(oc_ctx* c, double* hinvar) {
  if (!c || !hinvar) return EP_ERR_INVALID_ARG;
  cd H[10];
  potinvar_(c, H);
  for (int i = 0; i < 10; ++i) { hinvar[2 * i] = H[i].real(); hinvar[2 * i + 1] = H[i].imag(); }
  return EP_OK;
}

// Laplacian sum sto1c+sto2c+sto3c of psi (steppc.f90:35-37).
static void laplacian(oc_ctx* c) {
  std::vector<cd> t(c->N);
  deriv(c, 2, 0, c->psi.data(), c->lap.data());
  deriv(c, 2, 1, c->psi.data(), t.data());
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)c->N; ++i) c->lap[i] += t[i];
  deriv(c, 2, 2, c->psi.data(), t.data());
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)c->N; ++i) c->lap[i] += t[i];
}

// H-apply: timec*((lap)*h2o2m4 - pot4*psi) + cimp*uimp*psi with timec = 1,
// cimp = -1 (imaginary time) or timec = i, cimp = -i (real time, exactly
// steppc.f90:53).
static inline cd happly(const oc_ctx* c, cd lap, cd psi, double pot4, double uimp) {
  const cd L = lap * c->cfg.h2o2m4 - pot4 * psi;
  if (c->cfg.time_mode == EP_REAL_TIME) {
    const cd tL(-L.imag(), L.real());
    const cd ui(uimp * psi.imag(), -uimp * psi.real());
    return tL + ui;
  }
  return L - uimp * psi;
}

static bool impurity_moving(const oc_ctx* c) { return c->cfg.impurity == EP_IMPURITY_MOVING; }

// Field refresh between stages (steppc.f90:111-117, steprk.f90:164-174).
static int refresh(oc_ctx* c) {
  if (impurity_moving(c)) {
    int s = oc_potenimp(c);
    if (s) return s;
  }
  oc_poten(c);
  if (impurity_moving(c)) {
    const double mAg_u = c->cfg.mimpur * 0.0207569277;
    double F[3];
    oc_forceimp(c, F);
    for (int i = 0; i < 3; ++i) c->aimp[i] = F[i] / mAg_u;
    if (!c->cfg.fix_lambda) potinvar_(c, c->hinvar);
  }
  return EP_OK;
}

// steprk (steprk.f90:1-191).
int oc_steprk(oc_ctx* c, double deltat) {
  if (!c) return EP_ERR_INVALID_ARG;
  if (!c->have_field) return fail(c, EP_ERR_STATE, "poten() must run before steprk");
  const double s2 = std::sqrt(2.0);
  const double arun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 1.0 / 6.0};
  const double brun[4] = {2.0, 1.0, 1.0, 2.0};
  const double crun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 0.5};
  const long long N = (long long)c->N;
  const bool mov = impurity_moving(c);
  for (int jr = 0; jr < 4; ++jr) {
    laplacian(c);
    const double a = arun[jr], b = brun[jr], cr = crun[jr];
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < N; ++i) {
      const cd h = happly(c, c->lap[i], c->psi[i], c->pot4[i], c->uimp[i]);
      const cd aux2 = a * (h - b * c->q[i]);
      c->q[i] = c->q[i] + 3.0 * aux2 - cr * h;
      if (jr == 0) {
        c->hpsiold[1][i] = c->hpsiold[0][i];
        c->hpsiold[0][i] = h;
        c->psiold[2][i] = c->psiold[1][i];
        c->psiold[1][i] = c->psiold[0][i];
        c->psiold[0][i] = c->psi[i];
      }
      c->psi[i] = c->psi[i] + deltat * aux2;
      c->den[i] = std::norm(c->psi[i]);
    }
    for (long long i = 0; i < N; ++i)
      if (!(c->den[i] > 0.0)) return fail(c, EP_ERR_NONFINITE, "steprk: density not positive");
    if (mov) {
      for (int k = 0; k < 3; ++k) {
        double ax = a * (c->vimp[k] - b * c->qr[k]);
        c->qr[k] = c->qr[k] + 3.0 * ax - cr * c->vimp[k];
        if (jr == 0) {
          c->rimpold[k][2] = c->rimpold[k][1];
          c->rimpold[k][1] = c->rimpold[k][0];
          c->rimpold[k][0] = c->rimp[k];
        }
        c->rimp[k] = c->rimp[k] + deltat * ax;
      }
      for (int k = 0; k < 3; ++k) {
        double ax = a * (c->aimp[k] - b * c->qv[k]);
        c->qv[k] = c->qv[k] + 3.0 * ax - cr * c->aimp[k];
        if (jr == 0) {
          c->aimpold[k][1] = c->aimpold[k][0];
          c->aimpold[k][0] = c->aimp[k];
          c->vimpold[k][2] = c->vimpold[k][1];
          c->vimpold[k][1] = c->vimpold[k][0];
          c->vimpold[k][0] = c->vimp[k];
        }
        c->vimp[k] = c->vimp[k] + deltat * ax;
      }
      if (!c->cfg.fix_lambda) {
        for (int k = 0; k < 10; ++k) {
          cd ax = a * (c->hinvar[k] - b * c->qiv[k]);
          c->qiv[k] = c->qiv[k] + 3.0 * ax - cr * c->hinvar[k];
          if (jr == 0) {
            c->hinvarold[k][1] = c->hinvarold[k][0];
            c->hinvarold[k][0] = c->hinvar[k];
            c->invarold[k][2] = c->invarold[k][1];
            c->invarold[k][1] = c->invarold[k][0];
            c->invarold[k][0] = c->invar[k];
          }
          c->invar[k] = c->invar[k] + deltat * ax;
        }
      }
    }
    if (jr <= 2) refresh(c);
  }
  for (int i = 0; i < 3; ++i) { c->ioldp[i] = i; c->ioldr[i] = i; c->ioldv[i] = i; c->ioldiv[i] = i; }
  for (int i = 0; i < 2; ++i) { c->ioldh[i] = i; c->iolda[i] = i; c->ioldhiv[i] = i; }
  return EP_OK;
}

// steppc (steppc.f90:1-230).
int oc_steppc(oc_ctx* c, double deltat, ep_step_errors* err) {
  if (!c) return EP_ERR_INVALID_ARG;
  if (!c->have_field) return fail(c, EP_ERR_STATE, "poten() must run before steppc");
  const double c112 = 112.0 / 121.0, c9 = 9.0 / 121.0, c4o3 = 4.0 / 3.0;
  const long long N = (long long)c->N;
  const bool mov = impurity_moving(c);
  laplacian(c);
  {
    cd* po3 = c->psiold[c->ioldp[2]].data();
    cd* h1 = c->hpsiold[c->ioldh[0]].data();
    cd* h2 = c->hpsiold[c->ioldh[1]].data();
    const double f = c4o3 * deltat;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < N; ++i) {
      const cd h = happly(c, c->lap[i], c->psi[i], c->pot4[i], c->uimp[i]);
      const cd pp = po3[i] + f * (2.0 * h - h1[i] + 2.0 * h2[i]);
      po3[i] = c->psi[i];
      c->psi[i] = pp - c112 * c->pc[i];
      c->pc[i] = pp;
      h2[i] = h;
      c->den[i] = std::norm(c->psi[i]);
    }
    std::swap(c->ioldh[0], c->ioldh[1]);
  }
  if (mov) {
    double auxr[3];
    int r1 = c->ioldr[0], r2 = c->ioldr[1], r3 = c->ioldr[2];
    int v1 = c->ioldv[0], v2 = c->ioldv[1], v3 = c->ioldv[2];
    int a1 = c->iolda[0], a2 = c->iolda[1];
    (void)r1; (void)r2; (void)v3;
    for (int k = 0; k < 3; ++k)
      auxr[k] = c->rimpold[k][r3] + c4o3 * deltat * (2.0 * c->vimp[k] - c->vimpold[k][v1] + 2.0 * c->vimpold[k][v2]);
    for (int k = 0; k < 3; ++k) {
      c->rimpold[k][r3] = c->rimp[k];
      c->rimp[k] = auxr[k] - c112 * c->pcr[k];
      c->pcr[k] = auxr[k];
    }
    for (int k = 0; k < 3; ++k)
      auxr[k] = c->vimpold[k][v3] + c4o3 * deltat * (2.0 * c->aimp[k] - c->aimpold[k][a1] + 2.0 * c->aimpold[k][a2]);
    for (int k = 0; k < 3; ++k) {
      c->vimpold[k][v3] = auxr[k] - c112 * c->pcv[k];
      c->pcv[k] = auxr[k];
    }
    if (!c->cfg.fix_lambda) {
      cd auxc[10];
      int i3 = c->ioldiv[2], h1 = c->ioldhiv[0], h2 = c->ioldhiv[1];
      for (int k = 0; k < 10; ++k)
        auxc[k] = c->invarold[k][i3] + c4o3 * deltat * (2.0 * c->hinvar[k] - c->hinvarold[k][h1] + 2.0 * c->hinvarold[k][h2]);
      for (int k = 0; k < 10; ++k) {
        c->invarold[k][i3] = c->invar[k];
        c->invar[k] = auxc[k] - c112 * c->pciv[k];
        c->pciv[k] = auxc[k];
      }
    }
    for (int k = 0; k < 3; ++k) c->aimpold[k][a2] = c->aimp[k];
    for (int k = 0; k < 10; ++k) c->hinvarold[k][c->ioldhiv[1]] = c->hinvar[k];
    std::swap(c->iolda[0], c->iolda[1]);
    std::swap(c->ioldhiv[0], c->ioldhiv[1]);
  }
  refresh(c);
  laplacian(c);
  double errHe;
  {
    cd* po3 = c->psiold[c->ioldp[2]].data();
    cd* po2 = c->psiold[c->ioldp[1]].data();
    cd* h1 = c->hpsiold[c->ioldh[0]].data();
    cd* h2 = c->hpsiold[c->ioldh[1]].data();
    const double f = 3.0 * deltat;
    std::vector<double> apc(N), hp(N), nn(N);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < N; ++i) {
      const cd h = happly(c, c->lap[i], c->psi[i], c->pot4[i], c->uimp[i]);
      const cd ps = c->psi[i];
      const cd hps = c->cfg.time_mode == EP_REAL_TIME ? cd(-h.imag(), h.real()) : -h;
      hp[i] = (std::conj(ps) * hps).real();
      nn[i] = std::norm(ps);
      const cd p5 = 0.125 * (9.0 * po3[i] - po2[i] + f * (h + 2.0 * h1[i] - h2[i]));
      c->pc[i] = c->pc[i] - p5;
      c->psi[i] = p5 + c9 * c->pc[i];
      apc[i] = std::abs(c->pc[i]);
      c->den[i] = std::norm(c->psi[i]);
    }
    errHe = c9 * par_sum(N, [&](size_t i) { return apc[i]; }) / (double)N;
    const double hsum = par_sum(N, [&](size_t i) { return hp[i]; });
    const double nsum = par_sum(N, [&](size_t i) { return nn[i]; });
    c->last_mu = hsum / nsum;
    const int t = c->ioldp[2];
    c->ioldp[2] = c->ioldp[1]; c->ioldp[1] = c->ioldp[0]; c->ioldp[0] = t;
  }
  double errimp = 0, errvimp = 0, erriv = 0;
  if (mov) {
    double auxr[3];
    int r2 = c->ioldr[1], r3 = c->ioldr[2];
    int v1 = c->ioldv[0], v2 = c->ioldv[1], v3 = c->ioldv[2];
    int a1 = c->iolda[0], a2 = c->iolda[1];
    for (int k = 0; k < 3; ++k)
      auxr[k] = 0.125 * (9.0 * c->rimpold[k][r3] - c->rimpold[k][r2] +
                         3.0 * deltat * (c->vimpold[k][v3] + 2.0 * c->vimp[k] - c->vimpold[k][v1]));
    for (int k = 0; k < 3; ++k) {
      c->pcr[k] = c->pcr[k] - auxr[k];
      c->rimp[k] = auxr[k] + c9 * c->pcr[k];
      errimp += std::fabs(c9 * c->pcr[k]);
    }
    errimp *= 0.3333333333;
    { int t = c->ioldr[2]; c->ioldr[2] = c->ioldr[1]; c->ioldr[1] = c->ioldr[0]; c->ioldr[0] = t; }
    for (int k = 0; k < 3; ++k)
      auxr[k] = 0.125 * (9.0 * c->vimp[k] - c->vimpold[k][v2] +
                         3.0 * deltat * (c->aimp[k] + 2.0 * c->aimpold[k][a1] - c->aimpold[k][a2]));
    for (int k = 0; k < 3; ++k) {
      c->pcv[k] = c->pcv[k] - auxr[k];
      c->vimpold[k][v3] = c->vimp[k];
      c->vimp[k] = auxr[k] + c9 * c->pcv[k];
      errvimp += std::fabs(c9 * c->pcv[k]);
    }
    errvimp *= 0.3333333333;
    if (!c->cfg.fix_lambda) {
      cd auxc[10];
      int i3 = c->ioldiv[2], i2 = c->ioldiv[1], h1 = c->ioldhiv[0], h2 = c->ioldhiv[1];
      for (int k = 0; k < 10; ++k)
        auxc[k] = 0.125 * (9.0 * c->invarold[k][i3] - c->invarold[k][i2] +
                           3.0 * deltat * (c->hinvar[k] + 2.0 * c->hinvarold[k][h1] - c->hinvarold[k][h2]));
      // steppc.f90:199-217: the P state corrects components 1-6 and zeroes
      // 7-10; the D state corrects all ten
      const int nc = c->cfg.state == EP_STATE_D ? 10 : 6;
      for (int k = 0; k < nc; ++k) c->pciv[k] = c->pciv[k] - auxc[k];
      for (int k = 0; k < 10; ++k) c->invar[k] = cd(0);
      for (int k = 0; k < nc; ++k) c->invar[k] = auxc[k] + c9 * c->pciv[k];
      for (int k = 0; k < nc; ++k) erriv += std::abs(c9 * c->pciv[k]);
      erriv *= nc == 10 ? 0.1 : 0.1666666666666;
    }
    { int t = c->ioldv[2]; c->ioldv[2] = c->ioldv[1]; c->ioldv[1] = c->ioldv[0]; c->ioldv[0] = t; }
    { int t = c->ioldiv[2]; c->ioldiv[2] = c->ioldiv[1]; c->ioldiv[1] = c->ioldiv[0]; c->ioldiv[0] = t; }
  }
  if (err) { err->errHe = errHe; err->errimp = errimp; err->errvimp = errvimp; err->erriv = erriv; }
  if (!std::isfinite(errHe)) return fail(c, EP_ERR_NONFINITE, "steppc: non-finite corrector error");
  return EP_OK;
}

// Imaginary-time renormalisation: psi <- s psi, den <- |psi|^2 with
// s = sqrt(n4 / int|psi|^2); the multistep history (psiold, hpsiold, pc) is
// scaled by the same s so that it keeps describing one trajectory.
int oc_renormalize(oc_ctx* c, double* norm_before) {
  if (!c) return EP_ERR_INVALID_ARG;
  const double nrm = par_sum(c->N, [&](size_t i) { return std::norm(c->psi[i]); }) * c->dxyz;
  if (!(nrm > 0) || !std::isfinite(nrm)) return fail(c, EP_ERR_NONFINITE, "renormalize: bad norm");
  const double s = std::sqrt(c->cfg.n4 / nrm);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)c->N; ++i) {
    c->psi[i] *= s;
    c->den[i] = std::norm(c->psi[i]);
    for (int k = 0; k < 3; ++k) c->psiold[k][i] *= s;
    for (int k = 0; k < 2; ++k) c->hpsiold[k][i] *= s;
    c->pc[i] *= s;
  }
  c->last_norm = nrm;
  if (norm_before) *norm_before = nrm;
  return EP_OK;
}

int oc_run(oc_ctx* c, int nsteps, double deltat, ep_run_stats* st) {
  if (!c || nsteps < 0) return EP_ERR_INVALID_ARG;
  ep_step_errors e{};
  for (int s = 0; s < nsteps; ++s) {
    int r = oc_steppc(c, deltat, &e);
    if (r) return r;
    if (c->cfg.time_mode == EP_IMAGINARY_TIME && c->cfg.renormalize) {
      r = oc_renormalize(c, nullptr);
      if (r) return r;
    }
  }
  if (st) {
    st->errHe = e.errHe;
    st->mu = c->last_mu;
    st->norm = c->last_norm;
    st->steps_done = nsteps;
  }
  return EP_OK;
}

}  // extern "C"
