// ep_kernels_impl.cuh - bodies of the point-wise and reduction kernels.
#pragma once
#include "ep_kernels.cuh"
#include "ep_pairpot.h"

// Grid coordinate -xmax + h*i without contraction (x(i) of DFT4He3d.f90:248-256).
EP_DEV double coord(double xmax, double h, int i) { return __dadd_rn(-xmax, __dmul_rn(h, (double)i)); }

// |x - r_imp|^2 in potenimp.f90's order (zt = z^2, yt = y^2 + zt, x^2 + yt)
// without contraction: the table index int(1.5 + r/h) of update() then falls
// on the same side of a node as in an uncontracted FP64 evaluation (an FMA
// here moves r by an ulp, and where r/h sits on a node the parabola switches
// to the neighbouring three table points, a 1e-9 relative change of u_imp).
EP_DEV double rr2_nc(double xx, double yy, double zz) {
  return __dadd_rn(__dmul_rn(xx, xx), __dadd_rn(__dmul_rn(yy, yy), __dmul_rn(zz, zz)));
}

EP_DEV void idx3(const Geo& g, long long p, int& ix, int& iy, int& iz) {
  ix = (int)(p % g.nx);
  const long long r = p / g.nx;
  iy = (int)(r % g.ny);
  iz = (int)(r / g.ny);
}

// Parabolic interpolation in f(0:nint+1), the update() function of
// potenimp.f90:588-632, restated.
EP_DEV double interp_update(double r, int nint, double rmax, const double* __restrict__ f) {
  const double h = rmax / (nint - 1);
  const double c1oh = 1.0 / h;
  const double c1o2h2 = c1oh * c1oh * 0.5;
  int i0 = (int)(1.5 + r / h);
  i0 = min(max(i0, 1), nint);
  const double r0 = (i0 - 1) * h;
  const double f0 = f[i0];
  const bool lo = r < r0;
  const double f1 = f[lo ? i0 - 1 : i0 + 1];
  const double f2 = f[lo ? i0 + 1 : i0 - 1];
  const double aa = (f2 - 2.0 * f0 + f1) * c1o2h2;
  const double bb = ((lo ? f2 : f1) - f0) * c1oh - aa * (2.0 * r0 + h);
  const double cc = f0 - r0 * (bb + r0 * aa);
  return r * (aa * r + bb) + cc;
}

// Pair potential of the U+ integral (Select_Pot subset + Morse).
EP_DEV double pot_eval(const PotDev& v, double r) {
  return ep_pair_potential(v.kind, v.r_cutoff, v.umax, v.par, &v.s, r);
}

template <class T>
__global__ void k_potenimp(Geo g, double xmax, double ymax, double zmax, double hx, double hy, double hz,
                           double r0, double r1, double r2, const double* __restrict__ potpi,
                           const double* __restrict__ potdel, int npot, double rmax, double umax_sigma,
                           double2 iv0, double2 iv1, double2 iv2, double2 iv3, double2 iv4, double2 iv5,
                           T* __restrict__ vpi, T* __restrict__ delta, T* __restrict__ uimp) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N; p += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    idx3(g, p, ix, iy, iz);
    const double xx = coord(xmax, hx, ix) - r0;
    const double yy = coord(ymax, hy, iy) - r1;
    const double zz = coord(zmax, hz, iz) - r2;
    const double rr2 = rr2_nc(xx, yy, zz);
    const double r = sqrt(rr2);
    const double vp = interp_update(r, npot, rmax, potpi);
    const double dl = r > 1e-3 ? interp_update(r, npot, rmax, potdel) / rr2 : umax_sigma;
    const double ox = iv0.x * xx + iv2.x * yy + iv4.x * zz, oy = iv0.y * xx + iv2.y * yy + iv4.y * zz;
    const double ex = iv1.x * xx + iv3.x * yy + iv5.x * zz, ey = iv1.y * xx + iv3.y * yy + iv5.y * zz;
    const double u = vp + dl * ((ox * ox + oy * oy) + (ex * ex + ey * ey));
    vpi[p] = (T)vp;
    delta[p] = (T)dl;
    uimp[p] = (T)fmin(u, 1000.0);
  }
}

// D-state angular factors at x = r - rimp (potenimp.f90:68-117): the d
// harmonics a = (d1..d5) and the upper triangle of P in DGram's order.
EP_DEV void dstate_factors(double xx, double yy, double zz, double (&a)[5], double (&P)[15]) {
  const double sqr3 = sqrt(3.0), sqr3o2 = sqrt(3.0) / 2.0, insqr3 = 1.0 / sqrt(3.0), in3 = 1.0 / 3.0;
  const double d0 = xx * xx + yy * yy + zz * zz;
  const double d1 = sqr3 * xx * yy, d2 = sqr3 * yy * zz, d3 = (-xx * xx - yy * yy + 2.0 * zz * zz) / 2.0;
  const double d4 = sqr3 * xx * zz, d5 = sqr3o2 * (xx * xx - yy * yy);
  a[0] = d1; a[1] = d2; a[2] = d3; a[3] = d4; a[4] = d5;
  const double sd1 = d1 * d1, sd2 = d2 * d2, sd4 = d4 * d4, sd5 = d5 * d5;
  const double s35 = d3 + insqr3 * d5, f35 = d3 - insqr3 * d5;
  P[0] = in3 * (sd2 + sd4 + 4.0 * sd5);                 // (1,1)
  P[1] = -4.0 * in3 * d1 * d2 + insqr3 * d4 * d0;       // (1,2)
  P[2] = -2.0 * insqr3 * d2 * d4;                       // (1,3)
  P[3] = -4.0 * in3 * d1 * d4 + insqr3 * d2 * d0;       // (1,4)
  P[4] = -4.0 * in3 * d1 * d5;                          // (1,5)
  P[5] = in3 * (sd1 + sd4) + s35 * s35;                 // (2,2)
  P[6] = insqr3 * d1 * d4 - d2 * s35;                   // (2,3)
  P[7] = -4.0 * in3 * d2 * d4 + insqr3 * d1 * d0;       // (2,4)
  P[8] = -d1 * d4 - insqr3 * d2 * s35;                  // (2,5)
  P[9] = sd4 + sd2;                                     // (3,3)
  P[10] = insqr3 * d1 * d2 - d4 * f35;                  // (3,4)
  P[11] = insqr3 * (sd2 - sd4);                         // (3,5)
  P[12] = in3 * (sd1 + sd2) + f35 * f35;                // (4,4)
  P[13] = d1 * d2 + insqr3 * d4 * f35;                  // (4,5)
  P[14] = in3 * (sd2 + sd4 + 4.0 * sd1);                // (5,5)
}

template <class T>
__global__ void k_potenimp_d(Geo g, double xmax, double ymax, double zmax, double hx, double hy, double hz,
                             double r0, double r1, double r2, const double* __restrict__ potdel,
                             const double* __restrict__ potpidel, const double* __restrict__ potsigdel, int npot,
                             double rmax, double umax_pi, double umax_sigma, const __grid_constant__ DGram G,
                             T* __restrict__ delta, T* __restrict__ pidel, T* __restrict__ sigdel,
                             T* __restrict__ uimp) {
  const double gtr = G.g[0] + G.g[5] + G.g[9] + G.g[12] + G.g[14];
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N; p += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    idx3(g, p, ix, iy, iz);
    const double xx = coord(xmax, hx, ix) - r0;
    const double yy = coord(ymax, hy, iy) - r1;
    const double zz = coord(zmax, hz, iz) - r2;
    const double rr2 = rr2_nc(xx, yy, zz);
    const double r4 = rr2 * rr2;
    const double r = sqrt(rr2);
    const double dl = interp_update(r, npot, rmax, potdel);
    double pd = umax_pi, sd = umax_sigma;
    if (r > 1e-3) {
      pd = interp_update(r, npot, rmax, potpidel) / r4;
      sd = interp_update(r, npot, rmax, potsigdel) / r4;
    }
    double a[5], P[15];
    dstate_factors(xx, yy, zz, a, P);
    double qs = 0.0, qp = 0.0;
    int k = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
      for (int j = i; j < 5; ++j, ++k) {
        qs += a[i] * a[j] * G.g[k];
        qp += P[k] * G.g[k];
      }
    const double u = dl * gtr + pd * qs + sd * qp;
    delta[p] = (T)dl;
    pidel[p] = (T)pd;
    sigdel[p] = (T)sd;
    uimp[p] = (T)fmin(u, 1000.0);
  }
}

template <class T>
__global__ void k_impmoments_d(Geo g, const T* __restrict__ den, const T* __restrict__ dxd,
                               const T* __restrict__ dyd, const T* __restrict__ dzd, const T* __restrict__ uimp,
                               const T* __restrict__ delta, const T* __restrict__ pidel,
                               const T* __restrict__ sigdel, double xmax, double ymax, double zmax, double hx,
                               double hy, double hz, double r0, double r1, double r2, int izlo, int izhi,
                               double* __restrict__ partials) {
  Acc<double> acc[18];
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N; p += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    idx3(g, p, ix, iy, iz);
    const double u = dbl(uimp[p]);
    acc[0].add((double)dxd[p] * u);
    acc[1].add((double)dyd[p] * u);
    if (iz >= izlo && iz < izhi) acc[2].add((double)dzd[p] * u);
    const double xx = coord(xmax, hx, ix) - r0, yy = coord(ymax, hy, iy) - r1, zz = coord(zmax, hz, iz) - r2;
    const double rho = dbl(den[p]);
    const double dvd = (double)delta[p] * rho, dv1 = (double)pidel[p] * rho, dv2 = (double)sigdel[p] * rho;
    double a[5], P[15];
    dstate_factors(xx, yy, zz, a, P);
    int k = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
      for (int j = i; j < 5; ++j, ++k) acc[3 + k].add(P[k] * dv2 + a[i] * a[j] * dv1 + (i == j ? dvd : 0.0));
  }
  block_reduce_store_acc<18>(acc, partials);
}

// FP32 engine, P state: the impurity field in FP32 arithmetic (float tables,
// 1/h and the coordinates rounded once; a double per point would run on the
// FP64 pipe at 1/64 of the FP32 rate).  update() (potenimp.f90:588-632)
// evaluates, in both of its branches, the parabola through f(i0-1), f(i0),
// f(i0+1); here it is evaluated about r0 = (i0-1) h, which avoids the
// cancellation of its global coefficients in FP32.
EP_DEV float interp_update_f(float r, int nint, float h, float rh, const float* __restrict__ f) {
  int i0 = (int)(1.5f + r * rh);
  i0 = min(max(i0, 1), nint);
  const float r0 = (float)(i0 - 1) * h;
  const float fm = f[i0 - 1], f0 = f[i0], fp = f[i0 + 1];
  const float aa = (fp - 2.0f * f0 + fm) * (0.5f * rh * rh);
  const float b = (fp - f0) * rh - aa * h;
  const float d = r - r0;
  return f0 + d * (b + aa * d);
}

static __global__ void k_potenimp_f(Geo g, float xmax, float ymax, float zmax, float hx, float hy, float hz, float r0,
                             float r1, float r2, const float* __restrict__ potpi, const float* __restrict__ potdel,
                             int npot, float h, float rh, float umax_sigma, float2 iv0, float2 iv1, float2 iv2,
                             float2 iv3, float2 iv4, float2 iv5, float* __restrict__ vpi, float* __restrict__ delta,
                             float* __restrict__ uimp) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N; p += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    idx3(g, p, ix, iy, iz);
    const float xx = ((float)ix * hx - xmax) - r0;
    const float yy = ((float)iy * hy - ymax) - r1;
    const float zz = ((float)iz * hz - zmax) - r2;
    const float rr2 = xx * xx + (yy * yy + zz * zz);
    const float r = sqrtf(rr2);
    const float vp = interp_update_f(r, npot, h, rh, potpi);
    const float dl = r > 1e-3f ? interp_update_f(r, npot, h, rh, potdel) / rr2 : umax_sigma;
    const float ox = iv0.x * xx + iv2.x * yy + iv4.x * zz, oy = iv0.y * xx + iv2.y * yy + iv4.y * zz;
    const float ex = iv1.x * xx + iv3.x * yy + iv5.x * zz, ey = iv1.y * xx + iv3.y * yy + iv5.y * zz;
    const float u = vp + dl * ((ox * ox + oy * oy) + (ex * ex + ey * ey));
    vpi[p] = vp;
    delta[p] = dl;
    uimp[p] = fminf(u, 1000.0f);
  }
}

// FP32 engine, P state: forceimp sums and the six moments in compensated
// FP32 per thread, FP64 across threads and blocks.
static __global__ void k_impmoments_f(Geo g, const float* __restrict__ den, const float* __restrict__ dxd,
                               const float* __restrict__ dyd, const float* __restrict__ dzd,
                               const float* __restrict__ uimp, const float* __restrict__ vpi,
                               const float* __restrict__ delta, float xmax, float ymax, float zmax, float hx, float hy,
                               float hz, float r0, float r1, float r2, int izlo, int izhi,
                               double* __restrict__ partials) {
  Acc<float> acc[9];
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N; p += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    idx3(g, p, ix, iy, iz);
    const float u = uimp[p];
    acc[0].add(dxd[p] * u);
    acc[1].add(dyd[p] * u);
    if (iz >= izlo && iz < izhi) acc[2].add(dzd[p] * u);
    const float xx = ((float)ix * hx - xmax) - r0, yy = ((float)iy * hy - ymax) - r1,
                zz = ((float)iz * hz - zmax) - r2;
    const float a1 = den[p], a2 = delta[p], a3 = vpi[p];
    acc[3].add(a1 * (a2 * xx * xx + a3));
    acc[4].add(a1 * a2 * xx * yy);
    acc[5].add(a1 * a2 * xx * zz);
    acc[6].add(a1 * (a2 * yy * yy + a3));
    acc[7].add(a1 * a2 * yy * zz);
    acc[8].add(a1 * (a2 * zz * zz + a3));
  }
  block_reduce_store_acc<9>(acc, partials);
}

// Sum of |psi|^2 (block partials).
template <class T>
__global__ void k_normsum(const C2<T>* __restrict__ psi, long long N, double* __restrict__ partials) {
  Acc<double> acc[1];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const C2<T> v = psi[i];
    acc[0].add(dbl(v.x) * dbl(v.x) + dbl(v.y) * dbl(v.y));
  }
  block_reduce_store_acc<1>(acc, partials);
}

// Complex first derivative from global memory.
template <class T>
EP_DEV C2<T> d1c_global(const C2<T>* __restrict__ f, long long p, int i, int n, long long st, const T* w, int R,
                        int periodic) {
  C2<T> s = cmk<T>(T(0), T(0));
  for (int k = 1; k <= R; ++k) {
    int ip = i + k, im = i - k;
    C2<T> fp, fm;
    if (ip >= n) fp = periodic ? f[p + (long long)(ip - n - i) * st] : cmk<T>(T(0), T(0));
    else fp = f[p + (long long)k * st];
    if (im < 0) fm = periodic ? f[p + (long long)(im + n - i) * st] : cmk<T>(T(0), T(0));
    else fm = f[p - (long long)k * st];
    s = s + w[k] * (fp - fm);
  }
  return s;
}

template <class T>
__global__ void k_energy(Geo g, FdW<T> fd, Phys ph, const C2<T>* __restrict__ psi, const T* __restrict__ den,
                         const T* __restrict__ dencg, const T* __restrict__ delj4, const T* __restrict__ falfs,
                         const T* __restrict__ dxd, const T* __restrict__ dyd, const T* __restrict__ dzd,
                         const T* __restrict__ ix_, const T* __restrict__ iy_, const T* __restrict__ iz_,
                         const T* __restrict__ uimp, double xmax, double ymax, double zmax, double hx, double hy,
                         double hz, double r0, double r1, double r2, double zexc, const __grid_constant__ PotDev vplus,
                         int impurity, double* __restrict__ partials) {
  Acc<double> acc[8];
  const bool otc = ph.core == 1;
  const double aux1 = 0.5 * ph.cp4, aux2 = (1.0 / 3.0) * ph.cpp4;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N; p += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    idx3(g, p, ix, iy, iz);
    const C2<T> dx = d1c_global(psi, p, ix, g.nx, 1, fd.w1[0], fd.R, fd.periodic);
    const C2<T> dy = d1c_global(psi, p, iy, g.ny, (long long)g.nx, fd.w1[1], fd.R, fd.periodic);
    const C2<T> dz = d1c_global(psi, p, iz, g.nz, (long long)g.nx * g.ny, fd.w1[2], fd.R, fd.periodic);
    const double dn = dbl(den[p]), cg = dbl(dencg[p]);
    acc[0].add((dbl(dx.x) * dbl(dx.x) + dbl(dx.y) * dbl(dx.y)) + (dbl(dy.x) * dbl(dy.x) + dbl(dy.y) * dbl(dy.y)) +
               (dbl(dz.x) * dbl(dz.x) + dbl(dz.y) * dbl(dz.y)));
    acc[1].add((double)delj4[p] * dn);
    acc[2].add(dn * (cg * cg) * (aux1 + aux2 * cg));
    if (otc)
      acc[3].add(dbl(falfs[p]) * (dbl(dxd[p]) * dbl(ix_[p]) + dbl(dyd[p]) * dbl(iy_[p]) + dbl(dzd[p]) * dbl(iz_[p])));
    acc[4].add(dn * (1.0 + tanh(ph.beta * (dn - ph.den_m))));
    if (impurity) {
      const double a = r0 - coord(xmax, hx, ix), b = r1 - coord(ymax, hy, iy), c = r2 - coord(zmax, hz, iz);
      const double r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c)));
      if (r >= zexc) {
        acc[5].add(dn * (double)uimp[p]);
        acc[6].add(dn * pot_eval(vplus, r));
      }
    }
    acc[7].add(dn);
  }
  block_reduce_store_acc<8>(acc, partials);
}

template <class T>
__global__ void k_impmoments(Geo g, const T* __restrict__ den, const T* __restrict__ dxd,
                             const T* __restrict__ dyd, const T* __restrict__ dzd, const T* __restrict__ uimp,
                             const T* __restrict__ vpi, const T* __restrict__ delta, double xmax, double ymax,
                             double zmax, double hx, double hy, double hz, double r0, double r1, double r2,
                             int izlo, int izhi, double* __restrict__ partials) {
  Acc<double> acc[9];
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N; p += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    idx3(g, p, ix, iy, iz);
    const double u = dbl(uimp[p]);
    acc[0].add((double)dxd[p] * u);
    acc[1].add((double)dyd[p] * u);
    if (iz >= izlo && iz < izhi) acc[2].add((double)dzd[p] * u);
    const double xx = coord(xmax, hx, ix) - r0, yy = coord(ymax, hy, iy) - r1, zz = coord(zmax, hz, iz) - r2;
    const double a1 = dbl(den[p]), a2 = dbl(delta[p]), a3 = dbl(vpi[p]);
    acc[3].add(a1 * (a2 * xx * xx + a3));
    acc[4].add(a1 * a2 * xx * yy);
    acc[5].add(a1 * a2 * xx * zz);
    acc[6].add(a1 * (a2 * yy * yy + a3));
    acc[7].add(a1 * a2 * yy * zz);
    acc[8].add(a1 * (a2 * zz * zz + a3));
  }
  block_reduce_store_acc<9>(acc, partials);
}

// ---------------------------------------------------------------------------
// Sine integral Si(x): power series for |x| <= 4, else the continued fraction
// of E1(ix) by the modified Lentz method (Numerical Recipes 6.9).
EP_DEV double si_dev(double x) {
  const double ax = fabs(x);
  double r;
  if (ax <= 4.0) {
    double term = ax, sum = ax;
    const double x2 = ax * ax;
    for (int k = 1; k < 60; ++k) {
      term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
      const double t = term / (2.0 * k + 1.0);
      sum += t;
      if (fabs(t) < 1e-18 * fabs(sum)) break;
    }
    r = sum;
  } else {
    double br = 1.0, bi = ax, cr = 1e300, ci = 0.0;
    double den = br * br + bi * bi;
    double dr = br / den, di = -bi / den;
    double hr = dr, hi = di;
    for (int i = 2; i < 1000; ++i) {
      const double a = -(double)(i - 1) * (double)(i - 1);
      br += 2.0;
      // d = 1/(a*d + b)
      const double tr = a * dr + br, ti = a * di + bi;
      den = tr * tr + ti * ti;
      dr = tr / den;
      di = -ti / den;
      // c = b + a/c
      const double cd = cr * cr + ci * ci;
      const double ncr = br + a * cr / cd, nci = bi - a * ci / cd;
      cr = ncr;
      ci = nci;
      const double er = cr * dr - ci * di, ei = cr * di + ci * dr;
      const double nhr = hr * er - hi * ei, nhi = hr * ei + hi * er;
      hr = nhr;
      hi = nhi;
      if (fabs(er - 1.0) + fabs(ei) < 3e-16) break;
    }
    double s, c;
    sincos(ax, &s, &c);
    // h *= (cos x - i sin x)
    const double fi = hi * c - hr * s;
    r = 1.5707963267948966192313216916397514 + fi;
  }
  return x < 0 ? -r : r;
}

EP_DEV double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// Integral of sin(a t)/t^11 and sin(a t)/t^5 from x to infinity, closed forms
// of fforma.f90:73-137 (integration by parts down to Si).
EP_DEV double sinint_tail(double a, double x) {
  const double res = si_dev(a * x);
  return a > 0.0 ? 1.5707963267948966192313216916397514 - res : 1.5707963267948966192313216916397514 + res;
}
EP_DEV double sinx11_dev(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double bd = 40320.0 - 720.0 * y2 + 24.0 * (y2 * y2) - 2.0 * (y2 * y2 * y2) + (y2 * y2 * y2 * y2);
  const double cd = 362880.0 - 5040.0 * y2 + 120.0 * (y2 * y2) - 6.0 * (y2 * y2 * y2) + (y2 * y2 * y2 * y2);
  double s, c;
  sincos(y, &s, &c);
  const double res1 = (a * bd * c + cd * s / x) / (3628800.0 * ipow(x, 9));
  const double res2 = -(ipow(a, 10) * sinint_tail(a, x)) / 3628800.0;
  return res1 + res2;
}
EP_DEV double sinx5_dev(double a, double x) {
  const double y = a * x, y2 = y * y;
  double s, c;
  sincos(y, &s, &c);
  const double res1 = -(a * (-2.0 + y2) * c + (-6.0 + y2) * s / x) / (24.0 * x * x * x);
  const double res2 = (ipow(a, 4) * sinint_tail(a, x)) / 24.0;
  return res1 + res2;
}
EP_DEV double intcore_dev(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double d0 = x / ipow(a, 5), e0 = 1.0 / ipow(a, 6);
  const double bd = -120.0 * d0 + 20.0 * (d0 * y2) - (d0 * y2 * y2);
  const double ce = 120.0 * e0 - 60.0 * (e0 * y2) + 5.0 * (e0 * y2 * y2);
  double s, c;
  sincos(y, &s, &c);
  return bd * c + ce * s;
}

template <class T>
__global__ void k_formfactors(Geo g, const double* __restrict__ px, const double* __restrict__ py,
                              const double* __restrict__ pz, int core, double h4, double eps, double sigma,
                              double bforce, double l, T* __restrict__ fvlj, T* __restrict__ wcgk,
                              T* __restrict__ kalfs) {
  const double pi = 3.14159265358979323846264338327950288;
  const double twopi = 2.0 * pi;
  const double sigma6 = ipow(sigma, 6), aux1 = 8.0 * eps, aux3 = sigma6 / ipow(h4, 6);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.Nh; q += (long long)gridDim.x * blockDim.x) {
    const int ipx = (int)(q % g.nxh);
    const long long r = q / g.nxh;
    const int ipy = (int)(r % g.ny), ipz = (int)(r / g.ny);
    const double a = px[ipx], b = py[ipy], c = pz[ipz];
    const double p = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c)));
    double fv;
    if (fabs(p) < 1e-10) {
      fv = bforce;
    } else {
      const double a2 = twopi * p;
      const double t1 = sinx11_dev(a2, h4), t2 = sinx5_dev(a2, h4);
      if (core == 2) {
        const double v0 = aux1 * aux3 * (aux3 - 1.0) / ipow(h4, 4);
        fv = (aux1 * sigma6 * (sigma6 * t1 - t2) + v0 * intcore_dev(a2, h4)) / p;
      } else {
        fv = (aux1 * sigma6 * (sigma6 * t1 - t2)) / p;
      }
    }
    double wc = 1.0;
    if (p > 0.0) {
      const double arg = twopi * p * h4;
      double s, cc;
      sincos(arg, &s, &cc);
      const double aux = s - arg * cc;
      wc = fabs(aux) < 1e-10 ? 1.0 : 3.0 * aux / (arg * arg * arg);
    }
    const double t = pi * l * p;
    fvlj[q] = (T)fv;
    wcgk[q] = (T)wc;
    kalfs[q] = (T)exp(-(t * t));
  }
}
