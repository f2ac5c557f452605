// ep_pairpot.h - the He-X pair potentials of the Select_Pot registry this
// library evaluates itself (V_impur.f90:87-932), for host and device code.
#pragma once
#include <math.h>

#include "../../include/eff_pot.h"

#if defined(__CUDACC__)
#define EP_PP_HD __host__ __device__ inline
#else
#define EP_PP_HD inline
#endif

// He-M+ of Koutselos, Mason and Viehland, J. Chem. Phys. 93, 7125 (1990), as
// V_Koutselos_*_plus_gs (V_impur.f90:1704-1883): an exchange term
// v0 (A e^{-a Rs} - B e^{-b Rs}), Rs = x / rho, plus the damped induction and
// dispersion series -(C4' / x^4 + C6' / x^6 + C8' / x^8) h(x) with
// Cn' = Cn + alpha_n / 2 (He polarisabilities) and h = exp(-(1.28 R_m / x -
// 1)^2) below x = 1.28 R_m, 1 above; x in bohr, result in K.
// ion: 0 Na+, 1 K+, 2 Rb+, 3 Cs+.
EP_PP_HD double ep_koutselos(int ion, double r_angstrom) {
  // per ion: v0, rho, R_m, C4, C6, C8 (atomic units)
  const double tab[4][6] = {{0.2063, 0.7640, 4.55, 0.0, 1.424, 13.17},
                            {0.2690, 0.8589, 5.49, 0.0, 5.83, 72.05},
                            {0.3474, 0.8868, 5.85, 0.0, 8.8, 126.2},
                            {0.5092, 0.9241, 6.38, 0.0, 13.69, 236.4}};
  const double a_bohr = 0.529177, hartree = 27.2114, ev_k = 11604.448;
  const double A = 146.98, a_a = 1.5024, B = 70.198, b_b = 1.4041;
  const double a_d = 1.3831, a_q = 2.4434, a_o = 10.614;
  const double* t = tab[ion < 0 ? 0 : (ion > 3 ? 3 : ion)];
  const double cc4 = t[3] + a_d / 2.0, cc6 = t[4] + a_q / 2.0, cc8 = t[5] + a_o / 2.0;
  const double x = r_angstrom / a_bohr;
  const double rs = x / t[1];
  const double vex = t[0] * (A * exp(-a_a * rs) - B * exp(-b_b * rs));
  const double aux = t[2] * 1.28;
  double h = 1.0;
  if (x < aux) {
    h = 0.0;
    if (x != 0.0) {
      const double q = aux / x - 1.0;
      h = exp(-(q * q));
    }
  }
  double v = vex;
  if (x != 0.0) {
    const double x2 = x * x, x4 = x2 * x2, x6 = x4 * x2, x8 = x6 * x2;
    v = v + ((-cc4 / x4 - cc6 / x6) - cc8 / x8) * h;
  }
  return v * hartree * ev_k;
}

// Patil's alkali-He potential, S. H. Patil, J. Chem. Phys. 94, 8089 (1991),
// as V_alka (V_impur.f90:1097-1192): an exchange term from the alkali's
// valence density at the He (asymptotic form agran d^(2u) (1 + v/d)^2
// e^(-2d/a), u = a - 1, v = -a^2 u / 2) times the He moments r2, r4, r6,
// minus the damped dispersion c6 f_9(d)/d^6 + c8 f_11(d)/d^8, f_m = 1 -
// e^(-d/abar) sum_{n<=m} (d/abar)^n/n!, abar = (a + b)/4; d in bohr, result
// in K.  atom: 0 Li, 1 Na, 2 K, 3 Rb, 4 Cs.
EP_PP_HD double ep_patil(int atom, double r_angstrom) {
  // per atom: a, c6, c8, agran (b = 0.744, r2 = 2.37, r4 = 7.78, r6 = 50.5 for all)
  const double tab[5][4] = {{1.588, 22.5, 1.06e3, 0.0519},
                            {1.627, 24.7, 1.29e3, 0.0450},
                            {1.771, 38.9, 2.66e3, 0.0259},
                            {1.805, 44.6, 3.18e3, 0.0226},
                            {1.869, 51.2, 4.34e3, 0.0173}};
  const double* t = tab[atom < 0 ? 0 : (atom > 4 ? 4 : atom)];
  const double a = t[0], b = 0.744, c6 = t[1], c8 = t[2], agran = t[3];
  const double r2 = 2.37, r4 = 7.78, r6 = 50.5;
  const double bohr = 0.529177249, factor = 11604.448 * 27.211608;
  const double pi = 4.0 * atan(1.0);
  const double d = r_angstrom / bohr;
  const double abar = (a + b) / 4.0, u = a - 1.0, v = -0.5 * (a * a) * u;
  const double q = 1.0 + v / d;
  const double roa = agran * pow(d, 2.0 * u) * (q * q) * exp(-2.0 * d / a);
  double f[2];
  for (int l = 1; l <= 2; ++l) {
    double sum = 0.0, term = 1.0, fact = 1.0;
    const double y = d / abar;
    for (int n = 0; n <= 2 * l + 7; ++n) {
      if (n >= 2) fact *= (double)n;
      sum += term / fact;
      term *= y;
    }
    f[l - 1] = 1.0 - sum * exp(-d / abar);
  }
  const double a2 = a * a, d2 = d * d, d6 = d2 * d2 * d2;
  const double vimp = 4.0 * pi / 3.0 * roa * (r2 + 37.0 / 90.0 * r4 / a2 + 28.0 / 525.0 * r6 / (a2 * a2)) -
                      c6 * f[0] / d6 - c8 * f[1] / (d6 * d2);
  return vimp * factor;
}

// He-He of Aziz et al. (HFD form), as V_Aziz_He (V_impur.f90:970-990):
// eps (A e^(-alpha x + beta x^2) - F(x) (C6/x^6 + C8/x^8 + C10/x^10)),
// x = r / rm, F = e^(-(D/x - 1)^2) for x <= D, 1 beyond.
EP_PP_HD double ep_aziz_he(double rr) {
  const double eps = 10.948, A = 1.8443101e5, alpha = 10.43329537, beta = -2.27965105, D = 1.4826;
  const double C6 = 1.36745214, C8 = 0.42123807, C10 = 0.17473318, rm = 2.963;
  const double x = rr / rm;
  if (x == 0.0) return A * eps;
  double ff = 1.0;
  if (x <= D) {
    const double q = D / x - 1.0;
    ff = exp(-(q * q));
  }
  const double x2 = x * x, x6 = x2 * x2 * x2, x8 = x6 * x2, x10 = x8 * x2;
  return (A * exp(-alpha * x + beta * x2) - ff * (C6 / x6 + C8 / x8 + C10 / x10)) * eps;
}

// Tang-Toennies rare-gas-He potential, K. T. Tang and J. P. Toennies,
// Z. Phys. D 1, 91 (1986), as V_Ar_He / V_Xe_He (V_impur.f90:2681-2782):
// A e^(-b x) - sum_{n=3..9} f_2n(b x) C_2n / x^2n, with the damping f_2n =
// 1 - e^(-bx) sum_{k<=2n} (bx)^k / k! and C_12.. from the recursion C_2n =
// (C_2n-2 / C_2n-4)^3 C_2n-6; x in bohr, result in K.  atom: 0 Ar, 1 Xe.
EP_PP_HD double ep_tang_toennies(int atom, double r) {
  const double tab[2][5] = {{75.8953, 2.0589, 9.7697, 152.8468, 3249.728},
                            {74.9002, 1.8175, 21.5674, 430.148, 10610.21}};
  const double* t = tab[atom <= 0 ? 0 : 1];
  const double AA = t[0], BB = t[1];
  const double rbohr = 0.5292, to_k = 27.21 * 11604.0;
  double B[18], C[7], S[18];
  B[0] = BB;
  for (int i = 1; i < 18; ++i) B[i] = B[i - 1] * BB / (double)(i + 1);
  C[0] = t[2];
  C[1] = t[3];
  C[2] = t[4];
  for (int i = 3; i < 7; ++i) {
    const double q = C[i - 1] / C[i - 2];
    C[i] = q * q * q * C[i - 3];
  }
  const double rr = r / rbohr;
  const double e = exp(-BB * rr);
  double p = rr;
  S[0] = B[0] * p;
  for (int i = 1; i < 18; ++i) {
    p = p * rr;
    S[i] = S[i - 1] + B[i] * p;
  }
  double v = AA * e;
  const double s1 = 1.0 / (rr * rr);
  double sp = s1 * s1 * s1;
  for (int i = 0; i < 7; ++i) {
    const int kmax = 2 * i + 5;  // S(2i + 6) of the 1-based recursion
    v = v + ((S[kmax] + 1.0) * e - 1.0) * C[i] * sp;
    sp = sp * s1;
  }
  return v * to_k;
}

// He-Ag (V_Ag_gs / V_Ag_Pi / V_Ag_Sig, V_impur.f90:1038-1096): an HFD form
// A e^(-alpha r - beta r^2) - F(r) (C6/r^6 + C8/r^8 + C10/r^10 + C12/r^12),
// F = e^(-(D/r - 1)^2) for r <= D, 1 beyond; r in A, V in K.  The constants
// the reference writes without an exponent letter are default REAL there
// and enter as binary32 values (the float literals below).
EP_PP_HD double ep_ag(int which, double r) {
  double A, al, be, D, C6, C8, C10, C12;
  if (which <= 0) {
    A = (double)78741.3877f; al = (double)0.65299f; be = (double)0.36367f; D = (double)12.093f;
    C6 = 137042.07; C8 = 189386.217; C10 = 111358462.0; C12 = 1.17670377e10;
  } else if (which == 1) {
    A = 0.7095092e6; al = (double)1.9928f; be = (double)0.45500f; D = (double)4.0562f;
    C6 = 0.21661134e6; C8 = (double)123454.7952f; C10 = 0.307155024e6; C12 = 0.740464032e-10;
  } else {
    A = (double)40005.2f; al = (double)0.41529f; be = (double)0.14888f; D = (double)25.730f;
    C6 = 1.97443e-9; C8 = 3.37393e-6; C10 = (double)0.00788363f; C12 = 7.52624e12;
  }
  if (r == 0.0) return A;
  double ff = 1.0;
  if (r <= D) {
    const double q = D / r - 1.0;
    ff = exp(-(q * q));
  }
  const double r2 = r * r, r6 = r2 * r2 * r2, r8 = r6 * r2, r10 = r8 * r2, r12 = r10 * r2;
  return A * exp(-al * r - be * r2) - ff * (C6 / r6 + C8 / r8 + C10 / r10 + C12 / r12);
}

// He-Ba of Lovallo's fit (V_Ba_gs, V_impur.f90:1197-1210): 1297.1 K up to
// 3.7 A, beyond it even inverse powers 6 .. 18, summed from the highest.
EP_PP_HD double ep_ba_gs(double x) {
  if (x <= 3.7) return 1297.1;
  const double x2 = x * x, x6 = x2 * x2 * x2, x8 = x6 * x2, x10 = x8 * x2, x12 = x10 * x2, x14 = x12 * x2,
               x16 = x14 * x2, x18 = x16 * x2;
  return -6.146426949008034e14 / x18 + 1.6797251118695925e14 / x16 - 1.6513058293510484e13 / x14 +
         7.015334514979032e11 / x12 - 1.1066880774828484e10 / x10 + 4.900282758445466e7 / x8 -
         450294.6878721156 / x6;
}

// He-CH3I, Legendre component l of the m = 0 ground-state potential
// (V_CH3I_l and radpot, V_impur.f90:3079-3243): a Morse function d (1 -
// e^(-b (x - c)))^2 - d in hartree of x in bohr, and its own cutoff (umax_l
// for r <= 3.6 A).  The Morse parameters and two cutoff radii are default
// REAL literals in the reference (binary32 values).
EP_PP_HD double ep_ch3i(int l, double r) {
  const float dd[5] = {0.000185445f, -4.51657e-05f, 2.53688e-05f, -6.51825e-06f, 1.5032e-06f};
  const float bb[5] = {0.782913f, 0.837569f, 0.849398f, 0.779254f, 0.787553f};
  const float cc[5] = {9.5243f, 10.3772f, 10.6988f, 11.454f, 12.236f};
  const double umax[5] = {3.1648655845e3, -5.1115736616e3, 5.5581502684e3, -2.7398540818e3, 2.4025334047e3};
  const double rcut[5] = {3.6, (double)3.6f, 3.6, 3.6, (double)3.6f};
  const int k = l < 0 ? 0 : (l > 4 ? 4 : l);
  if (r <= rcut[k]) return umax[k];
  const double a_bohr = 0.529177, hartree = 27.2114, ev_k = 11604.448;
  const double x = r / a_bohr;
  const double d = (double)dd[k], b = (double)bb[k], c = (double)cc[k];
  const double e = 1.0 - exp(-b * (x - c));
  return (d * (e * e) - d) * hartree * ev_k;
}

// The He-surface and adatom potentials of the registry (V_impur.f90:939-965,
// 2417-2554, 3013-3030), V in K of one distance z in A:
//   0 graphene (V_grafeno): (A e^(-alpha z) - C4/z^4 - C6/z^6) meV
//   1 graphene without dispersion: Morse D (1 - e^(-alpha (z - Ze)))^2 - D, meV
//   2 TiO2: Morse in cm^-1 plus -1/2 (1 + tanh((z - z0)/a) c3 (c3/z)^3)
//   3 Au (V_Au): -De (1 + sum_k a_k r^k) e^(-a1 r), r = z - Re (Horner form)
//   4, 5 Au on TiO2 and its z derivative: even inverse powers 6..14 in meV
//        (Horner in 1/z^2), a constant for z <= 2
//   6, 7 Ag on graphene and its derivative: (A e^(-beta z) - C4/z^4) kcal/mol
//   8, 9 Au on graphene and its derivative: the same form in meV
EP_PP_HD double ep_surface(int which, double z) {
  const double mev_k = 11.604448;
  switch (which) {
    case 0: {
      const double z2 = z * z;
      return (554811.0 * exp(-3.21193 * z) - 1531.83 / (z2 * z2) - 22259.0 / (z2 * z2 * z2)) * mev_k;
    }
    case 1: {
      const double D = 0.493191, e = 1.0 - exp(-1.54605 * (z - 4.34871));
      return (D * (e * e) - D) * mev_k;
    }
    case 2: {
      const double de = 95.9583, e = 1.0 - exp(-1.47089 * (z - 4.22534));
      const double vz = de * (e * e) - de;
      const double c3 = 8.85163, q = c3 / z;
      const double vzd = -0.5 * (1.0 + tanh((z - 4.77765) / 1.06161) * c3 * (q * q * q));
      return (vz + vzd) * 1.4387770;
    }
    case 3: {
      const double a1 = 1.6417, a2 = -0.6164, a3 = 0.3770, a4 = -0.0549, a5 = 0.0018, a6 = 0.0046, a7 = -0.0010,
                   a8 = 0.0001, a9 = 2.7e-6, Re = 4.124, De = 20.301143;
      const double r = z - Re;
      return -De * (1.0 + r * (a1 + r * (a2 + r * (a3 + r * (a4 + r * (a5 + r * (a6 + r * (a7 + r * (a8 + r * a9))))))))) *
             exp(-a1 * r);
    }
    case 4:
    case 5: {
      const double C6 = -4.18518e6, C8 = 6.54459e7, C10 = -3.73112e8, C12 = 9.44942e8, C14 = -8.97265e8;
      if (!(z > 2.0)) return (which == 4 ? 1821.44287109375 : -5415.35400390625) * mev_k;
      const double a = 1.0 / z, a2 = a * a;
      if (which == 4)
        return (((((C14 * a2 + C12) * a2 + C10) * a2 + C8) * a2 + C6) * (a2 * a2 * a2)) * mev_k;
      return (((((-14.0 * C14 * a2 - 12.0 * C12) * a2 - 10.0 * C10) * a2 - 8.0 * C8) * a2 - 6.0 * C6) *
              (a2 * a2 * a2 * a)) *
             mev_k;
    }
    case 6:
    case 7: {
      const double A = 11557.3, beta = 2.33671, C4 = 1143.0, kcal_k = 5.03216592455e2;
      const double z2 = z * z, z4 = z2 * z2;
      if (which == 6) return (A * exp(-beta * z) - C4 / z4) * kcal_k;
      return (-A * beta * exp(-beta * z) + 4.0 * C4 / (z4 * z)) * kcal_k;
    }
    default: {
      const double A = 448058.0, beta = 2.12336, C4 = 83077.3;
      const double z2 = z * z, z4 = z2 * z2;
      if (which == 8) return (A * exp(-beta * z) - C4 / z4) * mev_k;
      return (-A * beta * exp(-beta * z) + 4.0 * C4 / (z4 * z)) * mev_k;
    }
  }
}

// Double-double arithmetic (Knuth's two-sum, the fused-multiply-add product
// error, and the normalisations of Dekker's and Bailey's double-double
// algorithms): 106-bit sums for the Real*16 fits.
struct ep_dd {
  double hi, lo;
};
EP_PP_HD ep_dd ep_dd_quick(double a, double b) {  // |a| >= |b|
  const double s = a + b;
  return ep_dd{s, b - (s - a)};
}
EP_PP_HD ep_dd ep_dd_sum2(double a, double b) {
  const double s = a + b, bb = s - a;
  return ep_dd{s, (a - (s - bb)) + (b - bb)};
}
EP_PP_HD ep_dd ep_dd_add(ep_dd a, ep_dd b) {
  ep_dd s = ep_dd_sum2(a.hi, b.hi);
  const ep_dd t = ep_dd_sum2(a.lo, b.lo);
  s = ep_dd_quick(s.hi, s.lo + t.hi);
  return ep_dd_quick(s.hi, s.lo + t.lo);
}
EP_PP_HD ep_dd ep_dd_mul(ep_dd a, ep_dd b) {
  const double p = a.hi * b.hi;
  const double e = fma(a.hi, b.hi, -p) + (a.hi * b.lo + a.lo * b.hi);
  return ep_dd_quick(p, e);
}
EP_PP_HD ep_dd ep_dd_recip(double x) {
  const double q = 1.0 / x;
  const double rem = fma(-q, x, 1.0);  // exact
  return ep_dd_quick(q, rem / x);
}

// The inverse-power fit s at x (the Param_LJ_* functions of V_impur.f90,
// e.g. V_Fausto_Rb_gs :2206-2250): core constant, parabola, then the sum
// over k in ascending order with x^-(k0+1) advanced by one factor 1/x per
// term.
EP_PP_HD double ep_series_value(const ep_series* s, double x) {
  if (x <= s->r_core) return s->f_core;
  if (x <= s->r0) return fabs(s->aa * (x * x) + s->bb * x + s->cc);
  const int n = s->n < EP_SERIES_MAX ? s->n : EP_SERIES_MAX;
  if (s->quad) {
    const ep_dd xq = ep_dd_recip(x);
    ep_dd p = xq;
    for (int i = 0; i < s->k0; ++i) p = ep_dd_mul(p, xq);
    ep_dd acc{0.0, 0.0};
    for (int k = 0; k < n; ++k) {
      acc = ep_dd_add(acc, ep_dd_mul(ep_dd{s->c_hi[k], s->c_lo[k]}, p));
      p = ep_dd_mul(p, xq);
    }
    return acc.hi + acc.lo;
  }
  const double xq = 1.0 / x;
  double p = xq;
  for (int i = 0; i < s->k0; ++i) p = p * xq;
  double acc = 0.0;
  for (int k = 0; k < n; ++k) {
    acc = acc + s->c_hi[k] * p;
    p = p * xq;
  }
  return acc;
}

// Func_Ba_plus_gs (V_impur.f90:1479-1497): the plain parabola up to r0, then
// even inverse powers x^-6, x^-8, ... in double.
EP_PP_HD double ep_evenpow_value(const ep_series* s, double x) {
  if (x <= s->r0) return s->aa * (x * x) + s->bb * x + s->cc;
  const int n = s->n < EP_SERIES_MAX ? s->n : EP_SERIES_MAX;
  const double x2 = x * x;
  double p = x2 * x2 * x2, sto = 0.0;
  for (int k = 0; k < n; ++k) {
    sto = sto + s->c_hi[k] / p;
    p = p * x2;
  }
  return sto;
}

// V_Cs_7s (V_impur.f90:1682-1702): x clamped below at x0 (r_core), the plain
// parabola up to r0, then Pg(1) e^(-Ps(1) x)/x + sum_{k>=2} Pg(k) x^(k-1)
// e^(-Ps(k) x) (Pg in c_hi, Ps in c_lo).
EP_PP_HD double ep_expfit_value(const ep_series* s, double xx) {
  const double x = xx < s->r_core ? s->r_core : xx;
  if (x <= s->r0) return s->aa * (x * x) + s->bb * x + s->cc;
  const int n = s->n < EP_SERIES_MAX ? s->n : EP_SERIES_MAX;
  double sto = s->c_hi[0] * exp(-s->c_lo[0] * x) / x, p = 1.0;
  for (int k = 1; k < n; ++k) {
    p = p * x;
    sto = sto + s->c_hi[k] * p * exp(-s->c_lo[k] * x);
  }
  return sto;
}

// Select_Pot for kind (EP_POT_*), its cutoff rule r < r_cutoff -> umax,
// parameters par (Morse: De, re, alpha; Koutselos, Patil, Tang-Toennies:
// the atom) and, for EP_POT_SERIES, the fit s.
EP_PP_HD double ep_pair_potential(int kind, double r_cutoff, double umax, const double* par, const ep_series* s,
                                  double r) {
  if (kind == EP_POT_NULL) return 0.0;
  if (r < r_cutoff) return umax;
  if (kind == EP_POT_MORSE) {
    const double e = exp(-par[2] * (r - par[1]));
    return par[0] * (e * e - 2.0 * e);
  }
  if (kind == EP_POT_KOUTSELOS) return ep_koutselos((int)par[0], r);
  if (kind == EP_POT_PATIL) return ep_patil((int)par[0], r);
  if (kind == EP_POT_AZIZ) return ep_aziz_he(r);
  if (kind == EP_POT_TANG_TOENNIES) return ep_tang_toennies((int)par[0], r);
  if (kind == EP_POT_SERIES && s) return ep_series_value(s, r);
  if (kind == EP_POT_AG) return ep_ag((int)par[0], r);
  if (kind == EP_POT_BA_GS) return ep_ba_gs(r);
  if (kind == EP_POT_CH3I) return ep_ch3i((int)par[0], r);
  if (kind == EP_POT_SURFACE) return ep_surface((int)par[0], r);
  if (kind == EP_POT_EVENPOW && s) return ep_evenpow_value(s, r);
  if (kind == EP_POT_EXPFIT && s) return ep_expfit_value(s, r);
  return 0.0;
}
