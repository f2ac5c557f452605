// ep_pairpot.h - the He-X pair potentials of the Select_Pot subset this
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

// Select_Pot for kind (EP_POT_*), its cutoff rule r < r_cutoff -> umax and
// parameters p0..p2 (Morse: De, re, alpha; Koutselos: the ion code).
EP_PP_HD double ep_pair_potential(int kind, double r_cutoff, double umax, double p0, double p1, double p2,
                                  double r) {
  if (kind == EP_POT_NULL) return 0.0;
  if (r < r_cutoff) return umax;
  if (kind == EP_POT_MORSE) {
    const double e = exp(-p2 * (r - p1));
    return p0 * (e * e - 2.0 * e);
  }
  if (kind == EP_POT_KOUTSELOS) return ep_koutselos((int)p0, r);
  return 0.0;
}
