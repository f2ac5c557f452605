// ep_dstate.h - host-side algebra of the D-state internal variables shared by
// the engine (potinvar, energy) and the driver (instates).
#pragma once
#include <cmath>
#include <complex>

namespace dstate {

typedef std::complex<double> cd;

// Spin-orbit matrix SOD over the ten internal variables (potenimp.f90:
// 429-451, instates.f90:549-571): the upper triangle as the reference lists
// it, the lower one its conjugate.  It is 2 L.S of l = 2, s = 1/2:
// eigenvalues 2 (j = 5/2, six states) and -3 (j = 3/2, four states).
inline void sod(cd (&S)[10][10]) {
  const cd uim(0.0, 1.0);
  const double sqr3 = std::sqrt(3.0);
  for (auto& row : S)
    for (auto& v : row) v = 0.0;
  S[0][3] = 1.0;  S[0][7] = -uim;  S[0][8] = 2.0 * uim;
  S[1][2] = -1.0; S[1][6] = -uim;  S[1][9] = -2.0 * uim;
  S[2][5] = -uim * sqr3; S[2][6] = uim; S[2][9] = -uim;
  S[3][4] = -uim * sqr3; S[3][7] = -uim; S[3][8] = -uim;
  S[4][7] = -sqr3; S[5][6] = sqr3; S[6][9] = -1.0; S[7][8] = 1.0;
  for (int i = 0; i < 10; ++i)
    for (int j = i; j < 10; ++j) S[j][i] = std::conj(S[i][j]);
}

// MatDSO = M (x) 1_2 + (als/2) SOD (potenimp.f90:405-469): element (i, j),
// M the 5x5 density-weighted field matrix (row-major).
inline cd matdso(const double* M, const cd (&S)[10][10], double als, int i, int j) {
  const double md = ((i & 1) == (j & 1)) ? M[5 * (i / 2) + j / 2] : 0.0;
  return md + 0.5 * als * S[i][j];
}

}  // namespace dstate
