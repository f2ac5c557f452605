// ep_instates.h - the internal variables of instates.f90 (default branch).
// P state (Lstate 'P'): the 6x6 matrix V + (Als/2) SO over
// (p_x up, p_x down, p_y up, p_y down, p_z up, p_z down) built from the
// density-weighted moments of the impurity field (instates.f90:123-193), its
// eigenvectors in ascending order of the eigenvalues, and the state
//   invar = (v_il + v_il+1) / sqrt(2),  il = 2 * instate (0-based)
// (instates.f90:356-362).  The eigenvalues come in Kramers pairs; any
// orthonormal basis of a pair gives the same energies and impurity field
// (time-reversal-even operators have no matrix elements between Kramers
// partners), so this solver's basis need not be EISPACK's.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "../ep_dstate.h"

namespace instates {

typedef std::complex<double> cd;

// Eigen-decomposition of a Hermitian n x n matrix (row-major a) by cyclic
// complex Jacobi rotations: w ascending, column k of v (v[i*n+k]) its vector.
inline void hermitian_eigen(int n, std::vector<cd> a, std::vector<double>& w, std::vector<cd>& v) {
  v.assign((size_t)n * n, cd(0));
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  auto A = [&](int i, int j) -> cd& { return a[(size_t)i * n + j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, diag = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) (i == j ? diag : off) += std::norm(A(i, j));
    if (off <= 1e-30 * (diag + off) || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const cd b = A(p, q);
        const double beta = std::abs(b);
        if (beta == 0.0) continue;
        // U = diag(1, e^{-i phi}) R, R the real rotation zeroing [[a,beta],[beta,d]]
        const cd e = b / beta;  // e^{i phi}
        const double theta = (A(q, q).real() - A(p, p).real()) / (2.0 * beta);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        const cd upp = c, upq = s, uqp = -s * std::conj(e), uqq = c * std::conj(e);
        for (int k = 0; k < n; ++k) {  // A <- A U
          const cd akp = A(k, p), akq = A(k, q);
          A(k, p) = akp * upp + akq * uqp;
          A(k, q) = akp * upq + akq * uqq;
        }
        for (int k = 0; k < n; ++k) {  // A <- U^H A
          const cd apk = A(p, k), aqk = A(q, k);
          A(p, k) = std::conj(upp) * apk + std::conj(uqp) * aqk;
          A(q, k) = std::conj(upq) * apk + std::conj(uqq) * aqk;
        }
        A(p, q) = A(q, p) = 0.0;
        for (int k = 0; k < n; ++k) {  // V <- V U
          cd& vkp = v[(size_t)k * n + p];
          cd& vkq = v[(size_t)k * n + q];
          const cd x = vkp, y = vkq;
          vkp = x * upp + y * uqp;
          vkq = x * upq + y * uqq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int i, int j) { return A(i, i).real() < A(j, j).real(); });
  std::vector<cd> vs((size_t)n * n);
  w.resize(n);
  for (int k = 0; k < n; ++k) {
    w[k] = A(idx[k], idx[k]).real();
    for (int i = 0; i < n; ++i) vs[(size_t)i * n + k] = v[(size_t)i * n + idx[k]];
  }
  v.swap(vs);
}

// V + (Als/2) SO of instates.f90:150-193 from m = (Vx, Vy, Vz, Vxy, Vxz, Vyz).
inline std::vector<cd> p_matrix(const double* m, double als) {
  const cd I(0.0, 1.0);
  std::vector<cd> M(36, cd(0));
  auto at = [&](int i, int j) -> cd& { return M[(size_t)(i - 1) * 6 + (j - 1)]; };
  at(1, 1) = at(2, 2) = m[0];
  at(3, 3) = at(4, 4) = m[1];
  at(5, 5) = at(6, 6) = m[2];
  at(1, 3) = at(2, 4) = at(3, 1) = at(4, 2) = m[3];
  at(1, 5) = at(2, 6) = at(5, 1) = at(6, 2) = m[4];
  at(3, 5) = at(4, 6) = at(5, 3) = at(6, 4) = m[5];
  const double h = 0.5 * als;
  at(1, 3) += -I * h;
  at(2, 4) += I * h;
  at(2, 5) += -1.0 * h;
  at(1, 6) += 1.0 * h;
  at(4, 5) += -I * h;
  at(3, 6) += -I * h;
  at(3, 1) += I * h;
  at(4, 2) += -I * h;
  at(5, 2) += -1.0 * h;
  at(6, 1) += 1.0 * h;
  at(5, 4) += I * h;
  at(6, 3) += I * h;
  return M;
}

// invar (10 complex as 20 doubles) for a P state instate 0..2.
inline void p_state(const double* moments, double als, int instate, double* invar) {
  std::vector<double> w;
  std::vector<cd> v;
  hermitian_eigen(6, p_matrix(moments, als), w, v);
  const int il = 2 * instate, il1 = il + 1;
  const double r = 1.0 / std::sqrt(2.0);
  for (int i = 0; i < 10; ++i) invar[2 * i] = invar[2 * i + 1] = 0.0;
  for (int i = 0; i < 6; ++i) {
    const cd z = r * v[(size_t)i * 6 + il] + r * v[(size_t)i * 6 + il1];
    invar[2 * i] = z.real();
    invar[2 * i + 1] = z.imag();
  }
}

// D state (instates.f90:440-612, default branch :642-647): MatDSO over the
// ten internal variables from the 5x5 density-weighted field matrix M
// (ep_impurity_matrix_d), its eigenvectors ascending, and
//   invar = (v_il + v_il+1) / sqrt(2),  il = 2 * instate (0-based, instate 0..4).
// Kramers pairs again make the choice of basis inside a pair immaterial.
inline void d_state(const double* M, double als_d, int instate, double* invar) {
  cd S[10][10];
  dstate::sod(S);
  std::vector<cd> A(100);
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) A[(size_t)i * 10 + j] = dstate::matdso(M, S, als_d, i, j);
  std::vector<double> w;
  std::vector<cd> v;
  hermitian_eigen(10, A, w, v);
  const int il = 2 * instate, il1 = il + 1;
  const double r = 1.0 / std::sqrt(2.0);
  for (int i = 0; i < 10; ++i) {
    const cd z = r * v[(size_t)i * 10 + il] + r * v[(size_t)i * 10 + il1];
    invar[2 * i] = z.real();
    invar[2 * i + 1] = z.imag();
  }
}

}  // namespace instates
