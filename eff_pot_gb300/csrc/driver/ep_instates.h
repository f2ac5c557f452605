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
#include <string>
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

// Jz = Lz + Sz over the internal variables, as instates.f90 writes its
// matrix elements (P: :246-258, D: :632-651); row-major nd x nd.
inline std::vector<cd> jz_matrix(int nd) {
  const cd I(0.0, 1.0);
  std::vector<cd> J((size_t)nd * nd, cd(0));
  auto at = [&](int i, int j) -> cd& { return J[(size_t)(i - 1) * nd + (j - 1)]; };
  if (nd == 6) {
    at(1, 1) = 0.5; at(1, 3) = -I; at(2, 2) = -0.5; at(2, 4) = -I; at(3, 1) = I; at(3, 3) = 0.5;
    at(4, 2) = I; at(4, 4) = -0.5; at(5, 5) = 0.5; at(6, 6) = -0.5;
  } else {
    at(9, 9) = 0.5; at(9, 1) = -2.0 * I; at(10, 10) = -0.5; at(10, 2) = -2.0 * I; at(3, 3) = 0.5;
    at(3, 7) = I; at(4, 4) = -0.5; at(4, 8) = I; at(5, 5) = 0.5; at(6, 6) = -0.5; at(7, 3) = -I;
    at(7, 7) = 0.5; at(8, 4) = -I; at(8, 8) = -0.5; at(1, 9) = 2.0 * I; at(1, 1) = 0.5;
    at(2, 10) = 2.0 * I; at(2, 2) = -0.5;
  }
  return J;
}

// Ldiag_jz (instates.f90:228-300 P, :613-690 D): the eigenvectors ki ..
// ki+njz-1 of the state matrix (columns of v, ascending) span one j
// manifold; Jz restricted to it is diagonalised and its il-th eigenvector
// (0-based, ascending <Jz>) taken back to the internal variables.  The
// result depends on the manifold, not on the basis the solver chose in it.
inline void diag_jz(int nd, const std::vector<cd>& v, int ki, int njz, int il, double* invar) {
  const std::vector<cd> J = jz_matrix(nd);
  std::vector<cd> M((size_t)njz * njz, cd(0));
  for (int a = 0; a < njz; ++a)
    for (int b = 0; b < njz; ++b) {
      cd t = 0.0;
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j)
          t += std::conj(v[(size_t)i * nd + ki + a]) * J[(size_t)i * nd + j] * v[(size_t)j * nd + ki + b];
      M[(size_t)a * njz + b] = t;
    }
  std::vector<double> w;
  std::vector<cd> z;
  hermitian_eigen(njz, M, w, z);
  for (int i = 0; i < 10; ++i) invar[2 * i] = invar[2 * i + 1] = 0.0;
  for (int i = 0; i < nd; ++i) {
    cd t = 0.0;
    for (int a = 0; a < njz; ++a) t += z[(size_t)a * njz + il] * v[(size_t)i * nd + ki + a];
    invar[2 * i] = t.real();
    invar[2 * i + 1] = t.imag();
  }
}

// Manifold (ki, njz) and Jz index il of Ldiag_jz from instate and Ljz
// ('' = the reference's default per instate); il < 0 for a wrong Ljz.
inline void jz_selection(bool d_state, int instate, std::string ljz, int& ki, int& njz, int& il) {
  il = -1;
  std::vector<std::string> names;
  if (!d_state) {
    if (instate == 0) {
      ki = 0; njz = 2;
      if (ljz.empty()) ljz = "-1/2";
      names = {"-1/2", "+1/2"};
    } else {
      ki = 2; njz = 4;
      if (ljz.empty()) ljz = instate == 1 ? "-3/2" : "-1/2";
      names = {"-3/2", "-1/2", "+1/2", "+3/2"};
    }
  } else {
    if (instate <= 1) {
      ki = 0; njz = 4;
      if (ljz.empty()) ljz = instate == 0 ? "-3/2" : "-1/2";
      names = {"-3/2", "-1/2", "+1/2", "+3/2"};
    } else {
      ki = 4; njz = 6;
      if (ljz.empty()) ljz = instate == 2 ? "-5/2" : instate == 3 ? "-3/2" : "-1/2";
      names = {"-5/2", "-3/2", "-1/2", "+1/2", "+3/2", "+5/2"};
    }
  }
  for (size_t k = 0; k < names.size(); ++k)
    if (names[k] == ljz) il = (int)k;
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

// invar (10 complex as 20 doubles) for a P state instate 0..2; jz_il >= 0:
// the Ldiag_jz state (ki, njz, jz_il) instead of the default pair.
inline void p_state(const double* moments, double als, int instate, double* invar, int ki = 0, int njz = 0,
                    int jz_il = -1) {
  std::vector<double> w;
  std::vector<cd> v;
  hermitian_eigen(6, p_matrix(moments, als), w, v);
  if (jz_il >= 0) {
    diag_jz(6, v, ki, njz, jz_il, invar);
    return;
  }
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
inline void d_state(const double* M, double als_d, int instate, double* invar, int ki = 0, int njz = 0,
                    int jz_il = -1) {
  cd S[10][10];
  dstate::sod(S);
  std::vector<cd> A(100);
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) A[(size_t)i * 10 + j] = dstate::matdso(M, S, als_d, i, j);
  std::vector<double> w;
  std::vector<cd> v;
  hermitian_eigen(10, A, w, v);
  if (jz_il >= 0) {
    diag_jz(10, v, ki, njz, jz_il, invar);
    return;
  }
  const int il = 2 * instate, il1 = il + 1;
  const double r = 1.0 / std::sqrt(2.0);
  for (int i = 0; i < 10; ++i) {
    const cd z = r * v[(size_t)i * 10 + il] + r * v[(size_t)i * 10 + il1];
    invar[2 * i] = z.real();
    invar[2 * i + 1] = z.imag();
  }
}

}  // namespace instates
