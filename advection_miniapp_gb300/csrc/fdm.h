// Fast-diagonalization (FDM) tables of the cellwise block-Jacobi
// preconditioner of the implicit solver: the counterpart of the reference's
// 1D set-up (advection_solver_implicit.cc:1020-1062) and
// CellwisePreconditionerFDM (advection_solver_implicit.cc:490-646).
//
// On the unit interval with the Lagrange basis on the k+1 Gauss points
// (diagonal mass W = diag(w)), the 1D advection operator with unit velocity
// of sign s and flux parameter alpha is
//   A1[i][j] = -sum_q l_i'(g_q) l_j(g_q) w_q
//              - l_i(0) l_j(0) (1 - alpha s) / 2 + l_i(1) l_j(1) (1 + alpha s) / 2,
// and W^{-1} A1 = V diag(lambda) V^{-1} (complex).  The tables hold lambda,
// V and V^{-1} W^{-1} for s = +1 and s = -1.
#pragma once

#include <complex>
#include <vector>

namespace adv
{
struct FdmTables
{
  int                               n = 0;
  std::vector<std::complex<double>> lambda[2]; // [sign index][i], sign index 0: s = +1, 1: s = -1
  std::vector<std::complex<double>> V[2];      // [i * n + j]
  std::vector<std::complex<double>> VinvW[2];  // V^{-1} W^{-1}, [i * n + j]
  std::vector<double>               A1[2];     // the real 1D operator W^{-1} A1, [i * n + j]
  double                            residual = 0.0; // max |W^{-1}A1 V - V Lambda| / |W^{-1}A1|
};

// Eigenvalues and right eigenvectors of a small complex matrix (n <= 8) by
// shifted QR iterations with deflation and inverse iteration.  Returns false
// if the iteration does not converge.
bool eigen_small(int n, const std::vector<std::complex<double>> &A, std::vector<std::complex<double>> &lambda,
                 std::vector<std::complex<double>> &V);

bool fdm_tables(int degree, double flux_alpha, FdmTables &t);
} // namespace adv
