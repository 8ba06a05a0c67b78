// 1D shape tables of FE_DGQ(k) on Gauss-Lobatto nodes, evaluated at the
// points of QGauss(k+1), in the forms the fused stage kernel uses.  This is
// the role deal.II's UnivariateShapeData plays for FEEvaluation (reference:
// advection_solver.cc:440-445 selects QGauss(k+1) for operator and mass).
#pragma once

#include <vector>

namespace adv
{
constexpr int kMaxN = 7; // n = k + 1 <= 7

struct Tables1D
{
  int    n = 0;
  double gl[kMaxN] = {};       // Gauss-Lobatto support points on [0,1]
  double gp[kMaxN] = {};       // Gauss points on [0,1]
  double gw[kMaxN] = {};       // Gauss weights on [0,1]
  double S[kMaxN][kMaxN] = {}; // S[q][i] = phi_i(g_q): nodal -> Gauss point values
  double Si[kMaxN][kMaxN] = {};// S^{-1}[i][q]: Gauss point values -> nodal
  double D[kMaxN][kMaxN] = {}; // collocation derivative on Gauss points, D[q][p] = l_p'(g_q)
  // Weighted transposed collocation derivative: Dw[q][p] = D[p][q] w_p / w_q.
  // Z = diag(1/w) D^T diag(w) carries the integration by parts of the volume
  // term into Gauss-point space with the quadrature weights cancelled.
  double Dw[kMaxN][kMaxN] = {};
  double l0[kMaxN] = {}, l1[kMaxN] = {};   // l_q(0), l_q(1): Gauss-Lagrange basis at the faces
  double lw0[kMaxN] = {}, lw1[kMaxN] = {}; // l_q(s) / w_q
  double dphi0[kMaxN] = {}, dphi1[kMaxN] = {}; // phi_i'(0), phi_i'(1) of the nodal basis
  double ld0[kMaxN] = {}, ld1[kMaxN] = {};     // l_q'(0), l_q'(1) of the Gauss-Lagrange basis
  double lwd0[kMaxN] = {}, lwd1[kMaxN] = {};   // l_q'(s) / w_q
  double Sd[kMaxN][kMaxN] = {}; // Sd[q][i] = phi_i'(g_q)

  void init(int degree);
};

void gauss_points(int n, double *pts, double *wts);
void gauss_lobatto_points(int n, double *pts);
double lagrange(const double *z, int n, int i, double x);
double lagrange_derivative(const double *z, int n, int i, double x);
bool invert_matrix(int n, const double *a, double *inv);

// Coefficients of the low-storage Runge-Kutta schemes; a has n_stages - 1 entries.
bool lsrk_coefficients(int scheme, std::vector<double> &a, std::vector<double> &b);
} // namespace adv
