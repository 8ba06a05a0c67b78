#include "tables.h"

#include <cmath>
#include <vector>

namespace adv
{
namespace
{
constexpr double kPi = 3.14159265358979323846;

// P_m(x), P_m'(x), P_m''(x) on (-1, 1)
void legendre3(int m, double x, double &p, double &dp, double &ddp)
{
  double pm1 = 1.0, pc = x;
  if (m == 0)
    {
      p = 1.0, dp = ddp = 0.0;
      return;
    }
  for (int j = 1; j < m; ++j)
    {
      const double pn = ((2 * j + 1) * x * pc - j * pm1) / (j + 1);
      pm1             = pc;
      pc              = pn;
    }
  p   = pc;
  dp  = m * (pm1 - x * pc) / (1.0 - x * x);
  ddp = (2.0 * x * dp - m * (m + 1.0) * p) / (1.0 - x * x);
}
} // namespace

void gauss_points(int n, double *pts, double *wts)
{
  for (int i = 0; i < n; ++i)
    {
      // Newton from the Tricomi-type initial guess, descending roots
      double x = std::cos(kPi * (4.0 * i + 3.0) / (4.0 * n + 2.0));
      double p, dp, ddp;
      for (int it = 0; it < 64; ++it)
        {
          legendre3(n, x, p, dp, ddp);
          const double dx = p / dp;
          x -= dx;
          if (std::fabs(dx) <= 1e-17)
            break;
        }
      legendre3(n, x, p, dp, ddp);
      pts[i] = 0.5 - 0.5 * x;
      wts[i] = 1.0 / ((1.0 - x * x) * dp * dp);
    }
}

void gauss_lobatto_points(int n, double *pts)
{
  pts[0]     = 0.0;
  pts[n - 1] = 1.0;
  for (int i = 1; i < n - 1; ++i)
    {
      double x = std::cos(kPi * i / (n - 1));
      double p, dp, ddp;
      for (int it = 0; it < 64; ++it)
        {
          legendre3(n - 1, x, p, dp, ddp);
          const double dx = dp / ddp;
          x -= dx;
          if (std::fabs(dx) <= 1e-17)
            break;
        }
      pts[i] = 0.5 - 0.5 * x;
    }
}

double lagrange(const double *z, int n, int i, double x)
{
  double v = 1.0;
  for (int j = 0; j < n; ++j)
    if (j != i)
      v *= (x - z[j]) / (z[i] - z[j]);
  return v;
}

double lagrange_derivative(const double *z, int n, int i, double x)
{
  double s = 0.0;
  for (int m = 0; m < n; ++m)
    if (m != i)
      {
        double v = 1.0 / (z[i] - z[m]);
        for (int j = 0; j < n; ++j)
          if (j != i && j != m)
            v *= (x - z[j]) / (z[i] - z[j]);
        s += v;
      }
  return s;
}

bool invert_matrix(int n, const double *a, double *inv)
{
  std::vector<double> m(a, a + n * n);
  for (int i = 0; i < n * n; ++i)
    inv[i] = (i % (n + 1) == 0) ? 1.0 : 0.0;
  for (int c = 0; c < n; ++c)
    {
      int p = c;
      for (int r = c + 1; r < n; ++r)
        if (std::fabs(m[r * n + c]) > std::fabs(m[p * n + c]))
          p = r;
      if (m[p * n + c] == 0.0)
        return false;
      for (int j = 0; j < n; ++j)
        {
          std::swap(m[c * n + j], m[p * n + j]);
          std::swap(inv[c * n + j], inv[p * n + j]);
        }
      const double d = 1.0 / m[c * n + c];
      for (int j = 0; j < n; ++j)
        {
          m[c * n + j] *= d;
          inv[c * n + j] *= d;
        }
      for (int r = 0; r < n; ++r)
        if (r != c && m[r * n + c] != 0.0)
          {
            const double f = m[r * n + c];
            for (int j = 0; j < n; ++j)
              {
                m[r * n + j] -= f * m[c * n + j];
                inv[r * n + j] -= f * inv[c * n + j];
              }
          }
    }
  return true;
}

void Tables1D::init(int degree)
{
  n = degree + 1;
  gauss_lobatto_points(n, gl);
  gauss_points(n, gp, gw);
  double s[kMaxN * kMaxN], si[kMaxN * kMaxN];
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i)
      {
        S[q][i]      = lagrange(gl, n, i, gp[q]);
        Sd[q][i]     = lagrange_derivative(gl, n, i, gp[q]);
        s[q * n + i] = S[q][i];
      }
  invert_matrix(n, s, si);
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q)
      Si[i][q] = si[i * n + q];
  // collocation derivative and face values of the Lagrange basis on the Gauss points
  for (int q = 0; q < n; ++q)
    for (int p = 0; p < n; ++p)
      D[q][p] = lagrange_derivative(gp, n, p, gp[q]);
  for (int q = 0; q < n; ++q)
    for (int p = 0; p < n; ++p)
      Dw[q][p] = D[p][q] * gw[p] / gw[q];
  for (int q = 0; q < n; ++q)
    {
      l0[q]  = lagrange(gp, n, q, 0.0);
      l1[q]  = lagrange(gp, n, q, 1.0);
      lw0[q] = l0[q] / gw[q];
      lw1[q] = l1[q] / gw[q];
      ld0[q]  = lagrange_derivative(gp, n, q, 0.0);
      ld1[q]  = lagrange_derivative(gp, n, q, 1.0);
      lwd0[q] = ld0[q] / gw[q];
      lwd1[q] = ld1[q] / gw[q];
    }
  for (int i = 0; i < n; ++i)
    {
      dphi0[i] = lagrange_derivative(gl, n, i, 0.0);
      dphi1[i] = lagrange_derivative(gl, n, i, 1.0);
    }
}

// Published low-storage Runge-Kutta tables (Kennedy, Carpenter & Lewis 2000;
// Tselios & Simos 2007), the same numbers as the reference's
// LowStorageRungeKuttaIntegrator (advection_solver.cc:826-898).
bool lsrk_coefficients(int scheme, std::vector<double> &a, std::vector<double> &b)
{
  switch (scheme)
    {
      case 0:
        b = {0.245170287303492, 0.184896052186740, 0.569933660509768};
        a = {0.755726351946097, 0.386954477304099};
        return true;
      case 1:
        b = {1153189308089. / 22510343858157., 1772645290293. / 4653164025191.,
             -1672844663538. / 4480602732383., 2114624349019. / 3568978502595.,
             5198255086312. / 14908931495163.};
        a = {970286171893. / 4311952581923., 6584761158862. / 12103376702013.,
             2251764453980. / 15575788980749., 26877169314380. / 34165994151039.};
        return true;
      case 2:
        b = {0.0941840925477795334, 0.149683694803496998, 0.285204742060440058,
             -0.122201846148053668, 0.0605151571191401122, 0.345986987898399296,
             0.186627171718797670};
        a = {0.241566650129646868 + b[0], 0.0423866513027719953 + b[1],
             0.215602732678803776 + b[2], 0.232328007537583987 + b[3],
             0.256223412574146438 + b[4], 0.0978694102142697230 + b[5]};
        return true;
      case 3:
        b = {2274579626619. / 23610510767302., 693987741272. / 12394497460941.,
             -347131529483. / 15096185902911., 1144057200723. / 32081666971178.,
             1562491064753. / 11797114684756., 13113619727965. / 44346030145118.,
             393957816125. / 7825732611452., 720647959663. / 6565743875477.,
             3559252274877. / 14424734981077.};
        a = {1107026461565. / 5417078080134., 38141181049399. / 41724347789894.,
             493273079041. / 11940823631197., 1851571280403. / 6147804934346.,
             11782306865191. / 62590030070788., 9452544825720. / 13648368537481.,
             4435885630781. / 26285702406235., 2357909744247. / 11371140753790.};
        return true;
      default:
        return false;
    }
}
} // namespace adv
