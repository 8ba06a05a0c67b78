// CPU oracle for the matrix-free DG advection operator: TEST INFRASTRUCTURE.
//
// A plain FP64 restatement of the reference miniapp's algorithm: the tests
// compare the CUDA path with it, and it is the timed CPU baseline.  Each function
// names the reference lines (kronbichler/advection_miniapp) it follows.  The
// arithmetic the reference delegates to deal.II (FEEvaluation,
// FEFaceEvaluation, CellwiseInverseMassMatrix, MatrixFree::loop; deal.II >=
// 9.2, CMakeLists.txt:30, not vendored) is restated from its published
// definition: sum factorization with 1D shape matrices of FE_DGQ on
// Gauss-Lobatto nodes evaluated at the points of QGauss(k+1), and the exact
// cellwise inverse of the Gauss-quadrature mass matrix, S^{-1} diag(1/JxW)
// S^{-T}.  Parity with the reference itself is unpinned (it cannot be built
// here and ships no outputs); see oracle.h.

#include "oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <vector>

namespace
{
constexpr double PI   = 3.14159265358979323846;
constexpr int    MAXN = 8;

// ------------------------------------------------------------------------
// 1D tables
// ------------------------------------------------------------------------

// Legendre polynomial P_m and its first two derivatives at x in (-1,1),
// by the three-term recurrence and the Legendre differential equation.
void legendre(int m, double x, double &p, double &dp, double &ddp)
{
  double p0 = 1.0, p1 = x;
  if (m == 0)
    {
      p = 1.0, dp = 0.0, ddp = 0.0;
      return;
    }
  for (int j = 2; j <= m; ++j)
    {
      const double p2 = ((2.0 * j - 1.0) * x * p1 - (j - 1.0) * p0) / j;
      p0 = p1;
      p1 = p2;
    }
  p   = p1;
  dp  = m * (p0 - x * p1) / (1.0 - x * x);
  ddp = (2.0 * x * dp - m * (m + 1.0) * p) / (1.0 - x * x);
}

// Gauss-Legendre points/weights on [0,1] (QGauss(n)), ascending.
void gauss_points(int n, double *pts, double *wts)
{
  for (int i = 0; i < n; ++i)
    {
      double x = std::cos(PI * (i + 0.75) / (n + 0.5));
      double p, dp, ddp;
      for (int it = 0; it < 100; ++it)
        {
          legendre(n, x, p, dp, ddp);
          const double dx = p / dp;
          x -= dx;
          if (std::abs(dx) < 1e-16)
            break;
        }
      legendre(n, x, p, dp, ddp);
      pts[i] = 0.5 * (1.0 - x);
      wts[i] = 1.0 / ((1.0 - x * x) * dp * dp);  // 2/((1-x^2)P'^2) halved for [0,1]
    }
}

// Gauss-Lobatto points on [0,1] (QGaussLobatto(n)), ascending.
void gauss_lobatto_points(int n, double *pts)
{
  pts[0]     = 0.0;
  pts[n - 1] = 1.0;
  const int m = n - 1;
  for (int i = 1; i < n - 1; ++i)
    {
      double x = std::cos(PI * i / m);
      double p, dp, ddp;
      for (int it = 0; it < 100; ++it)
        {
          legendre(m, x, p, dp, ddp);
          const double dx = dp / ddp;
          x -= dx;
          if (std::abs(dx) < 1e-16)
            break;
        }
      pts[i] = 0.5 * (1.0 - x);
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
    {
      if (m == i)
        continue;
      double v = 1.0 / (z[i] - z[m]);
      for (int j = 0; j < n; ++j)
        if (j != i && j != m)
          v *= (x - z[j]) / (z[i] - z[j]);
      s += v;
    }
  return s;
}

// Gauss-Jordan inverse with partial pivoting of a dense n x n matrix.
bool invert(int n, const double *a, double *inv)
{
  std::vector<double> m(a, a + n * n);
  for (int i = 0; i < n * n; ++i)
    inv[i] = 0.0;
  for (int i = 0; i < n; ++i)
    inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c)
    {
      int    piv  = c;
      double best = std::abs(m[c * n + c]);
      for (int r = c + 1; r < n; ++r)
        if (std::abs(m[r * n + c]) > best)
          best = std::abs(m[r * n + c]), piv = r;
      if (best == 0.0)
        return false;
      if (piv != c)
        for (int j = 0; j < n; ++j)
          {
            std::swap(m[c * n + j], m[piv * n + j]);
            std::swap(inv[c * n + j], inv[piv * n + j]);
          }
      const double d = 1.0 / m[c * n + c];
      for (int j = 0; j < n; ++j)
        m[c * n + j] *= d, inv[c * n + j] *= d;
      for (int r = 0; r < n; ++r)
        if (r != c)
          {
            const double f = m[r * n + c];
            if (f != 0.0)
              for (int j = 0; j < n; ++j)
                m[r * n + j] -= f * m[c * n + j], inv[r * n + j] -= f * inv[c * n + j];
          }
    }
  return true;
}

struct Tables
{
  int    n;
  double gl[MAXN], gp[MAXN], gw[MAXN];
  double S[MAXN][MAXN];  // S[q][i] = phi_i(g_q)
  double D[MAXN][MAXN];  // D[q][i] = phi_i'(g_q)
  double Si[MAXN][MAXN]; // S^{-1}, Si[i][q]
  double f[2][MAXN];     // phi_i(0), phi_i(1)
  double df[2][MAXN];    // phi_i'(0), phi_i'(1)

  void init(int degree)
  {
    n = degree + 1;
    gauss_lobatto_points(n, gl);
    gauss_points(n, gp, gw);
    double s[MAXN * MAXN], si[MAXN * MAXN];
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < n; ++i)
        {
          S[q][i]      = lagrange(gl, n, i, gp[q]);
          D[q][i]      = lagrange_derivative(gl, n, i, gp[q]);
          s[q * n + i] = S[q][i];
        }
    invert(n, s, si);
    for (int i = 0; i < n; ++i)
      for (int q = 0; q < n; ++q)
        Si[i][q] = si[i * n + q];
    for (int i = 0; i < n; ++i)
      for (int e = 0; e < 2; ++e)
        {
          f[e][i]  = lagrange(gl, n, i, double(e));
          df[e][i] = lagrange_derivative(gl, n, i, double(e));
        }
  }
};

// ------------------------------------------------------------------------
// Configuration-dependent point functions
// ------------------------------------------------------------------------

struct Physics
{
  oracle_config cfg;
  double        L[3];

  // Deformation of the structured box (mesh_type 1): every component is
  // shifted by A L_d sin(2 pi s_{d+1}) sin(2 pi s_{d+2}), s the unit-box
  // coordinate.  Plays the role of DeformedCubeManifold::push_forward
  // (advection_solver.cc:244-255) for the 3D deformation of the workload.
  void deform(const double x[3], double y[3]) const
  {
    double s[3];
    for (int d = 0; d < 3; ++d)
      s[d] = (x[d] - cfg.domain_lo[d]) / L[d];
    for (int d = 0; d < 3; ++d)
      y[d] = x[d] + cfg.deformation * L[d] * std::sin(2.0 * PI * s[(d + 1) % 3]) *
                      std::sin(2.0 * PI * s[(d + 2) % 3]);
  }

  // Transport velocity at x and time t.  Constant (ExactSolution::
  // get_transport_direction, advection_solver.cc:174-178) or the rotating,
  // divergence-free field scaled by cos(pi t / T) (TransportSpeed,
  // advection_solver_variable.cc:153-183, extended to 3D).
  void speed(const double x[3], double t, double a[3]) const
  {
    if (cfg.velocity_type == 0)
      {
        for (int d = 0; d < 3; ++d)
          a[d] = cfg.velocity[d];
        return;
      }
    const double fac = std::cos(PI * t / cfg.velocity_period);
    const double sx = std::sin(PI * x[0]), sy = std::sin(PI * x[1]);
    a[0] = fac * cfg.velocity[0] * sx * sx * std::sin(2.0 * PI * x[1]);
    a[1] = -fac * cfg.velocity[1] * sy * sy * std::sin(2.0 * PI * x[0]);
    a[2] = fac * cfg.velocity[2];
  }

  // Exact solution (the initial condition translated with the constant
  // velocity), the analogue of ExactSolution::value (advection_solver.cc:149-172).
  double exact(const double x[3], double t) const
  {
    const double *a = cfg.velocity;
    const double  tt = cfg.velocity_type == 0 ? t : 0.0;
    if (cfg.initial_condition == 0)
      {
        double s[3];
        for (int d = 0; d < 3; ++d)
          {
            double y = (x[d] - a[d] * tt - cfg.domain_lo[d]) / L[d] - cfg.ic_params[d];
            s[d]     = y - std::floor(y);
          }
        double r2 = 0.0;
        for (int d = 0; d < 3; ++d)
          r2 += (s[d] - 0.5) * (s[d] - 0.5);
        return std::sin(2.0 * PI * s[0]) * std::sin(2.0 * PI * s[1]) * std::sin(2.0 * PI * s[2]) +
               std::exp(-50.0 * r2);
      }
    if (cfg.initial_condition == 1)
      {
        double r2 = 0.0;
        for (int d = 0; d < 3; ++d)
          {
            const double y = x[d] - a[d] * tt - cfg.ic_params[d];
            r2 += y * y;
          }
        const double w = cfg.ic_params[3];
        return std::exp(-r2 / (w * w));
      }
    double r = std::sin(4.0 * PI * (x[0] - tt * a[0]));
    for (int d = 1; d < 3; ++d)
      r *= std::cos(4.0 * PI * (x[d] - tt * a[d]));
    return r;
  }

  double boundary(const double x[3], double t) const
  {
    return cfg.boundary_value == 1 ? exact(x, t) : 0.0;
  }
};

struct Face
{
  int64_t minus, plus;  // plus < 0: boundary face
  int     dir;
  int     side_minus, side_plus;  // reference coordinate xi_dir of the face in each cell
};

// ------------------------------------------------------------------------
// Operator data (what MatrixFree::reinit precomputes, advection_solver.cc:435-465)
// ------------------------------------------------------------------------

struct Op
{
  Physics ph;
  Tables  tb;
  int     n;
  int     nc[3];
  int64_t n_cells, n_dofs;
  double  h[3];
  bool    curved;
  bool    need_grad;

  // per cell and Gauss point: JxW, J^{-1} (row-major), position
  std::vector<double> jxw, jinv, xq;
  std::vector<Face>   faces;
  std::vector<int64_t> row_start[3]; // faces grouped by direction and row
  // per face and face point: JxW_f * n_minus (3), x (3), JxW_f; SIPG: J^{-1} on each side
  std::vector<double> f_nj, f_x, f_jxw, f_jinv_m, f_jinv_p;

  int64_t cell_index(int i, int j, int k) const { return i + (int64_t)nc[0] * (j + (int64_t)nc[1] * k); }

  void cell_lo(int64_t c, double lo[3]) const
  {
    const int i = int(c % nc[0]), j = int((c / nc[0]) % nc[1]), k = int(c / ((int64_t)nc[0] * nc[1]));
    const int ijk[3] = {i, j, k};
    for (int d = 0; d < 3; ++d)
      lo[d] = ph.cfg.domain_lo[d] + ijk[d] * h[d];
  }

  // Mapping of a cell: affine, or the degree-k Lagrange interpolation on the
  // Gauss-Lobatto support points of the deformed box (the role of
  // MappingQGeneric(k) with a manifold, advection_solver.cc:439, 1101-1125).
  void support_points(int64_t c, double *X) const
  {
    double lo[3];
    cell_lo(c, lo);
    for (int c2 = 0; c2 < n; ++c2)
      for (int c1 = 0; c1 < n; ++c1)
        for (int c0 = 0; c0 < n; ++c0)
          {
            const double x[3] = {lo[0] + h[0] * tb.gl[c0], lo[1] + h[1] * tb.gl[c1],
                                 lo[2] + h[2] * tb.gl[c2]};
            double *y = X + 3 * (c0 + n * (c1 + n * c2));
            if (curved)
              ph.deform(x, y);
            else
              y[0] = x[0], y[1] = x[1], y[2] = x[2];
          }
  }

  // position and Jacobian J[i][j] = dx_i/dxi_j at reference point xi
  void map_point(int64_t c, const double *X, const double xi[3], double x[3], double J[3][3]) const
  {
    if (!curved)
      {
        double lo[3];
        cell_lo(c, lo);
        for (int d = 0; d < 3; ++d)
          {
            x[d] = lo[d] + h[d] * xi[d];
            for (int e = 0; e < 3; ++e)
              J[d][e] = d == e ? h[d] : 0.0;
          }
        return;
      }
    double v[3][MAXN], dv[3][MAXN];
    for (int d = 0; d < 3; ++d)
      for (int i = 0; i < n; ++i)
        v[d][i] = lagrange(tb.gl, n, i, xi[d]), dv[d][i] = lagrange_derivative(tb.gl, n, i, xi[d]);
    for (int d = 0; d < 3; ++d)
      {
        x[d] = 0.0;
        for (int e = 0; e < 3; ++e)
          J[d][e] = 0.0;
      }
    // sums over the support points relative to the first one: the
    // derivative weights sum to zero, and on absolute coordinates (size ~1)
    // the Jacobian (size ~h) would carry rounding of a few ulps of 1 that
    // depends on the order of the sums
    for (int c2 = 0; c2 < n; ++c2)
      for (int c1 = 0; c1 < n; ++c1)
        for (int c0 = 0; c0 < n; ++c0)
          {
            const double *y  = X + 3 * (c0 + n * (c1 + n * c2));
            const double  w  = v[0][c0] * v[1][c1] * v[2][c2];
            const double  w0 = dv[0][c0] * v[1][c1] * v[2][c2];
            const double  w1 = v[0][c0] * dv[1][c1] * v[2][c2];
            const double  w2 = v[0][c0] * v[1][c1] * dv[2][c2];
            for (int d = 0; d < 3; ++d)
              {
                const double yr = y[d] - X[d];
                x[d] += w * yr;
                J[d][0] += w0 * yr;
                J[d][1] += w1 * yr;
                J[d][2] += w2 * yr;
              }
          }
    for (int d = 0; d < 3; ++d)
      x[d] += X[d];
  }

  static double inverse3(const double J[3][3], double *Ji)
  {
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double id = 1.0 / det;
    Ji[0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
    Ji[1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    Ji[2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    Ji[3] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    Ji[4] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[5] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    Ji[6] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
    Ji[7] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    Ji[8] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    return det;
  }

  void tangential(int d, int &t1, int &t2) const
  {
    t1 = d == 0 ? 1 : 0;
    t2 = d == 2 ? 1 : 2;
  }

  int setup(const oracle_config &cfg)
  {
    ph.cfg = cfg;
    if (cfg.degree < 1 || cfg.degree > 6)
      return 1;
    for (int d = 0; d < 3; ++d)
      {
        if (cfg.n_cells[d] < 1 || !(cfg.domain_hi[d] > cfg.domain_lo[d]))
          return 1;
        ph.L[d] = cfg.domain_hi[d] - cfg.domain_lo[d];
        nc[d]   = cfg.n_cells[d];
        h[d]    = ph.L[d] / nc[d];
      }
    tb.init(cfg.degree);
    n         = tb.n;
    curved    = cfg.mesh_type == 1;
    need_grad = cfg.factor_skew != 0.0 || cfg.diffusion != 0.0;
    n_cells   = (int64_t)nc[0] * nc[1] * nc[2];
    const int64_t nq = (int64_t)n * n * n;
    n_dofs    = n_cells * nq;
    jxw.resize(n_cells * nq);
    jinv.resize(n_cells * nq * 9);
    xq.resize(n_cells * nq * 3);

#pragma omp parallel
    {
      std::vector<double> X(3 * nq);
#pragma omp for schedule(static)
      for (int64_t c = 0; c < n_cells; ++c)
        {
          support_points(c, X.data());
          for (int q2 = 0; q2 < n; ++q2)
            for (int q1 = 0; q1 < n; ++q1)
              for (int q0 = 0; q0 < n; ++q0)
                {
                  const int64_t q      = q0 + n * (q1 + n * q2);
                  const double  xi[3]  = {tb.gp[q0], tb.gp[q1], tb.gp[q2]};
                  double        x[3], J[3][3];
                  map_point(c, X.data(), xi, x, J);
                  const double det = inverse3(J, &jinv[(c * nq + q) * 9]);
                  jxw[c * nq + q]  = det * tb.gw[q0] * tb.gw[q1] * tb.gw[q2];
                  for (int d = 0; d < 3; ++d)
                    xq[(c * nq + q) * 3 + d] = x[d];
                }
        }
    }

    // faces, grouped by direction and row (the two tangential cell indices),
    // ordered along the row so that rows touch disjoint cells
    for (int d = 0; d < 3; ++d)
      {
        int t1, t2;
        tangential(d, t1, t2);
        const int npos = cfg.periodic ? nc[d] : nc[d] + 1;
        row_start[d].clear();
        for (int j2 = 0; j2 < nc[t2]; ++j2)
          for (int j1 = 0; j1 < nc[t1]; ++j1)
            {
              row_start[d].push_back((int64_t)faces.size());
              for (int p = 0; p < npos; ++p)
                {
                  int ijk[3];
                  ijk[t1] = j1, ijk[t2] = j2;
                  Face f;
                  f.dir = d;
                  if (cfg.periodic)
                    {
                      ijk[d]      = (p - 1 + nc[d]) % nc[d];
                      f.minus     = cell_index(ijk[0], ijk[1], ijk[2]);
                      ijk[d]      = p;
                      f.plus      = cell_index(ijk[0], ijk[1], ijk[2]);
                      f.side_minus = 1, f.side_plus = 0;
                    }
                  else if (p == 0)
                    {
                      ijk[d]  = 0;
                      f.minus = cell_index(ijk[0], ijk[1], ijk[2]);
                      f.plus  = -1;
                      f.side_minus = 0, f.side_plus = 0;
                    }
                  else if (p == nc[d])
                    {
                      ijk[d]  = nc[d] - 1;
                      f.minus = cell_index(ijk[0], ijk[1], ijk[2]);
                      f.plus  = -1;
                      f.side_minus = 1, f.side_plus = 0;
                    }
                  else
                    {
                      ijk[d]  = p - 1;
                      f.minus = cell_index(ijk[0], ijk[1], ijk[2]);
                      ijk[d]  = p;
                      f.plus  = cell_index(ijk[0], ijk[1], ijk[2]);
                      f.side_minus = 1, f.side_plus = 0;
                    }
                  faces.push_back(f);
                }
            }
        row_start[d].push_back((int64_t)faces.size());
      }

    const int64_t nf  = (int64_t)faces.size();
    const int64_t nfq = (int64_t)n * n;
    f_nj.resize(nf * nfq * 3);
    f_x.resize(nf * nfq * 3);
    f_jxw.resize(nf * nfq);
    if (cfg.diffusion != 0.0)
      {
        f_jinv_m.resize(nf * nfq * 9);
        f_jinv_p.resize(nf * nfq * 9);
      }
#pragma omp parallel
    {
      std::vector<double> X(3 * nq), Xp(3 * nq);
#pragma omp for schedule(static)
      for (int64_t fi = 0; fi < nf; ++fi)
        {
          const Face &f = faces[fi];
          int         t1, t2;
          tangential(f.dir, t1, t2);
          support_points(f.minus, X.data());
          if (f.plus >= 0 && !f_jinv_p.empty())
            support_points(f.plus, Xp.data());
          for (int q2 = 0; q2 < n; ++q2)
            for (int q1 = 0; q1 < n; ++q1)
              {
                const int64_t fq = q1 + n * q2;
                double        xi[3];
                xi[f.dir] = f.side_minus;
                xi[t1] = tb.gp[q1], xi[t2] = tb.gp[q2];
                double x[3], J[3][3], Ji[9];
                map_point(f.minus, X.data(), xi, x, J);
                const double det = inverse3(J, Ji);
                // area-weighted normal N = det(J) J^{-T} e_dir points to +xi_dir
                double N[3], nrm = 0.0;
                for (int i = 0; i < 3; ++i)
                  N[i] = det * Ji[f.dir * 3 + i], nrm += N[i] * N[i];
                nrm             = std::sqrt(nrm);
                const double sg = f.side_minus == 1 ? 1.0 : -1.0;
                const double wf = tb.gw[q1] * tb.gw[q2];
                for (int i = 0; i < 3; ++i)
                  {
                    f_nj[(fi * nfq + fq) * 3 + i] = sg * N[i] * wf;
                    f_x[(fi * nfq + fq) * 3 + i]  = x[i];
                  }
                f_jxw[fi * nfq + fq] = nrm * wf;
                if (!f_jinv_m.empty())
                  {
                    for (int i = 0; i < 9; ++i)
                      f_jinv_m[(fi * nfq + fq) * 9 + i] = Ji[i];
                    if (f.plus >= 0)
                      {
                        xi[f.dir] = f.side_plus;
                        double xp[3], Jp[3][3];
                        map_point(f.plus, Xp.data(), xi, xp, Jp);
                        inverse3(Jp, &f_jinv_p[(fi * nfq + fq) * 9]);
                      }
                  }
              }
        }
    }
    return 0;
  }
};

// ------------------------------------------------------------------------
// Sum-factorization kernels (what FEEvaluation / FEFaceEvaluation and
// CellwiseInverseMassMatrix do inside deal.II)
// ------------------------------------------------------------------------

// out = M applied along direction dir of an N^3 array (x fastest):
// tr == false: out[..q..] = sum_i M[q][i] in[..i..]; tr == true: sum_i M[i][q] in[..i..]
template <int N, int dir, bool tr, bool add>
inline void apply3(const double (&M)[MAXN][MAXN], const double *in, double *out)
{
  constexpr int s  = dir == 0 ? 1 : dir == 1 ? N : N * N;
  constexpr int s1 = dir == 0 ? N : 1;
  constexpr int s2 = dir == 2 ? N : N * N;
  for (int k2 = 0; k2 < N; ++k2)
    for (int k1 = 0; k1 < N; ++k1)
      {
        const int base = k1 * s1 + k2 * s2;
        double    x[N];
        for (int i = 0; i < N; ++i)
          x[i] = in[base + i * s];
        for (int q = 0; q < N; ++q)
          {
            double sum = 0.0;
            for (int i = 0; i < N; ++i)
              sum += (tr ? M[i][q] : M[q][i]) * x[i];
            if (add)
              out[base + q * s] += sum;
            else
              out[base + q * s] = sum;
          }
      }
}

// same on an N^2 face array
template <int N, int dir, bool tr, bool add>
inline void apply2(const double (&M)[MAXN][MAXN], const double *in, double *out)
{
  constexpr int s  = dir == 0 ? 1 : N;
  constexpr int s1 = dir == 0 ? N : 1;
  for (int k1 = 0; k1 < N; ++k1)
    {
      const int base = k1 * s1;
      double    x[N];
      for (int i = 0; i < N; ++i)
        x[i] = in[base + i * s];
      for (int q = 0; q < N; ++q)
        {
          double sum = 0.0;
          for (int i = 0; i < N; ++i)
            sum += (tr ? M[i][q] : M[q][i]) * x[i];
          if (add)
            out[base + q * s] += sum;
          else
            out[base + q * s] = sum;
        }
    }
}

template <int N>
struct Kernels
{
  static constexpr int NQ = N * N * N;
  static constexpr int NF = N * N;

  // index of cell-local DoF/point with coordinate a along dir and face index
  // (b, c) along the sorted tangential directions
  static inline int idx3(int dir, int a, int b, int c)
  {
    if (dir == 0)
      return a + N * (b + N * c);
    if (dir == 1)
      return b + N * (a + N * c);
    return b + N * (c + N * a);
  }

  // values (and optionally reference gradients) at the Gauss points of a cell
  static void evaluate_cell(const Tables &tb, const double *u, double *val, double (*grad)[NQ])
  {
    double t1[NQ], t2[NQ];
    apply3<N, 0, false, false>(tb.S, u, t1);
    apply3<N, 1, false, false>(tb.S, t1, t2);
    apply3<N, 2, false, false>(tb.S, t2, val);
    if (grad)
      {
        apply3<N, 0, false, false>(tb.D, u, t1);
        apply3<N, 1, false, false>(tb.S, t1, t2);
        apply3<N, 2, false, false>(tb.S, t2, grad[0]);
        apply3<N, 0, false, false>(tb.S, u, t1);
        apply3<N, 1, false, false>(tb.D, t1, t2);
        apply3<N, 2, false, false>(tb.S, t2, grad[1]);
        apply3<N, 1, false, false>(tb.S, t1, t2);
        apply3<N, 2, false, false>(tb.D, t2, grad[2]);
      }
  }

  // dst += integral of val * v + sum_j grad_j * d_j v (reference gradients)
  static void integrate_cell(const Tables &tb, const double *val, const double (*grad)[NQ], double *dst)
  {
    double t1[NQ], t2[NQ];
    double acc[NQ];
    apply3<N, 2, true, false>(tb.D, grad[2], t1);
    if (val)
      apply3<N, 2, true, true>(tb.S, val, t1);
    apply3<N, 1, true, false>(tb.S, t1, t2);
    apply3<N, 2, true, false>(tb.S, grad[1], t1);
    apply3<N, 1, true, true>(tb.D, t1, t2);
    apply3<N, 0, true, false>(tb.S, t2, acc);
    apply3<N, 2, true, false>(tb.S, grad[0], t1);
    apply3<N, 1, true, false>(tb.S, t1, t2);
    apply3<N, 0, true, true>(tb.D, t2, acc);
    for (int i = 0; i < NQ; ++i)
      dst[i] += acc[i];
  }

  // values (side value vector f[side]) and reference gradients at the face
  // points of one cell face
  static void evaluate_face(const Tables &tb, const double *u, int dir, int side, double *val,
                            double (*grad)[NF])
  {
    double lay[NF], dlay[NF], t[NF];
    for (int c = 0; c < N; ++c)
      for (int b = 0; b < N; ++b)
        {
          double s = 0.0, ds = 0.0;
          for (int a = 0; a < N; ++a)
            {
              s += tb.f[side][a] * u[idx3(dir, a, b, c)];
              ds += tb.df[side][a] * u[idx3(dir, a, b, c)];
            }
          lay[b + N * c]  = s;
          dlay[b + N * c] = ds;
        }
    apply2<N, 0, false, false>(tb.S, lay, t);
    apply2<N, 1, false, false>(tb.S, t, val);
    if (grad)
      {
        int t1 = dir == 0 ? 1 : 0, t2 = dir == 2 ? 1 : 2;
        // normal derivative
        apply2<N, 0, false, false>(tb.S, dlay, t);
        apply2<N, 1, false, false>(tb.S, t, grad[dir]);
        // tangential derivatives
        apply2<N, 0, false, false>(tb.D, lay, t);
        apply2<N, 1, false, false>(tb.S, t, grad[t1]);
        apply2<N, 0, false, false>(tb.S, lay, t);
        apply2<N, 1, false, false>(tb.D, t, grad[t2]);
      }
  }

  // dst += face integral of val * v + sum_j grad_j d_j v
  static void integrate_face(const Tables &tb, const double *val, const double (*grad)[NF], int dir,
                             int side, double *dst)
  {
    double lay[NF], dlay[NF] = {}, t[NF];
    apply2<N, 1, true, false>(tb.S, val, t);
    apply2<N, 0, true, false>(tb.S, t, lay);
    if (grad)
      {
        int t1 = dir == 0 ? 1 : 0, t2 = dir == 2 ? 1 : 2;
        apply2<N, 1, true, false>(tb.S, grad[t1], t);
        apply2<N, 0, true, true>(tb.D, t, lay);
        apply2<N, 1, true, false>(tb.D, grad[t2], t);
        apply2<N, 0, true, true>(tb.S, t, lay);
        apply2<N, 1, true, false>(tb.S, grad[dir], t);
        apply2<N, 0, true, false>(tb.S, t, dlay);
      }
    for (int c = 0; c < N; ++c)
      for (int b = 0; b < N; ++b)
        for (int a = 0; a < N; ++a)
          {
            double v = tb.f[side][a] * lay[b + N * c];
            if (grad)
              v += tb.df[side][a] * dlay[b + N * c];
            dst[idx3(dir, a, b, c)] += v;
          }
  }

  // ---- workers of the operator (advection_solver.cc:469-631,
  //      advection_diffusion_solver.cc:531-613 for the viscous terms)

  static void cell_worker(const Op &op, int64_t c, const double *src, double *dst, double t)
  {
    const Tables &tb   = op.tb;
    const auto   &cfg  = op.ph.cfg;
    const double  skew = cfg.factor_skew, nu = cfg.diffusion;
    double        val[NQ], grad[3][NQ], gout[3][NQ], vout[NQ];
    evaluate_cell(tb, src + c * NQ, val, op.need_grad ? grad : nullptr);
    for (int q = 0; q < NQ; ++q)
      {
        const double *Ji  = &op.jinv[(c * NQ + q) * 9];
        const double  JxW = op.jxw[c * NQ + q];
        double        a[3];
        op.ph.speed(&op.xq[(c * NQ + q) * 3], t, a);
        double G[3], V = 0.0;
        for (int i = 0; i < 3; ++i)
          G[i] = (1.0 - skew) * a[i] * val[q];
        if (op.need_grad)
          {
            double gu[3];
            for (int i = 0; i < 3; ++i)
              gu[i] = Ji[0 * 3 + i] * grad[0][q] + Ji[1 * 3 + i] * grad[1][q] + Ji[2 * 3 + i] * grad[2][q];
            for (int i = 0; i < 3; ++i)
              G[i] -= nu * gu[i];
            V = -skew * (a[0] * gu[0] + a[1] * gu[1] + a[2] * gu[2]);
          }
        for (int j = 0; j < 3; ++j)
          gout[j][q] = JxW * (Ji[j * 3 + 0] * G[0] + Ji[j * 3 + 1] * G[1] + Ji[j * 3 + 2] * G[2]);
        vout[q] = JxW * V;
      }
    integrate_cell(tb, op.need_grad ? vout : nullptr, gout, dst + c * NQ);
  }

  // interior or boundary face: numerical flux and SIPG terms
  static void face_worker(const Op &op, int64_t fi, const double *src, double *dst, double t)
  {
    const Face   &f    = op.faces[fi];
    const Tables &tb   = op.tb;
    const auto   &cfg  = op.ph.cfg;
    const double  skew = cfg.factor_skew, alpha = cfg.flux_alpha, nu = cfg.diffusion;
    const bool    visc = nu != 0.0;
    const double  sigma =
      cfg.penalty_factor * (cfg.degree + 1.0) * (cfg.degree + 1.0) / op.h[f.dir];
    double um[NF], up[NF], gm[3][NF], gp[3][NF];
    double vm[NF], vp[NF], dm[3][NF], dp[3][NF];
    evaluate_face(tb, src + f.minus * NQ, f.dir, f.side_minus, um, visc ? gm : nullptr);
    if (f.plus >= 0)
      evaluate_face(tb, src + f.plus * NQ, f.dir, f.side_plus, up, visc ? gp : nullptr);
    for (int q = 0; q < NF; ++q)
      {
        const double *nj  = &op.f_nj[(fi * NF + q) * 3];
        const double *x   = &op.f_x[(fi * NF + q) * 3];
        const double  jxw = op.f_jxw[fi * NF + q];
        double        a[3];
        op.ph.speed(x, t, a);
        const double an    = a[0] * nj[0] + a[1] * nj[1] + a[2] * nj[2]; // (a.n) JxW_f
        const double u_m   = um[q];
        const double u_p   = f.plus >= 0 ? up[q] : op.ph.boundary(x, t);
        const double flux  = 0.5 * ((u_m + u_p) * an + alpha * std::abs(an) * (u_m - u_p));
        vm[q]              = -flux + skew * an * u_m;
        vp[q]              = flux - skew * an * u_p;
        if (visc)
          {
            double nrm[3];
            for (int i = 0; i < 3; ++i)
              nrm[i] = nj[i] / jxw;
            const double *Jm = &op.f_jinv_m[(fi * NF + q) * 9];
            double        dnm = 0.0;
            for (int i = 0; i < 3; ++i)
              dnm += nrm[i] * (Jm[0 * 3 + i] * gm[0][q] + Jm[1 * 3 + i] * gm[1][q] + Jm[2 * 3 + i] * gm[2][q]);
            double jump, avg_dn;
            const double *Jp = f.plus >= 0 ? &op.f_jinv_p[(fi * NF + q) * 9] : nullptr;
            if (f.plus >= 0)
              {
                double dnp = 0.0;
                for (int i = 0; i < 3; ++i)
                  dnp += nrm[i] * (Jp[0 * 3 + i] * gp[0][q] + Jp[1 * 3 + i] * gp[1][q] + Jp[2 * 3 + i] * gp[2][q]);
                jump   = u_m - u_p;
                avg_dn = 0.5 * (dnm + dnp);
              }
            else
              {
                // Dirichlet data by the mirror principle: u+ = 2g - u-, grad u+ = grad u-
                jump   = 2.0 * (u_m - u_p);
                avg_dn = dnm;
              }
            const double pen = (-sigma * nu * jump + nu * avg_dn) * jxw;
            vm[q] += pen;
            vp[q] -= pen;
            // + <[u], nu {d_n v}>: coefficient of d_n v on each side
            const double cn = 0.5 * nu * jump * jxw;
            for (int j = 0; j < 3; ++j)
              {
                dm[j][q] = cn * (Jm[j * 3 + 0] * nrm[0] + Jm[j * 3 + 1] * nrm[1] + Jm[j * 3 + 2] * nrm[2]);
                if (f.plus >= 0)
                  dp[j][q] = cn * (Jp[j * 3 + 0] * nrm[0] + Jp[j * 3 + 1] * nrm[1] + Jp[j * 3 + 2] * nrm[2]);
              }
          }
      }
    integrate_face(tb, vm, visc ? dm : nullptr, f.dir, f.side_minus, dst + f.minus * NQ);
    if (f.plus >= 0)
      integrate_face(tb, vp, visc ? dp : nullptr, f.dir, f.side_plus, dst + f.plus * NQ);
  }

  // dst = L(t) src: data.loop with cell, inner-face and boundary-face workers
  static void apply_unscaled(const Op &op, const double *src, double *dst, double t)
  {
    const int64_t nd = op.n_dofs;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nd; ++i)
      dst[i] = 0.0;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < op.n_cells; ++c)
      cell_worker(op, c, src, dst, t);
    for (int d = 0; d < 3; ++d)
      {
        const auto   &rs    = op.row_start[d];
        const int64_t nrows = (int64_t)rs.size() - 1;
#pragma omp parallel for schedule(static)
        for (int64_t r = 0; r < nrows; ++r)
          for (int64_t fi = rs[r]; fi < rs[r + 1]; ++fi)
            face_worker(op, fi, src, dst, t);
      }
  }

  // CellwiseInverseMassMatrix::apply: S^{-1} diag(1/JxW) S^{-T} per cell
  static void inverse_mass(const Op &op, const double *src, double *dst)
  {
    const Tables &tb = op.tb;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < op.n_cells; ++c)
      {
        double t1[NQ], t2[NQ];
        apply3<N, 0, true, false>(tb.Si, src + c * NQ, t1);
        apply3<N, 1, true, false>(tb.Si, t1, t2);
        apply3<N, 2, true, false>(tb.Si, t2, t1);
        for (int q = 0; q < NQ; ++q)
          t1[q] /= op.jxw[c * NQ + q];
        apply3<N, 0, false, false>(tb.Si, t1, t2);
        apply3<N, 1, false, false>(tb.Si, t2, t1);
        apply3<N, 2, false, false>(tb.Si, t1, dst + c * NQ);
      }
  }

  // project_initial: u0 at the Gauss points, transform_from_q_points_to_basis
  static void project(const Op &op, double t, double *dst)
  {
    const Tables &tb = op.tb;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < op.n_cells; ++c)
      {
        double v[NQ], t1[NQ], t2[NQ];
        for (int q = 0; q < NQ; ++q)
          v[q] = op.ph.exact(&op.xq[(c * NQ + q) * 3], t);
        apply3<N, 0, false, false>(tb.Si, v, t1);
        apply3<N, 1, false, false>(tb.Si, t1, t2);
        apply3<N, 2, false, false>(tb.Si, t2, dst + c * NQ);
      }
  }

  static void mass_energy(const Op &op, const double *u, double out[3])
  {
    double m = 0.0, e = 0.0, hs = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : m, e, hs)
    for (int64_t c = 0; c < op.n_cells; ++c)
      {
        double val[NQ], grad[3][NQ];
        evaluate_cell(op.tb, u + c * NQ, val, grad);
        for (int q = 0; q < NQ; ++q)
          {
            const double *Ji  = &op.jinv[(c * NQ + q) * 9];
            const double  JxW = op.jxw[c * NQ + q];
            double        g2  = 0.0;
            for (int i = 0; i < 3; ++i)
              {
                const double gi = Ji[0 * 3 + i] * grad[0][q] + Ji[1 * 3 + i] * grad[1][q] + Ji[2 * 3 + i] * grad[2][q];
                g2 += gi * gi;
              }
            m += val[q] * JxW;
            e += val[q] * val[q] * JxW;
            hs += g2 * JxW;
          }
      }
    out[0] = m, out[1] = e, out[2] = hs;
  }
};

// ------------------------------------------------------------------------
// Dense cross-check implementation
// ------------------------------------------------------------------------

struct DenseCell
{
  int                 n, nq, nf;
  std::vector<double> B, G[3];                 // nq x nq
  std::vector<double> BF[3][2], GF[3][2][3];   // per dir, side: nf x nq

  explicit DenseCell(const Tables &tb)
  {
    n  = tb.n;
    nq = n * n * n;
    nf = n * n;
    B.assign(nq * nq, 0.0);
    for (int j = 0; j < 3; ++j)
      G[j].assign(nq * nq, 0.0);
    for (int q = 0; q < nq; ++q)
      for (int i = 0; i < nq; ++i)
        {
          const int q0 = q % n, q1 = (q / n) % n, q2 = q / (n * n);
          const int i0 = i % n, i1 = (i / n) % n, i2 = i / (n * n);
          B[q * nq + i]    = tb.S[q0][i0] * tb.S[q1][i1] * tb.S[q2][i2];
          G[0][q * nq + i] = tb.D[q0][i0] * tb.S[q1][i1] * tb.S[q2][i2];
          G[1][q * nq + i] = tb.S[q0][i0] * tb.D[q1][i1] * tb.S[q2][i2];
          G[2][q * nq + i] = tb.S[q0][i0] * tb.S[q1][i1] * tb.D[q2][i2];
        }
    for (int d = 0; d < 3; ++d)
      for (int s = 0; s < 2; ++s)
        {
          BF[d][s].assign(nf * nq, 0.0);
          for (int j = 0; j < 3; ++j)
            GF[d][s][j].assign(nf * nq, 0.0);
          const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
          for (int fq = 0; fq < nf; ++fq)
            for (int i = 0; i < nq; ++i)
              {
                const int    ii[3] = {i % n, (i / n) % n, i / (n * n)};
                const int    q1 = fq % n, q2 = fq / n;
                double       v[3], dv[3];
                v[d]   = tb.f[s][ii[d]];
                dv[d]  = tb.df[s][ii[d]];
                v[t1]  = tb.S[q1][ii[t1]];
                dv[t1] = tb.D[q1][ii[t1]];
                v[t2]  = tb.S[q2][ii[t2]];
                dv[t2] = tb.D[q2][ii[t2]];
                BF[d][s][fq * nq + i] = v[0] * v[1] * v[2];
                for (int j = 0; j < 3; ++j)
                  {
                    double w = 1.0;
                    for (int e = 0; e < 3; ++e)
                      w *= e == j ? dv[e] : v[e];
                    GF[d][s][j][fq * nq + i] = w;
                  }
              }
        }
  }
};

void dense_apply(const Op &op, const double *src, double *dst, double t)
{
  const DenseCell dc(op.tb);
  const int       nq = dc.nq, nf = dc.nf;
  const auto     &cfg  = op.ph.cfg;
  const double    skew = cfg.factor_skew, alpha = cfg.flux_alpha, nu = cfg.diffusion;
  const bool      visc = nu != 0.0;
  for (int64_t i = 0; i < op.n_dofs; ++i)
    dst[i] = 0.0;
  std::vector<double> val(nq), gr[3], out(nq);
  for (int j = 0; j < 3; ++j)
    gr[j].resize(nq);
  for (int64_t c = 0; c < op.n_cells; ++c)
    {
      const double *u = src + c * nq;
      for (int q = 0; q < nq; ++q)
        {
          double s = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
          for (int i = 0; i < nq; ++i)
            {
              s += dc.B[q * nq + i] * u[i];
              g0 += dc.G[0][q * nq + i] * u[i];
              g1 += dc.G[1][q * nq + i] * u[i];
              g2 += dc.G[2][q * nq + i] * u[i];
            }
          val[q] = s, gr[0][q] = g0, gr[1][q] = g1, gr[2][q] = g2;
        }
      std::fill(out.begin(), out.end(), 0.0);
      for (int q = 0; q < nq; ++q)
        {
          const double *Ji  = &op.jinv[(c * nq + q) * 9];
          const double  JxW = op.jxw[c * nq + q];
          double        a[3];
          op.ph.speed(&op.xq[(c * nq + q) * 3], t, a);
          double gu[3];
          for (int i = 0; i < 3; ++i)
            gu[i] = Ji[0 * 3 + i] * gr[0][q] + Ji[1 * 3 + i] * gr[1][q] + Ji[2 * 3 + i] * gr[2][q];
          double G[3];
          for (int i = 0; i < 3; ++i)
            G[i] = (1.0 - skew) * a[i] * val[q] - nu * gu[i];
          const double V = -skew * (a[0] * gu[0] + a[1] * gu[1] + a[2] * gu[2]) * JxW;
          double       gref[3];
          for (int j = 0; j < 3; ++j)
            gref[j] = JxW * (Ji[j * 3 + 0] * G[0] + Ji[j * 3 + 1] * G[1] + Ji[j * 3 + 2] * G[2]);
          for (int i = 0; i < nq; ++i)
            out[i] += dc.B[q * nq + i] * V + dc.G[0][q * nq + i] * gref[0] +
                      dc.G[1][q * nq + i] * gref[1] + dc.G[2][q * nq + i] * gref[2];
        }
      for (int i = 0; i < nq; ++i)
        dst[c * nq + i] += out[i];
    }
  const double sigma_base = cfg.penalty_factor * (cfg.degree + 1.0) * (cfg.degree + 1.0);
  for (int64_t fi = 0; fi < (int64_t)op.faces.size(); ++fi)
    {
      const Face &f = op.faces[fi];
      const int   d = f.dir;
      const double sigma = sigma_base / op.h[d];
      for (int q = 0; q < nf; ++q)
        {
          const double *nj  = &op.f_nj[(fi * nf + q) * 3];
          const double *x   = &op.f_x[(fi * nf + q) * 3];
          const double  jxw = op.f_jxw[fi * nf + q];
          const double *Bm  = &dc.BF[d][f.side_minus][q * nq];
          const double *Bp  = &dc.BF[d][f.side_plus][q * nq];
          const double *um = src + f.minus * nq, *upv = f.plus >= 0 ? src + f.plus * nq : nullptr;
          double        u_m = 0.0, u_p = 0.0, grm[3] = {0, 0, 0}, grp[3] = {0, 0, 0};
          for (int i = 0; i < nq; ++i)
            {
              u_m += Bm[i] * um[i];
              if (upv)
                u_p += Bp[i] * upv[i];
              for (int j = 0; j < 3; ++j)
                {
                  grm[j] += dc.GF[d][f.side_minus][j][q * nq + i] * um[i];
                  if (upv)
                    grp[j] += dc.GF[d][f.side_plus][j][q * nq + i] * upv[i];
                }
            }
          if (!upv)
            u_p = op.ph.boundary(x, t);
          double a[3];
          op.ph.speed(x, t, a);
          const double an   = a[0] * nj[0] + a[1] * nj[1] + a[2] * nj[2];
          const double flux = 0.5 * ((u_m + u_p) * an + alpha * std::abs(an) * (u_m - u_p));
          double       vm = -flux + skew * an * u_m, vp = flux - skew * an * u_p;
          double       cm[3] = {0, 0, 0}, cp[3] = {0, 0, 0};
          if (visc)
            {
              double nrm[3];
              for (int i = 0; i < 3; ++i)
                nrm[i] = nj[i] / jxw;
              const double *Jm  = &op.f_jinv_m[(fi * nf + q) * 9];
              double        dnm = 0.0, dnp = 0.0;
              for (int i = 0; i < 3; ++i)
                dnm += nrm[i] * (Jm[i] * grm[0] + Jm[3 + i] * grm[1] + Jm[6 + i] * grm[2]);
              double jump, avg;
              const double *Jp = upv ? &op.f_jinv_p[(fi * nf + q) * 9] : nullptr;
              if (upv)
                {
                  for (int i = 0; i < 3; ++i)
                    dnp += nrm[i] * (Jp[i] * grp[0] + Jp[3 + i] * grp[1] + Jp[6 + i] * grp[2]);
                  jump = u_m - u_p, avg = 0.5 * (dnm + dnp);
                }
              else
                jump = 2.0 * (u_m - u_p), avg = dnm;
              const double pen = (-sigma * nu * jump + nu * avg) * jxw;
              vm += pen, vp -= pen;
              const double cn = 0.5 * nu * jump * jxw;
              for (int j = 0; j < 3; ++j)
                {
                  cm[j] = cn * (Jm[j * 3] * nrm[0] + Jm[j * 3 + 1] * nrm[1] + Jm[j * 3 + 2] * nrm[2]);
                  if (upv)
                    cp[j] = cn * (Jp[j * 3] * nrm[0] + Jp[j * 3 + 1] * nrm[1] + Jp[j * 3 + 2] * nrm[2]);
                }
            }
          for (int i = 0; i < nq; ++i)
            {
              double add = Bm[i] * vm;
              for (int j = 0; j < 3; ++j)
                add += dc.GF[d][f.side_minus][j][q * nq + i] * cm[j];
              dst[f.minus * nq + i] += add;
              if (upv)
                {
                  double addp = Bp[i] * vp;
                  for (int j = 0; j < 3; ++j)
                    addp += dc.GF[d][f.side_plus][j][q * nq + i] * cp[j];
                  dst[f.plus * nq + i] += addp;
                }
            }
        }
    }
}

void dense_inverse_mass(const Op &op, const double *src, double *dst)
{
  const DenseCell     dc(op.tb);
  const int           nq = dc.nq;
  std::vector<double> M(nq * nq), y(nq);
  for (int64_t c = 0; c < op.n_cells; ++c)
    {
      for (int i = 0; i < nq; ++i)
        for (int j = 0; j < nq; ++j)
          {
            double s = 0.0;
            for (int q = 0; q < nq; ++q)
              s += dc.B[q * nq + i] * op.jxw[c * nq + q] * dc.B[q * nq + j];
            M[i * nq + j] = s;
          }
      // Cholesky M = L L^T in place (lower)
      for (int j = 0; j < nq; ++j)
        {
          double s = M[j * nq + j];
          for (int k = 0; k < j; ++k)
            s -= M[j * nq + k] * M[j * nq + k];
          M[j * nq + j] = std::sqrt(s);
          for (int i = j + 1; i < nq; ++i)
            {
              double t = M[i * nq + j];
              for (int k = 0; k < j; ++k)
                t -= M[i * nq + k] * M[j * nq + k];
              M[i * nq + j] = t / M[j * nq + j];
            }
        }
      for (int i = 0; i < nq; ++i)
        {
          double s = src[c * nq + i];
          for (int k = 0; k < i; ++k)
            s -= M[i * nq + k] * y[k];
          y[i] = s / M[i * nq + i];
        }
      for (int i = nq - 1; i >= 0; --i)
        {
          double s = y[i];
          for (int k = i + 1; k < nq; ++k)
            s -= M[k * nq + i] * dst[c * nq + k];
          dst[c * nq + i] = s / M[i * nq + i];
        }
    }
}

// ------------------------------------------------------------------------
// LSRK coefficients: LowStorageRungeKuttaIntegrator (advection_solver.cc:826-898),
// published tables of Kennedy, Carpenter & Lewis (2000) and Tselios & Simos (2007)
// ------------------------------------------------------------------------

int lsrk_tables(int scheme, std::vector<double> &a, std::vector<double> &b)
{
  switch (scheme)
    {
      case ORACLE_LSRK_3_3:
        b = {0.245170287303492, 0.184896052186740, 0.569933660509768};
        a = {0.755726351946097, 0.386954477304099};
        return 0;
      case ORACLE_LSRK_5_4:
        b = {1153189308089. / 22510343858157., 1772645290293. / 4653164025191.,
             -1672844663538. / 4480602732383., 2114624349019. / 3568978502595.,
             5198255086312. / 14908931495163.};
        a = {970286171893. / 4311952581923., 6584761158862. / 12103376702013.,
             2251764453980. / 15575788980749., 26877169314380. / 34165994151039.};
        return 0;
      case ORACLE_LSRK_7_4:
        b = {0.0941840925477795334, 0.149683694803496998, 0.285204742060440058,
             -0.122201846148053668, 0.0605151571191401122, 0.345986987898399296,
             0.186627171718797670};
        a = {0.241566650129646868 + b[0], 0.0423866513027719953 + b[1],
             0.215602732678803776 + b[2], 0.232328007537583987 + b[3],
             0.256223412574146438 + b[4], 0.0978694102142697230 + b[5]};
        return 0;
      case ORACLE_LSRK_9_5:
        b = {2274579626619. / 23610510767302., 693987741272. / 12394497460941.,
             -347131529483. / 15096185902911., 1144057200723. / 32081666971178.,
             1562491064753. / 11797114684756., 13113619727965. / 44346030145118.,
             393957816125. / 7825732611452., 720647959663. / 6565743875477.,
             3559252274877. / 14424734981077.};
        a = {1107026461565. / 5417078080134., 38141181049399. / 41724347789894.,
             493273079041. / 11940823631197., 1851571280403. / 6147804934346.,
             11782306865191. / 62590030070788., 9452544825720. / 13648368537481.,
             4435885630781. / 26285702406235., 2357909744247. / 11371140753790.};
        return 0;
      default:
        return 1;
    }
}

template <template <int> class F, typename... Args>
void dispatch(int n, Args &&...args)
{
  switch (n)
    {
      case 2: F<2>::run(args...); break;
      case 3: F<3>::run(args...); break;
      case 4: F<4>::run(args...); break;
      case 5: F<5>::run(args...); break;
      case 6: F<6>::run(args...); break;
      case 7: F<7>::run(args...); break;
      default: break;
    }
}

// cellwise mass matrix S^T diag(JxW) S
template <int N>
struct RunMass
{
  static void run(const Op &op, const double *src, double *dst)
  {
    constexpr int NQ = N * N * N;
    const Tables &tb = op.tb;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < op.n_cells; ++c)
      {
        double t1[NQ], t2[NQ];
        apply3<N, 0, false, false>(tb.S, src + c * NQ, t1);
        apply3<N, 1, false, false>(tb.S, t1, t2);
        apply3<N, 2, false, false>(tb.S, t2, t1);
        for (int q = 0; q < NQ; ++q)
          t1[q] *= op.jxw[c * NQ + q];
        apply3<N, 0, true, false>(tb.S, t1, t2);
        apply3<N, 1, true, false>(tb.S, t2, t1);
        apply3<N, 2, true, false>(tb.S, t1, dst + c * NQ);
      }
  }
};

// CellwisePreconditionerFDM (advection_solver_implicit.cc:490-646) inside the
// block-Jacobi loop of precondition_block_jacobi (:1283-1340)
template <int N>
struct RunFdm
{
  static void run(const Op &op, const double *lam, const double *Vt, const double *VWt, const double *src,
                  double *dst, double mass_factor)
  {
    using cd         = std::complex<double>;
    constexpr int NQ = N * N * N;
    const Tables &tb = op.tb;
    cd            L[2][N], V[2][N][N], VW[2][N][N];
    for (int s = 0; s < 2; ++s)
      for (int i = 0; i < N; ++i)
        {
          L[s][i] = cd(lam[s * 2 * N + 2 * i], lam[s * 2 * N + 2 * i + 1]);
          for (int j = 0; j < N; ++j)
            {
              V[s][i][j]  = cd(Vt[s * 2 * N * N + 2 * (i * N + j)], Vt[s * 2 * N * N + 2 * (i * N + j) + 1]);
              VW[s][i][j] = cd(VWt[s * 2 * N * N + 2 * (i * N + j)], VWt[s * 2 * N * N + 2 * (i * N + j) + 1]);
            }
        }
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < op.n_cells; ++c)
      {
        // average contravariant velocity and volume of the cell
        double v[3] = {0, 0, 0}, vol = 0.0;
        for (int q = 0; q < NQ; ++q)
          {
            const double *Ji = &op.jinv[(c * NQ + q) * 9];
            double        a[3];
            op.ph.speed(&op.xq[(c * NQ + q) * 3], 0.0, a);
            const double JxW = op.jxw[c * NQ + q];
            for (int d = 0; d < 3; ++d)
              v[d] += (Ji[d * 3 + 0] * a[0] + Ji[d * 3 + 1] * a[1] + Ji[d * 3 + 2] * a[2]) * JxW;
            vol += JxW;
          }
        int sg[3];
        for (int d = 0; d < 3; ++d)
          {
            v[d] /= vol;
            sg[d] = v[d] < 0.0 ? 1 : 0;
          }
        // residual to the collocation basis: S^{-T}
        double t1[NQ], t2[NQ];
        apply3<N, 0, true, false>(tb.Si, src + c * NQ, t1);
        apply3<N, 1, true, false>(tb.Si, t1, t2);
        apply3<N, 2, true, false>(tb.Si, t2, t1);
        cd x[NQ], y[NQ];
        for (int q = 0; q < NQ; ++q)
          x[q] = t1[q];
        // V^{-1} W^{-1} in each direction
        for (int d = 0; d < 3; ++d)
          {
            const int st = d == 0 ? 1 : d == 1 ? N : N * N;
            for (int q = 0; q < NQ; ++q)
              {
                const int id = (q / st) % N, base = q - id * st;
                cd        s  = 0.0;
                for (int k = 0; k < N; ++k)
                  s += VW[sg[d]][id][k] * x[base + k * st];
                y[q] = s;
              }
            std::copy(y, y + NQ, x);
          }
        for (int q = 0; q < NQ; ++q)
          {
            const int ii[3] = {q % N, (q / N) % N, q / (N * N)};
            cd        diag  = mass_factor;
            for (int d = 0; d < 3; ++d)
              diag += v[d] * L[sg[d]][ii[d]];
            x[q] *= (1.0 / vol) / diag;
          }
        for (int d = 0; d < 3; ++d)
          {
            const int st = d == 0 ? 1 : d == 1 ? N : N * N;
            for (int q = 0; q < NQ; ++q)
              {
                const int id = (q / st) % N, base = q - id * st;
                cd        s  = 0.0;
                for (int k = 0; k < N; ++k)
                  s += V[sg[d]][id][k] * x[base + k * st];
                y[q] = s;
              }
            std::copy(y, y + NQ, x);
          }
        for (int q = 0; q < NQ; ++q)
          t1[q] = x[q].real();
        // back to the nodal basis: S^{-1}
        apply3<N, 0, false, false>(tb.Si, t1, t2);
        apply3<N, 1, false, false>(tb.Si, t2, t1);
        apply3<N, 2, false, false>(tb.Si, t1, dst + c * NQ);
      }
  }
};

template <int N> struct RunApply { static void run(const Op &op, const double *s, double *d, double t) { Kernels<N>::apply_unscaled(op, s, d, t); } };
template <int N> struct RunInvMass { static void run(const Op &op, const double *s, double *d) { Kernels<N>::inverse_mass(op, s, d); } };
template <int N> struct RunProject { static void run(const Op &op, double t, double *d) { Kernels<N>::project(op, t, d); } };
template <int N> struct RunMassEnergy { static void run(const Op &op, const double *u, double *o) { Kernels<N>::mass_energy(op, u, o); } };

} // namespace

struct oracle_op
{
  Op op;
  std::vector<double> tmp;
};

extern "C" {

int oracle_create(const oracle_config *cfg, oracle_op **out)
{
  if (!cfg || !out)
    return 1;
  auto h = std::make_unique<oracle_op>();
  if (int e = h->op.setup(*cfg))
    return e;
  *out = h.release();
  return 0;
}

void oracle_destroy(oracle_op *op) { delete op; }

int64_t oracle_n_dofs(const oracle_op *op) { return op->op.n_dofs; }
int64_t oracle_n_cells(const oracle_op *op) { return op->op.n_cells; }
void    oracle_set_num_threads(int n) { omp_set_num_threads(n); }
int     oracle_get_max_threads(void) { return omp_get_max_threads(); }

int oracle_tables(int degree, double *gl, double *gp, double *gw, double *S, double *D, double *Sinv)
{
  if (degree < 1 || degree > 6)
    return 1;
  Tables tb;
  tb.init(degree);
  const int n = tb.n;
  for (int i = 0; i < n; ++i)
    gl[i] = tb.gl[i], gp[i] = tb.gp[i], gw[i] = tb.gw[i];
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i)
      S[q * n + i] = tb.S[q][i], D[q * n + i] = tb.D[q][i], Sinv[q * n + i] = tb.Si[q][i];
  return 0;
}

int oracle_apply_unscaled(oracle_op *h, const double *src, double *dst, double t)
{
  if (src == dst)
    return 2;
  dispatch<RunApply>(h->op.n, h->op, src, dst, t);
  return 0;
}

int oracle_inverse_mass(oracle_op *h, const double *src, double *dst)
{
  dispatch<RunInvMass>(h->op.n, h->op, src, dst);
  return 0;
}

int oracle_apply(oracle_op *h, const double *src, double *dst, double t)
{
  if (src == dst)
    {
      h->tmp.resize(h->op.n_dofs);
      dispatch<RunApply>(h->op.n, h->op, src, h->tmp.data(), t);
      dispatch<RunInvMass>(h->op.n, h->op, h->tmp.data(), dst);
      return 0;
    }
  dispatch<RunApply>(h->op.n, h->op, src, dst, t);
  dispatch<RunInvMass>(h->op.n, h->op, dst, dst);
  return 0;
}

// AdvectionOperation::perform_stage, advection_solver.cc:695-756: loop into
// vec_ki, cell_loop of the inverse mass into next_ri, then the post-lambda
// u += b k; next_ri = u_old + a k (a == 0: only u).
int oracle_perform_stage(oracle_op *h, double t, double b_dt, double a_dt, const double *r_in,
                         double *k, double *u, double *r_out)
{
  Op &op = h->op;
  if (r_out == u)
    return 2;
  double *kbuf = k;
  if (k == r_in)
    {
      h->tmp.resize(op.n_dofs);
      kbuf = h->tmp.data();
    }
  dispatch<RunApply>(op.n, op, r_in, kbuf, t);
  dispatch<RunInvMass>(op.n, op, kbuf, r_out);
  const int64_t nd = op.n_dofs;
  if (a_dt == 0.0)
    {
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < nd; ++i)
        u[i] = u[i] + b_dt * r_out[i];
    }
  else
    {
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < nd; ++i)
        {
          const double ki = r_out[i], si = u[i];
          u[i]            = si + b_dt * ki;
          r_out[i]        = si + a_dt * ki;
        }
    }
  return 0;
}

int oracle_lsrk_coefficients(int scheme, double *a, double *b, int *n_stages)
{
  std::vector<double> av, bv;
  if (lsrk_tables(scheme, av, bv))
    return 1;
  for (size_t i = 0; i < av.size(); ++i)
    a[i] = av[i];
  for (size_t i = 0; i < bv.size(); ++i)
    b[i] = bv[i];
  *n_stages = (int)bv.size();
  return 0;
}

// LowStorageRungeKuttaIntegrator::perform_time_step, advection_solver.cc:906-939
int oracle_lsrk_step(oracle_op *h, int scheme, double t, double dt, double *u, double *r, double *k)
{
  std::vector<double> ai, bi;
  if (lsrk_tables(scheme, ai, bi))
    return 1;
  oracle_perform_stage(h, t, bi[0] * dt, ai[0] * dt, u, r, u, r);
  double sum_previous_bi = 0.0;
  for (size_t s = 1; s < bi.size(); ++s)
    {
      const double c_i = sum_previous_bi + ai[s - 1];
      oracle_perform_stage(h, t + c_i * dt, bi[s] * dt, s == bi.size() - 1 ? 0.0 : ai[s] * dt, r,
                           k, u, r);
      sum_previous_bi += bi[s - 1];
    }
  return 0;
}

int oracle_project(oracle_op *h, double t, double *dst)
{
  dispatch<RunProject>(h->op.n, h->op, t, dst);
  return 0;
}

int oracle_mass_energy(oracle_op *h, const double *u, double out[3])
{
  dispatch<RunMassEnergy>(h->op.n, h->op, u, out);
  return 0;
}

// VectorTools::integrate_difference with QGauss(k+2) for the error and
// QGauss(k+1) for the norm of the exact solution (advection_solver.cc:1183-1208)
int oracle_l2_error(oracle_op *h, const double *u, double t, double out[2])
{
  const Op &op = h->op;
  const int n = op.n, m = n + 1, nq = n * n * n;
  double    ep[MAXN + 1], ew[MAXN + 1];
  gauss_points(m, ep, ew);
  std::vector<double> SE(m * n);
  for (int q = 0; q < m; ++q)
    for (int i = 0; i < n; ++i)
      SE[q * n + i] = lagrange(op.tb.gl, n, i, ep[q]);
  double err2 = 0.0, nrm2 = 0.0;
#pragma omp parallel reduction(+ : err2, nrm2)
  {
    std::vector<double> X(3 * nq);
#pragma omp for schedule(static)
    for (int64_t c = 0; c < op.n_cells; ++c)
      {
        op.support_points(c, X.data());
        const double *uc = u + c * nq;
        for (int q2 = 0; q2 < m; ++q2)
          for (int q1 = 0; q1 < m; ++q1)
            for (int q0 = 0; q0 < m; ++q0)
              {
                const double xi[3] = {ep[q0], ep[q1], ep[q2]};
                double       x[3], J[3][3], Ji[9];
                op.map_point(c, X.data(), xi, x, J);
                const double det = Op::inverse3(J, Ji);
                double       uh  = 0.0;
                for (int i2 = 0; i2 < n; ++i2)
                  for (int i1 = 0; i1 < n; ++i1)
                    {
                      const double w = SE[q1 * n + i1] * SE[q2 * n + i2];
                      for (int i0 = 0; i0 < n; ++i0)
                        uh += w * SE[q0 * n + i0] * uc[i0 + n * (i1 + n * i2)];
                    }
                const double ue = op.ph.exact(x, t);
                err2 += (uh - ue) * (uh - ue) * det * ew[q0] * ew[q1] * ew[q2];
              }
        for (int q = 0; q < nq; ++q)
          {
            const double ue = op.ph.exact(&op.xq[(c * nq + q) * 3], t);
            nrm2 += ue * ue * op.jxw[c * nq + q];
          }
      }
  }
  out[0] = std::sqrt(err2);
  out[1] = std::sqrt(nrm2);
  return 0;
}

double oracle_min_vertex_distance(oracle_op *h)
{
  const Op &op = h->op;
  double    hmin = 1e300;
#pragma omp parallel for schedule(static) reduction(min : hmin)
  for (int64_t c = 0; c < op.n_cells; ++c)
    {
      double lo[3], v[8][3];
      op.cell_lo(c, lo);
      for (int k = 0; k < 8; ++k)
        {
          const double x[3] = {lo[0] + op.h[0] * (k & 1), lo[1] + op.h[1] * ((k >> 1) & 1),
                               lo[2] + op.h[2] * ((k >> 2) & 1)};
          if (op.curved)
            op.ph.deform(x, v[k]);
          else
            v[k][0] = x[0], v[k][1] = x[1], v[k][2] = x[2];
        }
      for (int a = 0; a < 8; ++a)
        for (int b = a + 1; b < 8; ++b)
          {
            const double dx = v[a][0] - v[b][0], dy = v[a][1] - v[b][1], dz = v[a][2] - v[b][2];
            hmin            = std::min(hmin, std::sqrt(dx * dx + dy * dy + dz * dz));
          }
    }
  return hmin;
}

// setup_dofs time step, advection_solver.cc:1155-1165 (before the rounding to
// FINAL_TIME / ceil(FINAL_TIME / dt))
double oracle_time_step(oracle_op *h, double courant)
{
  // advective limit: setup_dofs, advection_solver.cc:1155-1165
  const double *a     = h->op.ph.cfg.velocity;
  const double  anrm  = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double  k     = std::max(1, h->op.ph.cfg.degree);
  const double  hmin  = oracle_min_vertex_distance(h);
  const double  dt_a  = courant * hmin / anrm / std::pow(k, 1.5);
  // with SIPG diffusion nu, the explicit limit 0.3 h^2 / (nu (k+1)^4) is
  // combined harmonically (a builder rule: the reference integrates its
  // advection-diffusion problem implicitly, advection_diffusion_solver.cc:1463)
  const double nu = h->op.ph.cfg.diffusion;
  const double k1 = h->op.ph.cfg.degree + 1.0;
  if (!(nu > 0.0))
    return dt_a;
  const double dt_d = 0.3 * hmin * hmin / (nu * k1 * k1 * k1 * k1);
  return anrm > 0.0 ? 1.0 / (1.0 / dt_a + 1.0 / dt_d) : dt_d;
}

int oracle_support_points(oracle_op *h, double *xyz)
{
  const Op &op = h->op;
  const int nq = op.n * op.n * op.n;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < op.n_cells; ++c)
    op.support_points(c, xyz + c * nq * 3);
  return 0;
}

int oracle_interpolate(oracle_op *h, double t, double *dst)
{
  const Op &op = h->op;
  const int nq = op.n * op.n * op.n;
#pragma omp parallel
  {
    std::vector<double> X(3 * nq);
#pragma omp for schedule(static)
    for (int64_t c = 0; c < op.n_cells; ++c)
      {
        op.support_points(c, X.data());
        for (int i = 0; i < nq; ++i)
          dst[c * nq + i] = op.ph.exact(&X[3 * i], t);
      }
  }
  return 0;
}

int oracle_apply_mass(oracle_op *h, const double *src, double *dst)
{
  if (src == dst)
    return 2;
  dispatch<RunMass>(h->op.n, h->op, src, dst);
  return 0;
}

int oracle_vmult(oracle_op *h, const double *src, double *dst, double mass_factor, double t)
{
  if (src == dst)
    return 2;
  const int64_t nd = h->op.n_dofs;
  h->tmp.resize(nd);
  dispatch<RunApply>(h->op.n, h->op, src, h->tmp.data(), t);
  dispatch<RunMass>(h->op.n, h->op, src, dst);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nd; ++i)
    dst[i] = mass_factor * dst[i] - h->tmp[i];
  return 0;
}

int oracle_fdm_apply(oracle_op *h, const double *lambda, const double *V, const double *VinvW,
                     const double *src, double *dst, double mass_factor)
{
  if (src == dst)
    return 2;
  dispatch<RunFdm>(h->op.n, h->op, lambda, V, VinvW, src, dst, mass_factor);
  return 0;
}

int oracle_apply_unscaled_dense(oracle_op *h, const double *src, double *dst, double t)
{
  if (src == dst)
    return 2;
  dense_apply(h->op, src, dst, t);
  return 0;
}

int oracle_inverse_mass_dense(oracle_op *h, const double *src, double *dst)
{
  if (src == dst)
    return 2;
  dense_inverse_mass(h->op, src, dst);
  return 0;
}

} // extern "C"
