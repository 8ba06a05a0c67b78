#include "geometry.h"

#include <algorithm>
#include <cmath>

namespace adv
{
namespace
{
constexpr double kPi = 3.14159265358979323846;

// Position x and Jacobian J[i][j] = dx_i / dxi_j of the degree-k mapping with
// support points X (n^3 points x 3, x fastest) at a tensor grid of reference
// points; V_d / W_d hold the nodal basis values / derivatives at the np_d
// points of direction d.  Output per point p = p0 + np0 (p1 + np1 p2):
// x[3 p + i], J[9 p + 3 i + j].
void map_grid(int n, const double *X, int np0, const double *V0, const double *W0, int np1,
              const double *V1, const double *W1, int np2, const double *V2, const double *W2,
              double *x, double *J)
{
  std::vector<double> A(np2 * n * n * 3), Az(np2 * n * n * 3);
  for (int p2 = 0; p2 < np2; ++p2)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a)
        for (int i = 0; i < 3; ++i)
          {
            double s = 0.0, sd = 0.0;
            for (int c = 0; c < n; ++c)
              {
                const double v = X[3 * (a + n * (b + n * c)) + i];
                s += V2[p2 * n + c] * v;
                sd += W2[p2 * n + c] * v;
              }
            A[((p2 * n + b) * n + a) * 3 + i]  = s;
            Az[((p2 * n + b) * n + a) * 3 + i] = sd;
          }
  std::vector<double> B(np2 * np1 * n * 3), By(B.size()), Bz(B.size());
  for (int p2 = 0; p2 < np2; ++p2)
    for (int p1 = 0; p1 < np1; ++p1)
      for (int a = 0; a < n; ++a)
        for (int i = 0; i < 3; ++i)
          {
            double s = 0.0, sy = 0.0, sz = 0.0;
            for (int b = 0; b < n; ++b)
              {
                const int k = ((p2 * n + b) * n + a) * 3 + i;
                s += V1[p1 * n + b] * A[k];
                sy += W1[p1 * n + b] * A[k];
                sz += V1[p1 * n + b] * Az[k];
              }
            const int o = ((p2 * np1 + p1) * n + a) * 3 + i;
            B[o] = s, By[o] = sy, Bz[o] = sz;
          }
  for (int p2 = 0; p2 < np2; ++p2)
    for (int p1 = 0; p1 < np1; ++p1)
      for (int p0 = 0; p0 < np0; ++p0)
        {
          const int p = p0 + np0 * (p1 + np1 * p2);
          for (int i = 0; i < 3; ++i)
            {
              double s = 0.0, s0 = 0.0, s1 = 0.0, s2 = 0.0;
              for (int a = 0; a < n; ++a)
                {
                  const int k = ((p2 * np1 + p1) * n + a) * 3 + i;
                  s += V0[p0 * n + a] * B[k];
                  s0 += W0[p0 * n + a] * B[k];
                  s1 += V0[p0 * n + a] * By[k];
                  s2 += V0[p0 * n + a] * Bz[k];
                }
              x[3 * p + i]         = s;
              J[9 * p + 3 * i + 0] = s0;
              J[9 * p + 3 * i + 1] = s1;
              J[9 * p + 3 * i + 2] = s2;
            }
        }
}

double det_inverse(const double *J, double *Ji)
{
  const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
  const double id = 1.0 / det;
  Ji[0] = (J[4] * J[8] - J[5] * J[7]) * id;
  Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id;
  Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
  Ji[3] = (J[5] * J[6] - J[3] * J[8]) * id;
  Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id;
  Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
  Ji[6] = (J[3] * J[7] - J[4] * J[6]) * id;
  Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id;
  Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
  return det;
}

// map_grid on the support points relative to the cell's first support point
// X[0..2], with that point added back to the positions.  The Jacobian is a
// derivative of the interpolant (the derivative weights sum to zero): summed
// over absolute coordinates of size ~1 it cancels to entries of size ~h and
// carries rounding of a few ulps of 1, which depends on the order of the sums
// (about 4e-13 relative at h = 1/64); relative coordinates are of size ~h,
// so that rounding drops to a few ulps of the entries themselves.
void map_grid_rel(int n, double *X, int np0, const double *V0, const double *W0, int np1, const double *V1,
                  const double *W1, int np2, const double *V2, const double *W2, double *x, double *J)
{
  const int    nq    = n * n * n;
  const double x0[3] = {X[0], X[1], X[2]};
  for (int p = 0; p < nq; ++p)
    for (int i = 0; i < 3; ++i)
      X[3 * p + i] -= x0[i];
  map_grid(n, X, np0, V0, W0, np1, V1, W1, np2, V2, W2, x, J);
  for (int p = 0; p < np0 * np1 * np2; ++p)
    for (int i = 0; i < 3; ++i)
      x[3 * p + i] += x0[i];
}

// support points of the cell with global indices (ix, iy, iz)
void cell_support_points(const adv_config &cfg, const Mesh &m, const Tables1D &tb, int ix, int iy, int iz,
                         double *X)
{
  const int    n     = m.n;
  const double lo[3] = {m.lo[0] + ix * m.h[0], m.lo[1] + iy * m.h[1], m.lo[2] + iz * m.h[2]};
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        {
          const double p[3] = {lo[0] + m.h[0] * tb.gl[i], lo[1] + m.h[1] * tb.gl[j],
                               lo[2] + m.h[2] * tb.gl[k]};
          double      *y    = X + 3 * (i + n * (j + n * k));
          if (m.curved)
            deform_point(cfg, m.L, p, y);
          else
            y[0] = p[0], y[1] = p[1], y[2] = p[2];
        }
}

// support points of local cell c
void cell_support_points(const adv_config &cfg, const Mesh &m, const Tables1D &tb, int64_t c, double *X)
{
  cell_support_points(cfg, m, tb, int(c % m.nc[0]), int((c / m.nc[0]) % m.nc[1]),
                      int(c / ((int64_t)m.nc[0] * m.nc[1])) + m.zoff, X);
}
} // namespace

void deform_point(const adv_config &cfg, const double L[3], const double x[3], double y[3])
{
  double s[3];
  for (int d = 0; d < 3; ++d)
    s[d] = (x[d] - cfg.domain_lo[d]) / L[d];
  for (int d = 0; d < 3; ++d)
    y[d] = x[d] + cfg.deformation * L[d] * std::sin(2.0 * kPi * s[(d + 1) % 3]) *
                    std::sin(2.0 * kPi * s[(d + 2) % 3]);
}

void velocity_field(const adv_config &cfg, const double x[3], double b[3])
{
  if (cfg.velocity_type == ADV_VELOCITY_CONSTANT)
    {
      b[0] = cfg.velocity[0], b[1] = cfg.velocity[1], b[2] = cfg.velocity[2];
      return;
    }
  const double sx = std::sin(kPi * x[0]), sy = std::sin(kPi * x[1]);
  b[0] = cfg.velocity[0] * sx * sx * std::sin(2.0 * kPi * x[1]);
  b[1] = -cfg.velocity[1] * sy * sy * std::sin(2.0 * kPi * x[0]);
  b[2] = cfg.velocity[2];
}

void support_points(const adv_config &cfg, const Mesh &m, const Tables1D &tb, int64_t c, double *X)
{
  cell_support_points(cfg, m, tb, c, X);
}

int setup_mesh(const adv_config &cfg, Mesh &m)
{
  m.n        = cfg.degree + 1;
  m.curved   = cfg.mesh_type == ADV_MESH_DEFORMED;
  m.periodic = cfg.periodic != 0;
  m.uniform  = !m.curved && cfg.velocity_type == ADV_VELOCITY_CONSTANT && cfg.diffusion == 0.0;
  m.n_cells  = 1;
  for (int d = 0; d < 3; ++d)
    {
      m.nc[d] = cfg.n_cells[d];
      m.lo[d] = cfg.domain_lo[d];
      m.L[d]  = cfg.domain_hi[d] - cfg.domain_lo[d];
      m.h[d]  = m.L[d] / m.nc[d];
      m.n_cells *= m.nc[d];
    }
  m.pmask = m.periodic ? 7 : 0;
  for (int d = 0; d < 3; ++d)
    {
      m.npos[d]    = m.periodic ? m.nc[d] : m.nc[d] + 1;
      m.n_faces[d] = (int64_t)m.npos[d] * m.nc[m.t1(d)] * m.nc[m.t2(d)];
    }
  m.n_dofs     = m.n_cells * m.n * m.n * m.n;
  m.cell_begin = 0;
  m.cell_end   = m.n_cells;
  m.gnz        = m.nc[2];
  return 0;
}

int setup_slab(const adv_config &cfg, int z_begin, int z_end, Mesh &m)
{
  setup_mesh(cfg, m);
  const int nz = cfg.n_cells[2];
  if (z_begin < 0 || z_end > nz || z_begin >= z_end)
    return -1;
  m.slab     = true;
  m.ghost_lo = m.periodic || z_begin > 0;
  m.ghost_hi = m.periodic || z_end < nz;
  m.zoff     = z_begin - (m.ghost_lo ? 1 : 0);
  m.nc[2]    = (z_end - z_begin) + (m.ghost_lo ? 1 : 0) + (m.ghost_hi ? 1 : 0);
  m.pmask    = m.periodic ? 3 : 0; // z neighbours come from the ghost layers
  m.n_cells  = (int64_t)m.nc[0] * m.nc[1] * m.nc[2];
  for (int d = 0; d < 3; ++d)
    {
      m.npos[d]    = ((m.pmask >> d) & 1) ? m.nc[d] : m.nc[d] + 1;
      m.n_faces[d] = (int64_t)m.npos[d] * m.nc[m.t1(d)] * m.nc[m.t2(d)];
    }
  m.n_dofs     = m.n_cells * m.n * m.n * m.n;
  const int64_t layer = (int64_t)m.nc[0] * m.nc[1];
  m.cell_begin = m.ghost_lo ? layer : 0;
  m.cell_end   = m.cell_begin + layer * (z_end - z_begin);
  return 0;
}

void compute_geometry(const adv_config &cfg, const Mesh &m, const Tables1D &tb, HostGeometry &g)
{
  const int    n = m.n, nq = n * n * n, nf = n * n;
  const double alpha = cfg.flux_alpha;

  // minimum vertex distance over all cells (setup_dofs, advection_solver.cc:1155-1160)
  double hmin = 1e300;
#pragma omp parallel for reduction(min : hmin) schedule(static)
  for (int64_t c = m.cell_begin; c < m.cell_end; ++c)
    {
      const int ix = int(c % m.nc[0]), iy = int((c / m.nc[0]) % m.nc[1]),
                iz = int(c / ((int64_t)m.nc[0] * m.nc[1])) + m.zoff;
      double v[8][3];
      for (int k = 0; k < 8; ++k)
        {
          const double p[3] = {m.lo[0] + (ix + (k & 1)) * m.h[0], m.lo[1] + (iy + ((k >> 1) & 1)) * m.h[1],
                               m.lo[2] + (iz + ((k >> 2) & 1)) * m.h[2]};
          if (m.curved)
            deform_point(cfg, m.L, p, v[k]);
          else
            v[k][0] = p[0], v[k][1] = p[1], v[k][2] = p[2];
        }
      for (int a = 0; a < 8; ++a)
        for (int b = a + 1; b < 8; ++b)
          {
            const double dx = v[a][0] - v[b][0], dy = v[a][1] - v[b][1], dz = v[a][2] - v[b][2];
            hmin            = std::min(hmin, std::sqrt(dx * dx + dy * dy + dz * dz));
          }
    }
  g.h_min = hmin;

  g.fdm_cell.assign((size_t)m.n_cells * 4, 0.0);
  if (m.uniform)
    {
      const double V = m.h[0] * m.h[1] * m.h[2];
      for (int64_t c = 0; c < m.n_cells; ++c)
        {
          for (int d = 0; d < 3; ++d)
            g.fdm_cell[4 * c + d] = cfg.velocity[d] / m.h[d];
          g.fdm_cell[4 * c + 3] = 1.0 / V;
        }
    }
  if (m.uniform)
    {
      const double V = m.h[0] * m.h[1] * m.h[2];
      g.idet_const   = 1.0 / V;
      for (int d = 0; d < 3; ++d)
        {
          g.cv[d] = cfg.velocity[d] / m.h[d];
          g.P[d]  = 0.5 * (g.cv[d] + alpha * std::fabs(g.cv[d]));
          g.M[d]  = 0.5 * (g.cv[d] - alpha * std::fabs(g.cv[d]));
        }
    }
  else
    {
      g.cell.assign((size_t)m.n_cells * 4 * nq, 0.0);
      double S[kMaxN * kMaxN], Sd[kMaxN * kMaxN];
      for (int q = 0; q < n; ++q)
        for (int i = 0; i < n; ++i)
          S[q * n + i] = tb.S[q][i], Sd[q * n + i] = tb.Sd[q][i];
#pragma omp parallel
      {
        std::vector<double> X(3 * nq), x(3 * nq), J(9 * nq);
#pragma omp for schedule(static)
        for (int64_t c = 0; c < m.n_cells; ++c)
          {
            cell_support_points(cfg, m, tb, c, X.data());
            map_grid_rel(n, X.data(), n, S, Sd, n, S, Sd, n, S, Sd, x.data(), J.data());
            double *out = &g.cell[(size_t)c * 4 * nq];
            double  vavg[3] = {0.0, 0.0, 0.0}, vol = 0.0;
            for (int q = 0; q < nq; ++q)
              {
                double       Ji[9], b[3];
                const double det = det_inverse(&J[9 * q], Ji);
                velocity_field(cfg, &x[3 * q], b);
                const double w = tb.gw[q % n] * tb.gw[(q / n) % n] * tb.gw[q / (n * n)];
                for (int d = 0; d < 3; ++d)
                  {
                    out[d * nq + q] = det * (Ji[3 * d + 0] * b[0] + Ji[3 * d + 1] * b[1] + Ji[3 * d + 2] * b[2]);
                    vavg[d] += out[d * nq + q] * w;
                  }
                out[3 * nq + q] = 1.0 / det;
                vol += det * w;
              }
            for (int d = 0; d < 3; ++d)
              g.fdm_cell[4 * c + d] = vavg[d] / vol;
            g.fdm_cell[4 * c + 3] = 1.0 / vol;
          }
      }
    }

  // faces: coefficients (field case) and Dirichlet point positions
  for (int d = 0; d < 3; ++d)
    {
      const bool need_coef = !m.uniform;
      const bool need_x    = !m.periodic;
      if (!need_coef && !need_x)
        continue;
      if (need_coef)
        g.face[d].assign((size_t)m.n_faces[d] * 2 * nf, 0.0);
      if (need_x)
        g.face_x[d].assign((size_t)m.n_faces[d] * 3 * nf, 0.0);
      const int t1 = m.t1(d), t2 = m.t2(d);
#pragma omp parallel
      {
        std::vector<double> X(3 * nq), x(3 * nf), J(9 * nf);
        double              V[3][kMaxN * kMaxN], W[3][kMaxN * kMaxN];
#pragma omp for schedule(static)
        for (int64_t f = 0; f < m.n_faces[d]; ++f)
          {
            const int p  = int(f % m.npos[d]);
            const int j1 = int((f / m.npos[d]) % m.nc[t1]);
            const int j2 = int(f / ((int64_t)m.npos[d] * m.nc[t1]));
            const bool wrap     = (m.pmask >> d) & 1;
            const bool boundary = !wrap && (p == 0 || p == m.nc[d]);
            if (!need_coef && !boundary)
              continue;
            // the cell on the low side (or the only cell of a boundary face)
            int ijk[3];
            ijk[t1] = j1, ijk[t2] = j2;
            int side;
            if (wrap)
              ijk[d] = (p - 1 + m.nc[d]) % m.nc[d], side = 1;
            else if (p == 0)
              ijk[d] = 0, side = 0;
            else
              ijk[d] = p - 1, side = 1;
            // global z index of that cell: a slab takes the cell the whole
            // mesh takes (across a periodic seam the wrapped one), so that
            // both compute bit-identical face data
            int gz = ijk[2] + m.zoff;
            if (d == 2 && m.slab)
              {
                const int pg = p + m.zoff;
                if (m.periodic)
                  gz = (pg - 1 + m.gnz) % m.gnz, side = 1;
                else if (pg == 0)
                  gz = 0, side = 0;
                else
                  gz = pg - 1, side = 1;
              }
            cell_support_points(cfg, m, tb, ijk[0], ijk[1], gz, X.data());
            // 1D tables: normal direction at xi_d = side, tangential at the Gauss points
            int np[3];
            for (int e = 0; e < 3; ++e)
              {
                if (e == d)
                  {
                    np[e] = 1;
                    for (int a = 0; a < n; ++a)
                      {
                        V[e][a] = lagrange(tb.gl, n, a, double(side));
                        W[e][a] = lagrange_derivative(tb.gl, n, a, double(side));
                      }
                  }
                else
                  {
                    np[e] = n;
                    for (int q = 0; q < n; ++q)
                      for (int a = 0; a < n; ++a)
                        V[e][q * n + a] = tb.S[q][a], W[e][q * n + a] = tb.Sd[q][a];
                  }
              }
            map_grid_rel(n, X.data(), np[0], V[0], W[0], np[1], V[1], W[1], np[2], V[2], W[2], x.data(),
                         J.data());
            // grid point (p0, p1, p2) -> face point (q1 along t1, q2 along t2)
            for (int q2 = 0; q2 < n; ++q2)
              for (int q1 = 0; q1 < n; ++q1)
                {
                  int pp[3];
                  pp[d] = 0, pp[t1] = q1, pp[t2] = q2;
                  const int gpt = pp[0] + np[0] * (pp[1] + np[1] * pp[2]);
                  const int fq  = q1 + n * q2;
                  if (need_coef)
                    {
                      double       Ji[9], b[3];
                      const double det = det_inverse(&J[9 * gpt], Ji);
                      velocity_field(cfg, &x[3 * gpt], b);
                      const double cc = det * (Ji[3 * d + 0] * b[0] + Ji[3 * d + 1] * b[1] + Ji[3 * d + 2] * b[2]);
                      // (P, M) pairs per face point: one 16-byte load in the kernels
                      g.face[d][(size_t)f * 2 * nf + 2 * fq]     = 0.5 * (cc + alpha * std::fabs(cc));
                      g.face[d][(size_t)f * 2 * nf + 2 * fq + 1] = 0.5 * (cc - alpha * std::fabs(cc));
                    }
                  if (need_x && boundary)
                    for (int i = 0; i < 3; ++i)
                      g.face_x[d][((size_t)f * nf + fq) * 3 + i] = x[3 * gpt + i];
                }
          }
      }
    }
}
} // namespace adv
