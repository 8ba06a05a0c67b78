// Host-side structured mesh and geometry precompute: the part of
// AdvectionOperation::reinit / MatrixFree::reinit (advection_solver.cc:435-465)
// that computes Jacobians, JxW and normals, reduced to what the fused stage
// kernel streams.  For the velocity field b (constant, or the spatial part of
// the rotating field) it stores, per Gauss point q of a cell,
//     vt_d = det(J) (J^{-1} b)_d   (d = 0,1,2)   and   idet = 1 / det(J),
// and per Gauss point of a face normal to d (area normal N = det(J) J^{-T} e_d
// pointing to +xi_d, c = N . b)
//     P = (c + alpha |c|) / 2,   M = (c - alpha |c|) / 2.
// Quadrature weights are folded into the 1D tables (Tables1D::Dw, lw0/lw1), so
// no weight appears here.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/advection_gb300.h"
#include "tables.h"

namespace adv
{
struct Mesh
{
  int     n = 0;        // points per direction (degree + 1)
  int     nc[3] = {};   // cells per direction
  int64_t n_cells = 0;
  int64_t n_dofs  = 0;
  double  lo[3] = {}, L[3] = {}, h[3] = {};
  bool    curved   = false;
  bool    periodic = true;
  bool    uniform  = true; // affine + constant velocity: geometry is a set of constants
  int     npos[3] = {};    // face positions per direction (nc or nc + 1)
  int64_t n_faces[3] = {}; // faces per direction = npos * product of tangential counts
  // slab of a z-partitioned mesh: the local cells are the owned layers plus
  // one ghost layer on each side that has a neighbouring slab (or wraps
  // periodically); local layer 0 is global layer zoff.  h stays global.
  int     pmask      = 7;  // bit d: periodic wrap along d inside the local cells
  int     zoff       = 0;
  int     gnz        = 0;  // cells along z of the whole mesh
  int64_t cell_begin = 0, cell_end = 0; // owned local cells
  bool    slab       = false;
  bool    ghost_lo = false, ghost_hi = false;

  int t1(int d) const { return d == 0 ? 1 : 0; }
  int t2(int d) const { return d == 2 ? 1 : 2; }
  // face id of the face at position p along d with tangential cell indices (j1, j2)
  int64_t face_id(int d, int p, int j1, int j2) const
  {
    return p + (int64_t)npos[d] * (j1 + (int64_t)nc[t1(d)] * j2);
  }
};

struct HostGeometry
{
  // uniform case: per direction a_d / h_d and the face coefficients
  double cv[3] = {}, P[3] = {}, M[3] = {};
  double idet_const = 0.0;
  // field case: per cell [vt0 | vt1 | vt2 | idet] blocks of n^3 values
  std::vector<double> cell;
  // field case: per direction, per face n^2 (P, M) pairs (one per face point)
  std::vector<double> face[3];
  // Dirichlet: per direction, per face, n^2 points x 3 coordinates (boundary faces only hold data)
  std::vector<double> face_x[3];
  double h_min = 0.0;
  // per cell (v0, v1, v2, 1/|K|): JxW-weighted cell average of J^{-1} b and the
  // inverse cell volume (the cell data of the FDM preconditioner,
  // advection_solver_implicit.cc:1063-1076)
  std::vector<double> fdm_cell;
};

// Sine deformation of the box (mesh_type ADV_MESH_DEFORMED).
void deform_point(const adv_config &cfg, const double L[3], const double x[3], double y[3]);
// Velocity field at x (spatial part; the rotating field's cos(pi t/T) factor is applied at run time).
void velocity_field(const adv_config &cfg, const double x[3], double b[3]);

// support points of local cell c (Gauss-Lobatto nodes through the mapping),
// X[3 * (i + n (j + n k))]
void support_points(const adv_config &cfg, const Mesh &m, const Tables1D &tb, int64_t c, double *X);

int  setup_mesh(const adv_config &cfg, Mesh &m);
// local mesh of the slab of global z layers [z_begin, z_end) with its ghost layers
int  setup_slab(const adv_config &cfg, int z_begin, int z_end, Mesh &m);
void compute_geometry(const adv_config &cfg, const Mesh &m, const Tables1D &tb, HostGeometry &g);
} // namespace adv
