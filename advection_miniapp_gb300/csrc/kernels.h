// Host-visible launch interface of the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"

namespace adv
{
enum StageMode
{
  kModeApply     = 0, // r_out = out_scale * M^{-1} L r_in
  kModeStage     = 1, // u_out = u_in + b k, r_out = u_in + a k
  kModeLastStage = 2, // u_out = u_in + b k
  kModeVmult     = 3  // r_out = mass_factor M r_in - L r_in (weak form, the implicit operator)
};

// Arguments of the fused stage kernel (one launch = one LSRK stage or one
// operator application).  r_in must not alias u_out or r_out; u_out may alias
// u_in; r_out may alias u_in (each element is read before it is written by
// the same thread).
struct StageArgs
{
  const double *r_in;
  const double *u_in;
  double       *u_out;
  double       *r_out;
  double        b, a, out_scale;
  int           mode;
  int           swap_pm;  // velocity time factor < 0: exchange the upwind coefficients
  int           nc[3];
  int           npos[3];
  long long     n_cells;    // end of the processed cells (local index)
  long long     cell_begin; // first processed cell (a slab skips its lower ghost layer)
  int           periodic;   // bit d: wrap around along d
  int           uniform;  // affine mesh with constant velocity
  int           bc_exact; // Dirichlet data from the exact solution (else zero)
  int           gauss;    // vectors hold values at the Gauss points (collocation basis)
  double        cv[3], P[3], M[3]; // uniform case: a_d / h_d and face coefficients
  double        skew;
  float         cvf[3], Pf[3], Mf[3], skewf; // the same in binary32 for the FP32 operator
  int           has_skew;
  int           visc;        // SIPG diffusion on an affine mesh (field geometry)
  // SIPG constants per direction (V = cell volume, h = cell width, sigma the penalty):
  // K1 = nu sigma V / h, K2 = nu V / (2 h^2), cdiff = nu V / h^2
  double        K1[3], K2[3], cdiff[3];
  float         K1f[3], K2f[3], cdifff[3];
  double        adv_scale;   // velocity time factor, applied in-kernel when visc != 0
  float         adv_scalef;
  // face traces on field geometry without SIPG (FP64): the flux is the
  // upwind one (at every face point one of P, M is zero) with a constant
  // velocity and no skew term, so each face point reads only the trace of
  // its upwind cell; stages read and write only those (see stage_gauss.cuh)
  int           upwind_tr;
  double        mass_factor; // vmult mode: factor of the mass matrix
  float         mass_factorf;
  float         volf;        // uniform case: cell volume (det J)
  double        vol;
  const void   *cell_geo;    // field case: [vt0|vt1|vt2|idet] x n^3 per cell (T)
  const void   *face_geo[3]; // field case: n^2 (P, M) pairs per face (T)
  const double *face_x[3];   // Dirichlet faces: n^2 x 3 coordinates per face
  double        t;           // time of the Dirichlet data
  // collocation form with face traces: per cell [6][n^2] values at the face
  // points (x low, x high, y low, y high, z low, z high) of r_in (read) and
  // of the next stage's input (written: r_out, or u_out on a last stage), in
  // the operator's precision
  const void   *tr_in;
  void         *tr_out;
  // FP32 increments (optional): k += k_add before the update; k_out receives
  // k; the last stage adds u_base to its output; u_in == nullptr reads as 0
  const double *k_add;
  double       *k_out;
  const double *u_base;
  // FP32 increments with the anchor's k folded out (collocation form, inc32
  // != 0; K0 = L(u_a) of the block's FP64 anchor, e = u_in the increment
  // u - u_a - C K0 with C the sum of the b's since the anchor):
  //   stage:  u_out = e + b k;  r_out32 = binary32(e + inc_alpha K0 + a k)
  //           (k_add32 holds K0; the anchor itself, run by the FP64 kernel
  //           on u_a, writes k_out = K0, k_out32 = binary32(K0) and
  //           r_out32 = binary32(a K0) and nothing else);
  //   last:   u_out = u_base + (e + b k) + inc_alpha K0 (k_add holds K0)
  // r_in32 replaces r_in as the operator's input.
  int           inc32;
  float         inc_alphaf, inc_af;
  double        inc_alpha;
  const float  *r_in32;
  float        *r_out32;
  const float  *k_add32;
  float        *k_out32;
  ExactParams   ex;
};

// precision: 0 = FP64, 1 = FP32 operator
cudaError_t launch_stage(int n, int precision, const StageArgs &args, cudaStream_t stream);

// Collocation form of the stage (args.gauss != 0): r_in, u_in and the outputs
// hold the values at the (k+1)^3 Gauss points of every cell, the nodal basis
// of the Lagrange polynomials on those points.  The operator is the same
// polynomial map as the Gauss-Lobatto nodal form without its interpolation
// and inverse-mass sweeps.  Modes: apply, stage, last stage, and the
// implicit operator in weak form (vmult): r_out receives the dual
// coefficients on the Gauss-point basis, JxW (c u - L u) at each point.
cudaError_t launch_stage_gauss_fp64(int n, const StageArgs &args, cudaStream_t stream);
cudaError_t launch_stage_gauss_fp32(int n, const StageArgs &args, cudaStream_t stream);
cudaError_t upload_tables_gauss64(const DevTables<double> *d, const DevTables<float> *f);
cudaError_t upload_tables_gauss32(const DevTables<double> *d, const DevTables<float> *f);
// In-place change of basis of the cells [cell_begin, cell_end) of u:
// to_gauss: Gauss-Lobatto nodal values -> values at the Gauss points (S x S x S);
// otherwise the inverse (S^-1 x S^-1 x S^-1).  With traces (to_gauss only),
// also writes the face traces of the result in the layout of StageArgs::tr_in
// (width 2: values and reference normal derivatives, for SIPG).  upwind
// (width 1): only the traces an upwind-trace stage reads (StageArgs::
// upwind_tr), with the mesh and the FP64 face coefficients of *upwind.
cudaError_t launch_basis_change(int n, double *u, long long cell_begin, long long cell_end, bool to_gauss,
                                cudaStream_t stream, double *traces = nullptr, int width = 1,
                                const StageArgs *upwind = nullptr);
// In-place u <- (S^T x S^T x S^T) u for the cells [cell_begin, cell_end): the
// dual coefficients of a weak-form vector on the Gauss-point basis to those
// on the Gauss-Lobatto nodal basis (each nodal function is the combination
// sum_q S[q][i] l_q of the Gauss-point Lagrange functions).
cudaError_t launch_basis_dual_to_nodal(int n, double *u, long long cell_begin, long long cell_end,
                                       cudaStream_t stream);
// Face traces [6][width][n^2] per cell of the Gauss-point values in u (the
// values at the face points, with width 2 also the reference normal
// derivatives), for the cells [cell_begin, cell_end); u is not changed.
cudaError_t launch_face_traces(int n, const double *u, long long cell_begin, long long cell_end,
                               cudaStream_t stream, double *traces, int width, const StageArgs *upwind = nullptr);
// cells processed per CTA by the stage kernel (for launch accounting)
int stage_cells_per_block(int n, int precision);

// Upload the 1D tables (index n = points per direction) to every translation
// unit's constant memory on the current device.
cudaError_t upload_tables(const DevTables<double> *d, const DevTables<float> *f);
cudaError_t upload_tables_stage64(const DevTables<double> *d, const DevTables<float> *f);
cudaError_t upload_tables_stage32(const DevTables<double> *d, const DevTables<float> *f);
cudaError_t upload_tables_diag(const DevTables<double> *d, const DevTables<float> *f);
cudaError_t launch_stage_fp64(int n, const StageArgs &args, cudaStream_t stream);
cudaError_t launch_stage_fp32(int n, const StageArgs &args, cudaStream_t stream);
int stage_cells_per_block_fp64(int n);
int stage_cells_per_block_fp32(int n);

// Diagnostics and set-up kernels (diag_kernels.cu)
struct DiagArgs
{
  int           n;
  int           nc[3];
  long long     n_cells;    // end of the owned cells (local index)
  long long     cell_begin; // first owned cell
  int           zoff;       // global z index of local cell layer 0
  int           pad1;
  double        lo[3], L[3], h[3];
  int           curved;
  int           pad0;
  double        deformation;
  ExactParams   ex;
  // 1D data: Gauss-Lobatto nodes, Gauss points/weights (n), error-quadrature
  // points/weights (n + 1); nodal basis values / derivatives at the Gauss
  // points [q * n + i], S^{-1} [i * n + q]; at the error points [(n+1) x n]
  double gl[8], gp[8], gw[8], ep[8], ew[8];
  double S[49], Si[49], Sd[49];
  double SE[56], SEd[56];
  double Dc[49]; // collocation derivative on the Gauss points [q * n + p]
};
cudaError_t launch_project(const DiagArgs &g, double t, double *dst, cudaStream_t s);
// partial sums per block written to `partials` (3 per block); returns number of blocks
cudaError_t launch_mass_energy(const DiagArgs &g, const double *u, double *partials, int *n_blocks,
                               cudaStream_t s);
cudaError_t launch_l2_error(const DiagArgs &g, const double *u, double t, double *partials,
                            int *n_blocks, cudaStream_t s);
int diag_max_blocks(long long n_cells);
cudaError_t launch_fma_peak(int precision, double *out, int iters, int blocks, cudaStream_t s);
// independent chains per loop iteration of that microbenchmark
int fma_peak_chains(int precision);
} // namespace adv
