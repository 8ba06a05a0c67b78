/*
 * CPU oracle for the matrix-free DG advection operator: TEST INFRASTRUCTURE.
 *
 * This library restates, in plain FP64 C++ on the host, the algorithm of the
 * reference miniapp (kronbichler/advection_miniapp, advection_solver.cc and
 * its variants).  The tests compare the CUDA implementation in the
 * advection_miniapp_gb300 package with it, and it is the timed CPU baseline.  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark may load
 * it; the product never links or calls it.
 *
 * Parity status: the reference is a set of deal.II programs (deal.II >= 9.2,
 * not vendored, no pinned version) with no tests, golden vectors or recorded
 * outputs, and deal.II / MPI / LAPACK are not installed here, so the
 * reference cannot be run.  Parity with the reference itself is therefore
 * UNPINNED.  The restatement is pinned instead by self-made checks: tables
 * against numpy/scipy, a second dense-matrix implementation of every term,
 * exactness/convergence against analytic solutions, conservation and energy
 * decay, and the time-integration order of the Runge-Kutta schemes.
 *
 * The configuration struct shares its field layout with the product's
 * adv_config prefix so that tests can fill both from one description.
 */
#ifndef ADVECTION_ORACLE_H
#define ADVECTION_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_config
{
  int32_t degree;          /* polynomial degree k of FE_DGQ, 1..6 */
  int32_t n_cells[3];      /* cells per direction of the structured hex mesh */
  double  domain_lo[3];    /* lower corner of the box */
  double  domain_hi[3];    /* upper corner of the box */
  int32_t mesh_type;       /* 0: affine Cartesian; 1: sine-deformed, degree-k mapping */
  int32_t periodic;        /* 1: periodic in all directions; 0: Dirichlet on all faces */
  double  deformation;     /* amplitude A of x_d += A L_d sin(2 pi s_{d+1}) sin(2 pi s_{d+2}) */
  int32_t velocity_type;   /* 0: constant a; 1: rotating field times cos(pi t / T) */
  int32_t initial_condition; /* 0: sine product + Gaussian; 1: Gaussian blob; 2: sin/cos wave */
  double  velocity[3];     /* constant velocity, or amplitudes (v0, v1, v2) of the rotating field */
  double  velocity_period; /* T in cos(pi t / T) for the rotating field */
  double  flux_alpha;      /* 1: upwind (Lax-Friedrichs); 0: central */
  double  factor_skew;     /* 0: conservative; 0.5: skew-symmetric */
  double  diffusion;       /* SIPG diffusivity nu; 0 disables the viscous terms */
  double  penalty_factor;  /* SIPG penalty sigma = penalty_factor (k+1)^2 / h */
  int32_t boundary_value;  /* Dirichlet data: 0 zero; 1 the exact (translated) solution */
  int32_t reserved0;
  double  ic_params[8];    /* type 0: phase p[3]; type 1: centre c[3], width w; type 2: unused */
} oracle_config;

typedef struct oracle_op oracle_op;

/* LSRK schemes, in the order of the reference's enum (advection_solver.cc:83-89). */
enum
{
  ORACLE_LSRK_3_3 = 0,
  ORACLE_LSRK_5_4 = 1,
  ORACLE_LSRK_7_4 = 2,
  ORACLE_LSRK_9_5 = 3
};

int     oracle_create(const oracle_config *cfg, oracle_op **out);
void    oracle_destroy(oracle_op *op);
int64_t oracle_n_dofs(const oracle_op *op);
int64_t oracle_n_cells(const oracle_op *op);
void    oracle_set_num_threads(int n);
int     oracle_get_max_threads(void);

/* 1D tables of FE_DGQ(k) on Gauss-Lobatto nodes with QGauss(k+1), all on [0,1].
 * S[q*n+i] = phi_i(g_q), D[q*n+i] = phi_i'(g_q), Sinv = S^{-1}. */
int oracle_tables(int degree, double *gl_nodes, double *gauss_points,
                  double *gauss_weights, double *S, double *D, double *Sinv);

/* dst = L(t) src, the weak-form right-hand side before the inverse mass
 * (what data.loop writes into vec_ki, advection_solver.cc:710-718). */
int oracle_apply_unscaled(oracle_op *op, const double *src, double *dst, double t);
/* dst = M^{-1} src, cellwise (advection_solver.cc:635-657); dst may alias src. */
int oracle_inverse_mass(oracle_op *op, const double *src, double *dst);
/* dst = M^{-1} L(t) src (AdvectionOperation::apply, advection_solver.cc:661-691). */
int oracle_apply(oracle_op *op, const double *src, double *dst, double t);
/* AdvectionOperation::perform_stage (advection_solver.cc:695-756) with the
 * reference's aliasing patterns allowed. */
int oracle_perform_stage(oracle_op *op, double t, double b_dt, double a_dt,
                         const double *r_in, double *k, double *u, double *r_out);
/* LowStorageRungeKuttaIntegrator::perform_time_step (advection_solver.cc:906-939). */
int oracle_lsrk_step(oracle_op *op, int scheme, double t, double dt, double *u,
                     double *r, double *k);
int oracle_lsrk_coefficients(int scheme, double *a, double *b, int *n_stages);
/* project_initial (advection_solver.cc:760-784) of the exact solution at time t. */
int oracle_project(oracle_op *op, double t, double *dst);
/* compute_mass_and_energy (advection_solver.cc:787-818): {int u, int u^2, int |grad u|^2}. */
int oracle_mass_energy(oracle_op *op, const double *u, double out[3]);
/* L2 error as in output_results (advection_solver.cc:1183-1208):
 * out[0] = ||u_h - u(t)|| with QGauss(k+2), out[1] = ||u(t)|| with QGauss(k+1). */
int oracle_l2_error(oracle_op *op, const double *u, double t, double out[2]);
/* Time step rule (advection_solver.cc:1155-1165) without the final rounding. */
double oracle_time_step(oracle_op *op, double courant);
double oracle_min_vertex_distance(oracle_op *op);
/* Nodal interpolation of the exact solution at the Gauss-Lobatto support points. */
int oracle_interpolate(oracle_op *op, double t, double *dst);
/* Physical coordinates of every DoF's support point (3 doubles per DoF). */
int oracle_support_points(oracle_op *op, double *xyz);

/* Implicit solver pieces (advection_solver_implicit.cc).
 * dst = M src (cellwise mass matrix, QGauss(k+1)). */
int oracle_apply_mass(oracle_op *op, const double *src, double *dst);
/* vmult (advection_solver_implicit.cc:710-726): dst = mass_factor M src - L(t) src,
 * i.e. M/dt + A with A the left-hand-side advection operator. */
int oracle_vmult(oracle_op *op, const double *src, double *dst, double mass_factor, double t);
/* Block-Jacobi with the cellwise fast-diagonalization preconditioner
 * (CellwisePreconditionerFDM::vmult, advection_solver_implicit.cc:490-646, and
 * precondition_block_jacobi, :1283-1340): per cell, transform the residual to
 * the collocation basis on the Gauss points (S^{-T}), apply V^{-1}W^{-1} in
 * every direction, divide by (1/volume) / (mass_factor + sum_d v_d lambda_d),
 * apply V, take the real part and transform back (S^{-1}).  v is the cell
 * average of J^{-1} a (weighted by JxW); the tables of the sign of v_d are used.
 * Tables (interleaved re, im): lambda[2][2n], V[2][2n^2], VinvW[2][2n^2], index
 * 0 for positive, 1 for negative velocity. */
int oracle_fdm_apply(oracle_op *op, const double *lambda, const double *V, const double *VinvW,
                     const double *src, double *dst, double mass_factor);

/* Second, independent implementation with dense per-cell matrices: basis
 * evaluated at every 3D quadrature point, dense face matrices and a Cholesky
 * solve with the assembled cell mass matrix.  Slow; used to cross-check. */
int oracle_apply_unscaled_dense(oracle_op *op, const double *src, double *dst, double t);
int oracle_inverse_mass_dense(oracle_op *op, const double *src, double *dst);

#ifdef __cplusplus
}
#endif

#endif
