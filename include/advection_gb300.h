/*
 * advection_gb300: C ABI of the GB300-native (sm_103a) matrix-free DG
 * advection operator and its low-storage Runge-Kutta stage.
 *
 * The reference (kronbichler/advection_miniapp) exposes this path as a C++
 * class used through templates, not as an FFI.  Each entry point below names
 * the reference member it replaces; a C++ wrapper with the reference's own
 * call surface (AdvectionOperation / LowStorageRungeKuttaIntegrator) sits on
 * top in advection_gb300.hpp.
 *
 * Conventions
 *  - Vectors are caller-owned device buffers of n_dofs values (double unless
 *    stated), laid out cell by cell (cells lexicographic, x fastest) and,
 *    inside a cell, lexicographic over the (k+1)^3 Gauss-Lobatto support
 *    points (x fastest), like FE_DGQ's numbering.  adv_alloc_vector is a
 *    convenience; any cudaMalloc'ed buffer of the right size works.
 *  - Every call takes an explicit CUDA stream (NULL = legacy default stream)
 *    and returns an int status: 0 = ok, see ADV_ERR_*.  No exception crosses
 *    the ABI.  adv_last_error() gives a message for the calling thread.
 *  - A handle is not thread-safe (the reference operator is not re-entrant
 *    either: its `time` member is written in const methods,
 *    advection_solver.cc:397,706); distinct handles are independent.
 */
#ifndef ADVECTION_GB300_H
#define ADVECTION_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum
{
  ADV_OK               = 0,
  ADV_ERR_INVALID      = 1, /* bad argument or unsupported configuration */
  ADV_ERR_OUT_OF_MEMORY = 2,
  ADV_ERR_CUDA         = 3, /* a CUDA runtime call failed */
  ADV_ERR_ALIASING     = 4, /* vector aliasing pattern that cannot be honoured */
  ADV_ERR_NOT_CONVERGED = 5,
  ADV_ERR_TIMEOUT      = 6
};

/* ----------------------------------------------------------- enumerations */
enum { ADV_MESH_CARTESIAN = 0, ADV_MESH_DEFORMED = 1 };
enum { ADV_VELOCITY_CONSTANT = 0, ADV_VELOCITY_ROTATING = 1 };
enum { ADV_IC_SINE_GAUSS = 0, ADV_IC_BLOB = 1, ADV_IC_WAVE = 2 };
enum { ADV_BOUNDARY_ZERO = 0, ADV_BOUNDARY_EXACT = 1 };
/* FP32_INCREMENT: the FP32 operator on stage increments.  In adv_lsrk_steps
 * every anchor_interval-th step evaluates L(u_a) at its start u_a with the
 * FP64 operator, and every other stage until the next anchor evaluates
 * L(u_a) + L32(r_s - u_a), where r_s - u_a = O(j dt |L u|) (j steps after the
 * anchor) is carried in FP64 (exact for linear operators that do not depend
 * on time: constant velocity, periodic or zero Dirichlet data).  The FP32
 * round-off then scales with the increment instead of the solution.
 * Elsewhere (apply, perform_stage, other operators) it is the FP32
 * operator. */
enum { ADV_PRECISION_FP64 = 0, ADV_PRECISION_FP32_OPERATOR = 1, ADV_PRECISION_FP32_INCREMENT = 2 };
/* LSRK schemes in the order of the reference's enum (advection_solver.cc:83-89) */
enum { ADV_LSRK_3_3 = 0, ADV_LSRK_5_4 = 1, ADV_LSRK_7_4 = 2, ADV_LSRK_9_5 = 3 };

/*
 * Run-time replacement of the reference's compile-time parameter block
 * (advection_solver.cc:55-123; degree was a template argument there).
 */
/* Basis the fused step loop (adv_lsrk_steps / adv_lsrk_step) runs its
 * stages in.  The result is the same polynomial to round-off: AUTO picks the
 * faster form for the precision, NODAL keeps the Gauss-Lobatto nodal values of
 * the reference, COLLOCATION changes the solution to the values at the Gauss
 * points on entry and back on exit and skips the interpolation and
 * inverse-mass sweeps in every stage. */
#define ADV_FORM_AUTO 0
#define ADV_FORM_NODAL 1
#define ADV_FORM_COLLOCATION 2
/* collocation without the face traces that FP64 advection stages pass to the
 * next stage (same results bit for bit; for comparisons) */
#define ADV_FORM_COLLOCATION_NO_TRACES 3

typedef struct adv_config
{
  int32_t degree;            /* FE_DGQ degree k, 1..6 (n = k+1 points per direction) */
  int32_t n_cells[3];        /* structured hex mesh, cells per direction */
  double  domain_lo[3];      /* box corners (unit cube in the workloads) */
  double  domain_hi[3];
  int32_t mesh_type;         /* ADV_MESH_*: affine, or sine-deformed with a degree-k mapping */
  int32_t periodic;          /* 1: periodic in every direction; 0: Dirichlet on every face */
  double  deformation;       /* A in x_d += A L_d sin(2 pi s_{d+1}) sin(2 pi s_{d+2}) */
  int32_t velocity_type;     /* ADV_VELOCITY_* */
  int32_t initial_condition; /* ADV_IC_*: initial data / exact solution */
  double  velocity[3];       /* constant velocity, or amplitudes of the rotating field */
  double  velocity_period;   /* T in cos(pi t / T) of the rotating field */
  double  flux_alpha;        /* 1: upwind (Lax-Friedrichs), 0: central (advection_solver.cc:74-75) */
  double  factor_skew;       /* 0: conservative, 0.5: skew-symmetric (advection_solver.cc:106-108) */
  double  diffusion;         /* SIPG diffusivity; 0 disables the viscous terms */
  double  penalty_factor;    /* SIPG penalty sigma = penalty_factor (k+1)^2 / h */
  int32_t boundary_value;    /* ADV_BOUNDARY_*: Dirichlet data zero or the exact solution */
  int32_t reserved0;
  double  ic_params[8];      /* sine-Gauss: phase p[3]; blob: centre c[3], width w */
  /* ---- fields below have no counterpart in the oracle's configuration ---- */
  int32_t precision;         /* ADV_PRECISION_*: FP64, FP32 operator with FP64 vectors, FP32 increments */
  int32_t fused_form;        /* ADV_FORM_*: basis of the stages inside adv_lsrk_steps */
  int32_t anchor_interval;   /* FP32 increments: steps per FP64 anchor evaluation, 1..64 (0: 4) */
  int32_t reserved1[5];
} adv_config;

typedef struct adv_handle adv_handle;

/* Fills *cfg with the defaults of the constant-velocity periodic workload
 * (degree 3, 8^3 cells, velocity (1, 0.15, -0.05), upwind flux, FP64). */
void adv_config_default(adv_config *cfg);

/* AdvectionOperation::reinit (advection_solver.cc:435-465): builds the mesh,
 * the 1D tables and the geometry on the current device and uploads them. */
int adv_create(const adv_config *cfg, adv_handle **out);

/* Slab of a mesh partitioned along z, one per rank (the reference distributes
 * cells with parallel::distributed::Triangulation and exchanges face values
 * in MatrixFree::loop with DataAccessOnFaces::values, advection_solver.cc:
 * 678-679).  The handle owns global z layers [z_begin, z_end) and holds one
 * ghost layer of cells below and above wherever a neighbouring slab exists
 * (always on periodic meshes).  Its vectors are local: the ghost layers, then
 * the owned layers, cell-major with x fastest, n^3 nodal values per cell with
 * the z index slowest.  The caller fills the ghost layers of the source vector
 * before every adv_apply / adv_perform_stage / adv_vmult (only each ghost
 * cell's face layer next to the slab, or whole cells with diffusion);
 * diagnostics cover the owned cells and return per-slab sums to be added
 * across ranks.  Fused step loops and the implicit solver reject slabs. */
int adv_create_slab(const adv_config *cfg, int z_begin, int z_end, adv_handle **out);
/* Host-only layout of that slab: out[10] = {local dofs (with ghosts), first
 * owned dof, owned dofs, cells per z layer, dofs per cell, ghost layer below
 * (0/1), ghost layer above (0/1), values per cell exchanged (n^2 face layer,
 * n^3 with diffusion), local z layers, global z index of local layer 0}. */
int adv_slab_layout(const adv_config *cfg, int z_begin, int z_end, int64_t *out);
/* AdvectionOperation destructor (advection_solver.cc:349-372): frees device data. */
int adv_destroy(adv_handle *h);
const char *adv_last_error(void);

int adv_n_dofs(const adv_handle *h, int64_t *out);
int adv_n_cells(const adv_handle *h, int64_t *out);
/* Device bytes held by the handle (geometry, tables, scratch). */
int adv_device_bytes(const adv_handle *h, int64_t *out);

/* AdvectionOperation::initialize_dof_vector (advection_solver.cc:343-347). */
int adv_alloc_vector(adv_handle *h, double **out);
int adv_free_vector(adv_handle *h, double *vec);

/* AdvectionOperation::apply (advection_solver.cc:661-691): dst = M^{-1} L(t) src.
 * dst may alias src. */
int adv_apply(adv_handle *h, const double *src, double *dst, double t, void *stream);

/* AdvectionOperation::perform_stage (advection_solver.cc:695-756):
 *   k = M^{-1} L(t) r_in;  u <- u + b_dt k;  r_out <- u_old + a_dt k (a_dt != 0).
 * Honours the reference's aliasing patterns (r_in == u with k == r_out on the
 * first stage, r_in == r_out on later stages).  `k` is scratch: its contents
 * afterwards are unspecified. */
int adv_perform_stage(adv_handle *h, double t, double b_dt, double a_dt, const double *r_in,
                      double *k, double *u, double *r_out, void *stream);

/* LowStorageRungeKuttaIntegrator::perform_time_step (advection_solver.cc:906-939):
 * one step of scheme ADV_LSRK_* from time t with step dt.  u holds the solution;
 * r and k are scratch registers (unspecified contents afterwards). */
int adv_lsrk_step(adv_handle *h, int scheme, double t, double dt, double *u, double *r, double *k,
                  void *stream);
/* n_steps consecutive steps (the reference's time loop, advection_solver.cc:1275-1300,
 * without output). */
int adv_lsrk_steps(adv_handle *h, int scheme, double t, double dt, int n_steps, double *u,
                   double *r, double *k, void *stream);
/* adv_lsrk_steps on a solution in host memory (the reference's time loop
 * with its vectors in host memory, advection_solver.cc:1275-1300): u_host
 * (n_dofs values; page-locked for the copies to overlap) is copied into the
 * device vector u, advanced by n_steps steps and copied back.  The copies run
 * on two copy streams of the handle in chunks of z layers, overlapped with the
 * first stage (host -> device) and the last stage (device -> host); the
 * results are those of adv_lsrk_steps bit for bit.  u_host must stay
 * untouched until the stream has passed the call, and then holds the result;
 * u holds it too. */
int adv_lsrk_steps_host(adv_handle *h, int scheme, double t, double dt, int n_steps, double *u_host,
                        double *u, double *r, double *k, void *stream);
/* Number of stages and the (a, b) coefficients of a scheme (a has n_stages-1 entries). */
int adv_lsrk_coefficients(int scheme, double *a, double *b, int *n_stages);

/* AdvectionOperation::project_initial (advection_solver.cc:760-784) of the
 * exact solution at time t (t = 0: the initial condition). */
int adv_project(adv_handle *h, double t, double *dst, void *stream);

/* compute_mass_and_energy (advection_solver.cc:787-818): out = {int u, int u^2,
 * int |grad u|^2}.  Synchronises the stream. */
int adv_mass_energy(adv_handle *h, const double *u, double out[3], void *stream);

/* output_results' error (advection_solver.cc:1183-1208): out[0] = ||u - u_exact(t)||
 * with QGauss(k+2), out[1] = ||u_exact(t)|| with QGauss(k+1).  Synchronises. */
int adv_l2_error(adv_handle *h, const double *u, double t, double out[2], void *stream);

/* setup_dofs time step rule (advection_solver.cc:1155-1165), before rounding:
 * courant * h_min / |a| / k^1.5. */
int adv_time_step(adv_handle *h, double courant, double *dt);

/* Host <-> device copies of whole vectors (stream-ordered; synchronise before
 * reading host data). */
int adv_copy_to_host(adv_handle *h, const double *dev, double *host, void *stream);
int adv_copy_from_host(adv_handle *h, const double *host, double *dev, void *stream);

/* ------------------------------------------------------------ implicit solver
 * The implicit operator of advection_solver_implicit.cc: vmult = M/dt + A
 * (:703-726, 821-887) with A = -L the left-hand-side advection operator, the
 * inverse mass matrix, the block-Jacobi fast-diagonalization preconditioner
 * (precondition_block_jacobi, :1283-1340) and an FGMRES solver (SolverFGMRES,
 * :1498-1504) driving BDF2 time steps.  FP64 residuals, inner products,
 * orthogonalisation and updates; the preconditioner in FP32 or FP64. */
typedef struct adv_solver adv_solver;

/* AdvectionOperation::vmult: dst = mass_factor * M src - L(t) src (weak form). */
int adv_vmult(adv_handle *h, const double *src, double *dst, double mass_factor, double t, void *stream);
/* dst = M src, the cellwise mass matrix (QGauss(k+1)). */
int adv_apply_mass(adv_handle *h, const double *src, double *dst, void *stream);
/* Workspace of FGMRES(restart) (restart + 1 basis and restart preconditioned
 * vectors) and the FDM tables; precond_precision is ADV_PRECISION_FP64 or
 * ADV_PRECISION_FP32_OPERATOR.  Needs an FP64 handle without diffusion and a
 * linear operator (periodic, or zero Dirichlet data). */
int adv_solver_create(adv_handle *h, int restart, int precond_precision, adv_solver **out);
int adv_solver_destroy(adv_solver *s);
int adv_solver_device_bytes(const adv_solver *s, int64_t *out);
/* Block-Jacobi FDM preconditioner: dst ~ (mass_factor M - L_cell(t))^{-1} src,
 * cell by cell (CellwisePreconditionerFDM, advection_solver_implicit.cc:490-646). */
int adv_precondition(adv_solver *s, const double *src, double *dst, double mass_factor, double t, void *stream);
/* Solves (mass_factor M - L(t)) x = rhs with right-preconditioned flexible
 * GMRES from the initial guess in x, to ||rhs - A x|| <= rel_tol ||rhs||.
 * Returns ADV_ERR_NOT_CONVERGED after max_iterations. */
int adv_fgmres(adv_solver *s, double mass_factor, double t, const double *rhs, double *x, double rel_tol,
               int max_iterations, int *iterations, double *rel_residual, void *stream);
/* One BDF2 step to time t_new: (3 u_new - 4 u_n + u_nm1) / (2 dt) = M^{-1} L(t_new) u_new
 * (first_step != 0: implicit Euler, u_nm1 unused), initial guess 2 u_n - u_nm1.
 * Inputs and output are nodal; the linear system is solved with the vectors
 * on the Gauss-point basis (diagonal mass matrix, no basis sweeps in the
 * operator or the preconditioner) and stops when the nodal relative residual
 * ||rhs - A u_new|| / ||rhs|| is at most rel_tol, as adv_fgmres does. */
int adv_bdf2_step(adv_solver *s, double t_new, double dt, int first_step, const double *u_n, const double *u_nm1,
                  double *u_new, double rel_tol, int *iterations, void *stream);

/* ------------------------------------------------------------------ timing
 * The reference accumulates the wall time of its operator calls in
 * computing_times and prints it at destruction (advection_solver.cc:349-372,
 * 670-690, 708-755).  With timing on, each (outermost) call of adv_apply,
 * adv_perform_stage, adv_lsrk_steps, the diagnostics and the implicit entry
 * points records CUDA events around the work it enqueues; adv_timing waits
 * for them and returns the accumulated device time and the number of timed
 * calls.  Every entry point also opens an NVTX range named after itself. */
int adv_set_timing(adv_handle *h, int enable);
int adv_timing(adv_handle *h, double *seconds, int64_t *calls);

/* ------------------------------------------------------------------ output
 * output_results (advection_solver.cc:1220-1241): a VTU file with the
 * support points of every (owned) cell, k^3 hexahedra per cell and the point
 * fields "solution" and "analytic_solution" (exact solution at time t). */
int adv_write_vtu(adv_handle *h, const double *vec, double time, const char *path, void *stream);
/* The same from host values of the whole mesh (no device needed). */
int adv_write_vtu_host(const adv_config *cfg, const double *host_vec, double time, const char *path);
/* Raw state for restart: header (degree, cells, mesh type, time) + the owned
 * nodal values; adv_load_state rejects files of another configuration. */
int adv_save_state(adv_handle *h, const double *vec, double time, const char *path, void *stream);
int adv_load_state(adv_handle *h, double *vec, double *time, const char *path, void *stream);

/* ------------------------------------------------------------- serving loop
 * Continuous batching of independent solves on one GPU (no counterpart in the
 * reference, which runs one solve per program).  Requests (periodic affine n^3
 * meshes, constant velocity, any degree 1..6 and either precision) are admitted
 * FIFO while their three FP64 vectors fit memory_budget_bytes and at most
 * max_active solves run; solves of one (degree, precision) share batched
 * stage launches captured as a CUDA graph of steps_per_tick LSRK(5,4) steps
 * and replayed while solves join and leave; groups run on their own streams.
 * Each request's time step follows setup_dofs (advection_solver.cc:1155-1167):
 * dt = courant h / |a| / k^1.5 rounded to t_end / ceil(t_end / dt).  The
 * server is not thread-safe. */
typedef struct adv_server adv_server;

int adv_server_create(int64_t memory_budget_bytes, int steps_per_tick, int max_active, int keep_solutions,
                      adv_server **out);
int adv_server_destroy(adv_server *s);
/* Admission order: FIFO (default), or the queued request with the least work
 * (DoFs x steps) first; with max_active below the queue length the latter
 * lets short solves overtake long ones (lower median latency, longer tail). */
enum { ADV_SERVE_FIFO = 0, ADV_SERVE_SHORTEST_FIRST = 1 };
int adv_server_set_policy(adv_server *s, int policy);
/* Queues a solve of cfg (its initial condition) to t_end. */
int adv_server_submit(adv_server *s, const adv_config *cfg, double t_end, double courant, int64_t *request_id);
/* One scheduling round (non-blocking on the GPU): retire finished solves
 * (relative L2 error against the exact solution), admit queued ones, start the
 * next tick of idle groups.  *n_completed: solves retired in this round. */
int adv_server_poll(adv_server *s, int *n_completed);
/* Cancels a request: a queued one leaves the queue at once, a running one at
 * the end of its group's current tick (its memory then goes back); state 4. */
int adv_server_cancel(adv_server *s, int64_t request_id);
/* Polls until every submitted request is complete. */
int adv_server_drain(adv_server *s);
/* state: 0 queued, 1 running, 2 done, 3 failed at admission (its device
 * memory could not be allocated or its set-up launch failed; the server
 * carries on with the other requests), 4 cancelled; latency from submission
 * to retirement. */
int adv_server_result(adv_server *s, int64_t request_id, int *state, double *rel_l2_error, double *latency_s,
                      int *steps, double *dt);
/* Final solution of a done request (servers created with keep_solutions != 0). */
int adv_server_solution(adv_server *s, int64_t request_id, double *host_out, int64_t n);
/* out[8] = {submitted, queued, running, completed, device bytes in use, budget, ticks, kernel launches}. */
int adv_server_stats(const adv_server *s, int64_t *out);

/* 1D fast-diagonalization tables of the cellwise preconditioner (the 1D set-up
 * of advection_solver_implicit.cc:1020-1062): on the unit interval with the
 * Lagrange basis on the k+1 Gauss points, W^{-1} A1 = V diag(lambda) V^{-1}
 * for unit velocity of sign +1 (sign_index 0) or -1 (sign_index 1).  Complex
 * outputs are interleaved (re, im): lambda[2n], V[2n^2] and VinvW[2n^2]
 * (= V^{-1} W^{-1}) row-major; A1[n^2] is the real matrix W^{-1} A1;
 * residual = max |W^{-1}A1 V - V Lambda| / max |W^{-1}A1| over both signs.
 * Any output pointer may be NULL.  Host only. */
int adv_fdm_tables(int degree, double flux_alpha, int sign_index, double *lambda, double *V,
                   double *VinvW, double *A1, double *residual);

/* Number of kernel launches the library has issued on this handle. */
int adv_launch_count(const adv_handle *h, int64_t *out);

/* Measured FP64 (precision 0) / FP32 (1) fused multiply-add throughput of the
 * current device in TFLOP/s (FMA = 2 flops), for roofline denominators; 2:
 * FP64 instructions in the stage kernel's mix of FMA, MUL and ADD (7 : 4 : 3),
 * as 2 x instructions per second.  Synchronises. */
int adv_measure_fma_peak(int precision, double *tflops, void *stream);

/* No counterpart in the reference.  adv_perform_stage for callers that must
 * not allocate device memory during a solve: serving code that admits solves
 * under a fixed device-memory budget (an allocation mid-solve could exceed
 * it, or fail under memory pressure), latency-critical loops (cudaMalloc and
 * cudaFree can synchronise the device and stall other streams), and hosts
 * whose device memory is owned by another allocator.  adv_perform_stage
 * stages an output that aliases r_in in a handle-owned vector it allocates
 * on first use; this variant stages it in a file-scope device array of
 * ADV_NOALLOC_MAX_DOFS doubles (16 MiB) and calls no allocating routine.
 * adv_create (and adv_create_slab) looks up the array's device address
 * (cudaGetSymbolAddress) with the handle's device current and keeps it in
 * the handle; the lookup loads the library module that holds the array, so
 * its 16 MiB are committed on that device when the first handle is created
 * there, and stay until the process exits.  Meshes with more than
 * ADV_NOALLOC_MAX_DOFS DoFs are rejected with ADV_ERR_INVALID.  All calls
 * share the one array: calls whose kernels overlap on the GPU (different
 * streams, or different handles) race on it.  Nothing in it needs to start
 * at zero: each call overwrites every staged value before copying it out.
 * Same arguments, aliasing rules and results as adv_perform_stage; `k` is
 * not touched.  Traced and timed like the other entry points. */
#define ADV_NOALLOC_MAX_DOFS (1 << 21)
int adv_perform_stage_noalloc(adv_handle *h, double t, double b_dt, double a_dt, const double *r_in,
                              double *k, double *u, double *r_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif
