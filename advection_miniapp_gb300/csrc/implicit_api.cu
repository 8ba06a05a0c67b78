// Implicit time stepping: the GPU counterpart of the reference's implicit
// operator (AdvectionOperation::vmult, set_time, apply_inverse_mass_matrix,
// precondition_block_jacobi; advection_solver_implicit.cc:703-762,
// 1283-1340) and its FGMRES-driven time integrator
// (advection_solver_implicit.cc:1457-1525), here with BDF2.
//
// Linear solver: flexible GMRES(m) with right preconditioning, classical
// Gram-Schmidt applied twice, FP64 residuals, inner products, orthogonal
// basis and update; the block-Jacobi FDM preconditioner runs in FP32 or FP64.
// One host synchronisation per iteration (the new Hessenberg column and the
// norm come back together).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fdm.h"
#include "handle.h"
#include "implicit_kernels.h"

using adv::detail::fail;

struct adv_solver
{
  adv_handle *h                 = nullptr;
  int         restart           = 30;
  int         precond_precision = 1;
  int64_t     n                 = 0;
  double     *V = nullptr, *Z = nullptr, *w = nullptr, *tmp = nullptr, *b = nullptr;
  double     *d_small    = nullptr; // [coef1 (m+1) | coef2 (m+1) | norm | y (m)]
  double     *d_partials = nullptr;
  void       *d_tables   = nullptr;
  int64_t     bytes      = 0;
  // Gauss-basis solves: the Gauss-basis tolerance as a fraction of the nodal
  // one, from the ratio of the two relative residuals of the last solve (the
  // systems of consecutive time steps are alike), so that the nodal check at
  // convergence rarely fails and forces a restart
  double      gauss_tol_scale = 1.0;
};

namespace
{
int alloc(void **p, size_t bytes, int64_t &count)
{
  ADV_CUDA(cudaMalloc(p, bytes));
  count += (int64_t)bytes;
  return ADV_OK;
}

// gauss: src holds values at the Gauss points and dst receives the dual
// coefficients on the Gauss-point basis (the collocation-form stage kernel,
// no interpolation or integration sweeps); else both are on the nodal basis
int launch_vmult(adv_handle *h, const double *src, double *dst, double mass_factor, double t, cudaStream_t s,
                 bool gauss = false)
{
  adv::StageArgs A = adv::detail::base_args(*h, t);
  A.mode           = adv::kModeVmult;
  A.gauss          = gauss ? 1 : 0;
  A.r_in           = src;
  A.r_out          = dst;
  A.mass_factor    = mass_factor;
  A.mass_factorf   = (float)mass_factor;
  A.vol            = h->mesh.h[0] * h->mesh.h[1] * h->mesh.h[2];
  A.volf           = (float)A.vol;
  return adv::detail::launch(h, A, s);
}

int launch_mass_op(adv_handle *h, const double *src, double *dst, cudaStream_t s)
{
  adv::MassArgs A;
  A.src      = src;
  A.dst      = dst;
  A.n_cells  = h->mesh.n_cells;
  A.uniform  = h->mesh.uniform;
  A.vol      = h->mesh.h[0] * h->mesh.h[1] * h->mesh.h[2];
  A.cell_geo = static_cast<const double *>(h->d_cell_geo);
  ADV_CUDA(adv::launch_mass(h->mesh.n, A, s));
  ++h->launches;
  return ADV_OK;
}

double time_factor_of(const adv_handle &h, double t)
{
  return h.cfg.velocity_type == ADV_VELOCITY_CONSTANT ? 1.0 : std::cos(3.14159265358979323846 * t / h.cfg.velocity_period);
}

int norm2(adv_solver *S, const double *x, double *out, cudaStream_t s)
{
  ADV_CUDA(adv::launch_multi_dot(x, 0, 1, x, S->n, S->d_partials, S->d_small + 2 * (S->restart + 1), s));
  ADV_CUDA(cudaMemcpyAsync(out, S->d_small + 2 * (S->restart + 1), sizeof(double), cudaMemcpyDeviceToHost, s));
  ADV_CUDA(cudaStreamSynchronize(s));
  *out = std::sqrt(*out);
  return ADV_OK;
}
} // namespace

extern "C" {

int adv_vmult(adv_handle *h, const double *src, double *dst, double mass_factor, double t, void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_vmult", (cudaStream_t)stream);
  if (!h || !src || !dst)
    return fail(ADV_ERR_INVALID, "null argument");
  if (src == dst)
    return fail(ADV_ERR_ALIASING, "adv_vmult: dst must not alias src");
  if (int e = adv::detail::check_device(h))
    return e;
  return launch_vmult(h, src, dst, mass_factor, t, (cudaStream_t)stream);
}

int adv_apply_mass(adv_handle *h, const double *src, double *dst, void *stream)
{
  if (!h || !src || !dst)
    return fail(ADV_ERR_INVALID, "null argument");
  if (src == dst)
    return fail(ADV_ERR_ALIASING, "adv_apply_mass: dst must not alias src");
  if (!h->mesh.uniform && h->cfg.precision != ADV_PRECISION_FP64)
    return fail(ADV_ERR_INVALID, "adv_apply_mass needs an FP64 handle on curved meshes or with variable velocity");
  if (int e = adv::detail::check_device(h))
    return e;
  return launch_mass_op(h, src, dst, (cudaStream_t)stream);
}

int adv_solver_create(adv_handle *h, int restart, int precond_precision, adv_solver **out)
{
  if (!h || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  *out = nullptr;
  if (restart < 1 || restart > 60)
    return fail(ADV_ERR_INVALID, "restart must be in 1..60");
  if (precond_precision != ADV_PRECISION_FP64 && precond_precision != ADV_PRECISION_FP32_OPERATOR)
    return fail(ADV_ERR_INVALID, "unknown preconditioner precision");
  if (h->cfg.precision != ADV_PRECISION_FP64)
    return fail(ADV_ERR_INVALID, "the implicit solver needs an FP64 operator handle (residuals are FP64)");
  if (h->cfg.diffusion != 0.0)
    return fail(ADV_ERR_INVALID, "the implicit solver covers advection without diffusion");
  if (h->mesh.slab)
    return fail(ADV_ERR_INVALID, "the implicit solver runs on whole meshes (its inner products are not reduced "
                                 "across slabs)");
  if (!h->mesh.periodic && h->cfg.boundary_value != ADV_BOUNDARY_ZERO)
    return fail(ADV_ERR_INVALID, "the implicit solver needs periodic meshes or zero Dirichlet data (a linear operator)");
  if (int e = adv::detail::check_device(h))
    return e;
  adv::FdmTables t;
  if (!adv::fdm_tables(h->cfg.degree, h->cfg.flux_alpha, t))
    return fail(ADV_ERR_NOT_CONVERGED, "eigen-decomposition of the 1D operator did not converge");
  auto *S              = new adv_solver();
  S->h                 = h;
  S->restart           = restart;
  S->precond_precision = precond_precision;
  S->n                 = h->mesh.n_dofs;
  const size_t nb      = S->n * sizeof(double);
  int          rc      = ADV_OK;
  if ((rc = alloc((void **)&S->V, (restart + 1) * nb, S->bytes)) || (rc = alloc((void **)&S->Z, restart * nb, S->bytes)) ||
      (rc = alloc((void **)&S->w, nb, S->bytes)) || (rc = alloc((void **)&S->tmp, nb, S->bytes)) ||
      (rc = alloc((void **)&S->b, nb, S->bytes)) ||
      (rc = alloc((void **)&S->d_small, (3 * (restart + 1) + 1) * sizeof(double), S->bytes)) ||
      (rc = alloc((void **)&S->d_partials, adv::vec_partial_blocks(S->n) * (restart + 1) * sizeof(double), S->bytes)))
    {
      adv_solver_destroy(S);
      return rc;
    }
  // FDM tables per sign: [VWr VWi Vr Vi lr li]
  const int           n = t.n, per = 4 * n * n + 2 * n;
  std::vector<double> tab(2 * per);
  for (int si = 0; si < 2; ++si)
    {
      double *p = tab.data() + si * per;
      for (int i = 0; i < n * n; ++i)
        {
          p[i]             = t.VinvW[si][i].real();
          p[n * n + i]     = t.VinvW[si][i].imag();
          p[2 * n * n + i] = t.V[si][i].real();
          p[3 * n * n + i] = t.V[si][i].imag();
        }
      for (int i = 0; i < n; ++i)
        {
          p[4 * n * n + i]     = t.lambda[si][i].real();
          p[4 * n * n + n + i] = t.lambda[si][i].imag();
        }
    }
  if (precond_precision == ADV_PRECISION_FP64)
    {
      if ((rc = alloc(&S->d_tables, tab.size() * sizeof(double), S->bytes)) == ADV_OK)
        if (cudaMemcpy(S->d_tables, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
          rc = fail(ADV_ERR_CUDA, "upload of the FDM tables");
    }
  else
    {
      std::vector<float> tf(tab.begin(), tab.end());
      if ((rc = alloc(&S->d_tables, tf.size() * sizeof(float), S->bytes)) == ADV_OK)
        if (cudaMemcpy(S->d_tables, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
          rc = fail(ADV_ERR_CUDA, "upload of the FDM tables");
    }
  if (rc)
    {
      adv_solver_destroy(S);
      return rc;
    }
  *out = S;
  return ADV_OK;
}

int adv_solver_destroy(adv_solver *S)
{
  if (!S)
    return ADV_OK;
  cudaFree(S->V);
  cudaFree(S->Z);
  cudaFree(S->w);
  cudaFree(S->tmp);
  cudaFree(S->b);
  cudaFree(S->d_small);
  cudaFree(S->d_partials);
  cudaFree(S->d_tables);
  delete S;
  return ADV_OK;
}

int adv_solver_device_bytes(const adv_solver *S, int64_t *out)
{
  if (!S || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  *out = S->bytes;
  return ADV_OK;
}

} // extern "C"

namespace
{
// block-Jacobi FDM preconditioner; gauss: residual as dual coefficients and
// result as values on the Gauss-point basis
int precondition(adv_solver *S, const double *src, double *dst, double mass_factor, double t, cudaStream_t s,
                 bool gauss)
{
  adv_handle  *h = S->h;
  adv::FdmArgs A;
  std::memset(&A, 0, sizeof(A));
  A.src         = src;
  A.dst         = dst;
  A.n_cells     = h->mesh.n_cells;
  A.mass_factor = mass_factor;
  A.time_factor = time_factor_of(*h, t);
  A.gauss       = gauss ? 1 : 0;
  const void *cell = S->precond_precision == ADV_PRECISION_FP64 ? (const void *)h->d_fdm_cell_d
                                                                 : (const void *)h->d_fdm_cell_f;
  ADV_CUDA(adv::launch_fdm(h->mesh.n, S->precond_precision, A, S->d_tables, cell, s));
  ++h->launches;
  return ADV_OK;
}

int fgmres(adv_solver *S, double mass_factor, double t, const double *rhs, double *x, double rel_tol,
           int max_iterations, int *iterations, double *rel_residual, cudaStream_t s, bool gauss);
} // namespace

extern "C" {

int adv_precondition(adv_solver *S, const double *src, double *dst, double mass_factor, double t, void *stream)
{
  adv::detail::CallTrace trace_(S ? S->h : nullptr, "adv_precondition", (cudaStream_t)stream);
  if (!S || !src || !dst)
    return fail(ADV_ERR_INVALID, "null argument");
  if (src == dst)
    return fail(ADV_ERR_ALIASING, "adv_precondition: dst must not alias src");
  if (int e = adv::detail::check_device(S->h))
    return e;
  return precondition(S, src, dst, mass_factor, t, (cudaStream_t)stream, false);
}

int adv_fgmres(adv_solver *S, double mass_factor, double t, const double *rhs, double *x, double rel_tol,
               int max_iterations, int *iterations, double *rel_residual, void *stream)
{
  adv::detail::CallTrace trace_(S ? S->h : nullptr, "adv_fgmres", (cudaStream_t)stream);
  if (!S || !rhs || !x)
    return fail(ADV_ERR_INVALID, "null argument");
  if (rhs == x)
    return fail(ADV_ERR_ALIASING, "adv_fgmres: x must not alias rhs");
  if (int e = adv::detail::check_device(S->h))
    return e;
  return fgmres(S, mass_factor, t, rhs, x, rel_tol, max_iterations, iterations, rel_residual, (cudaStream_t)stream,
                false);
}

} // extern "C"

namespace
{
// FGMRES(m), right-preconditioned, CGS2.  gauss: rhs and the residuals are
// dual coefficients and x holds values on the Gauss-point basis; the
// iteration measures residuals in that basis but stops on the nodal
// residual ||S^T r|| / ||S^T rhs|| <= rel_tol (S^T = S^T x S^T x S^T), the
// criterion of the nodal solve, checked exactly whenever the Gauss-basis
// residual is below its own tolerance (which tightens if the check fails).
int fgmres(adv_solver *S, double mass_factor, double t, const double *rhs, double *x, double rel_tol,
           int max_iterations, int *iterations, double *rel_residual, cudaStream_t s, bool gauss)
{
  adv_handle   *h  = S->h;
  const int     m  = S->restart;
  const int64_t n  = S->n;
  double       *c1 = S->d_small, *c2 = S->d_small + (m + 1), *nrm = S->d_small + 2 * (m + 1),
         *ydev = S->d_small + 2 * (m + 1) + 1;
  double bnorm = 0.0;
  if (int e = norm2(S, rhs, &bnorm, s))
    return e;
  int    its = 0;
  double res = 0.0;
  if (bnorm == 0.0)
    {
      ADV_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
      if (iterations)
        *iterations = 0;
      if (rel_residual)
        *rel_residual = 0.0;
      return ADV_OK;
    }
  // the nodal norm of a dual vector on the Gauss-point basis (through S->w)
  auto nodal_norm = [&](const double *v, double *out) -> int {
    ADV_CUDA(cudaMemcpyAsync(S->w, v, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    ADV_CUDA(adv::launch_basis_dual_to_nodal(h->mesh.n, S->w, 0, h->mesh.n_cells, s));
    ++h->launches;
    return norm2(S, S->w, out, s);
  };
  double bnorm_nodal = bnorm, tol = gauss ? rel_tol * S->gauss_tol_scale : rel_tol;
  if (gauss)
    if (int e = nodal_norm(rhs, &bnorm_nodal))
      return e;
  std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), y(m), hh(2 * (m + 1) + 1);
  bool                converged = false;
  while (true)
    {
      // r = rhs - A x into V_0
      if (int e = launch_vmult(h, x, S->w, mass_factor, t, s, gauss))
        return e;
      ADV_CUDA(adv::launch_lincomb(S->V, 1.0, rhs, -1.0, S->w, n, s));
      double beta = 0.0;
      if (int e = norm2(S, S->V, &beta, s))
        return e;
      res = beta / bnorm;
      if (res <= tol)
        {
          if (!gauss)
            {
              converged = true;
              break;
            }
          double rn = 0.0;
          if (int e = nodal_norm(S->V, &rn))
            return e;
          const double res_nodal = rn / bnorm_nodal;
          if (res_nodal > 0.0)
            S->gauss_tol_scale = std::min(1.0, std::max(1.0 / 64.0, 0.9 * res / res_nodal));
          if (res_nodal <= rel_tol)
            {
              res       = res_nodal;
              converged = true;
              break;
            }
          tol = res * 0.5 * rel_tol / res_nodal;
        }
      if (its >= max_iterations)
        break;
      ADV_CUDA(adv::launch_lincomb(S->V, 1.0 / beta, S->V, 0.0, nullptr, n, s));
      std::fill(H.begin(), H.end(), 0.0);
      std::fill(g.begin(), g.end(), 0.0);
      g[0]  = beta;
      int k = 0; // columns built in this cycle
      for (int j = 0; j < m && its < max_iterations; ++j)
        {
          double *vj = S->V + j * n, *zj = S->Z + j * n;
          if (int e = precondition(S, vj, zj, mass_factor, t, s, gauss))
            return e;
          if (int e = launch_vmult(h, zj, S->w, mass_factor, t, s, gauss))
            return e;
          // classical Gram-Schmidt, twice
          ADV_CUDA(adv::launch_multi_dot(S->V, n, j + 1, S->w, n, S->d_partials, c1, s));
          ADV_CUDA(adv::launch_multi_axpy(S->w, S->V, n, j + 1, c1, -1.0, n, s));
          ADV_CUDA(adv::launch_multi_dot(S->V, n, j + 1, S->w, n, S->d_partials, c2, s));
          ADV_CUDA(adv::launch_multi_axpy(S->w, S->V, n, j + 1, c2, -1.0, n, s));
          ADV_CUDA(adv::launch_multi_dot(S->w, 0, 1, S->w, n, S->d_partials, nrm, s));
          ADV_CUDA(cudaMemcpyAsync(hh.data(), S->d_small, (2 * (m + 1) + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
          ADV_CUDA(cudaStreamSynchronize(s));
          const double hn = std::sqrt(hh[2 * (m + 1)]);
          for (int i = 0; i <= j; ++i)
            H[i * m + j] = hh[i] + hh[(m + 1) + i];
          H[(j + 1) * m + j] = hn;
          // Givens rotations
          for (int i = 0; i < j; ++i)
            {
              const double a = H[i * m + j], b = H[(i + 1) * m + j];
              H[i * m + j]       = cs[i] * a + sn[i] * b;
              H[(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
            }
          const double a = H[j * m + j], b = H[(j + 1) * m + j];
          const double r = std::hypot(a, b);
          cs[j]          = r == 0.0 ? 1.0 : a / r;
          sn[j]          = r == 0.0 ? 0.0 : b / r;
          H[j * m + j]       = r;
          H[(j + 1) * m + j] = 0.0;
          g[j + 1]           = -sn[j] * g[j];
          g[j]               = cs[j] * g[j];
          ++its;
          k   = j + 1;
          res = std::fabs(g[j + 1]) / bnorm;
          if (res <= tol || hn == 0.0)
            break;
          if (j + 1 < m)
            ADV_CUDA(adv::launch_lincomb(S->V + (j + 1) * n, 1.0 / hn, S->w, 0.0, nullptr, n, s));
        }
      // y = H^{-1} g, x += Z y
      for (int i = k - 1; i >= 0; --i)
        {
          double v = g[i];
          for (int l = i + 1; l < k; ++l)
            v -= H[i * m + l] * y[l];
          y[i] = v / H[i * m + i];
        }
      ADV_CUDA(cudaMemcpyAsync(ydev, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, s));
      ADV_CUDA(adv::launch_multi_axpy(x, S->Z, n, k, ydev, 1.0, n, s));
      ADV_CUDA(cudaStreamSynchronize(s)); // y lives on the host stack frame
    }
  if (iterations)
    *iterations = its;
  if (rel_residual)
    *rel_residual = res;
  if (!converged)
    return fail(ADV_ERR_NOT_CONVERGED, "FGMRES reached the iteration limit, relative residual " + std::to_string(res));
  return ADV_OK;
}
} // namespace

extern "C" {

int adv_bdf2_step(adv_solver *S, double t_new, double dt, int first_step, const double *u_n, const double *u_nm1,
                  double *u_new, double rel_tol, int *iterations, void *stream)
{
  adv::detail::CallTrace trace_(S ? S->h : nullptr, "adv_bdf2_step", (cudaStream_t)stream);
  if (!S || !u_n || !u_new || (!first_step && !u_nm1))
    return fail(ADV_ERR_INVALID, "null argument");
  if (u_new == u_n || u_new == u_nm1)
    return fail(ADV_ERR_ALIASING, "u_new must not alias u_n or u_nm1");
  if (!(dt > 0.0))
    return fail(ADV_ERR_INVALID, "dt must be positive");
  adv_handle *h = S->h;
  if (int e = adv::detail::check_device(h))
    return e;
  cudaStream_t    s  = (cudaStream_t)stream;
  const int64_t   n  = S->n;
  const int       nn = h->mesh.n;
  const long long nc = h->mesh.n_cells;
  // The system (c M - L) u_new = M rhs is solved on the Gauss-point basis:
  // values at the Gauss points for u, dual coefficients for the residuals.
  // There the mass matrix is diag(JxW), the operator is the collocation-form
  // stage kernel in weak form and the FDM preconditioner needs no basis
  // transforms; the stopping rule is the nodal relative residual.
  // S->tmp: u_n on the Gauss points; u_new: u_nm1 on the Gauss points, then
  // the initial guess and the solution, changed back to nodal values at the end
  ADV_CUDA(cudaMemcpyAsync(S->tmp, u_n, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  ADV_CUDA(adv::launch_basis_change(nn, S->tmp, 0, nc, true, s));
  ++h->launches;
  const double *geo = h->mesh.uniform ? nullptr : static_cast<const double *>(h->d_cell_geo);
  const double  vol = h->mesh.h[0] * h->mesh.h[1] * h->mesh.h[2];
  double        cm;
  if (first_step)
    {
      // BDF1: (M / dt - L) u_new = M u_n / dt, initial guess u_n
      cm = 1.0 / dt;
      ADV_CUDA(adv::launch_gauss_mass_lincomb(nn, S->b, 1.0 / dt, S->tmp, 0.0, nullptr, nc, geo, vol, s));
      ADV_CUDA(cudaMemcpyAsync(u_new, S->tmp, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
  else
    {
      // BDF2: (3/(2 dt) M - L) u_new = M (2 u_n - u_nm1 / 2) / dt, initial
      // guess 2 u_n - u_nm1
      cm = 1.5 / dt;
      ADV_CUDA(cudaMemcpyAsync(u_new, u_nm1, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      ADV_CUDA(adv::launch_basis_change(nn, u_new, 0, nc, true, s));
      ++h->launches;
      ADV_CUDA(adv::launch_gauss_mass_lincomb(nn, S->b, 2.0 / dt, S->tmp, -0.5 / dt, u_new, nc, geo, vol, s));
      ADV_CUDA(adv::launch_lincomb(u_new, 2.0, S->tmp, -1.0, u_new, n, s));
    }
  h->launches += 2;
  const int rc = fgmres(S, cm, t_new, S->b, u_new, rel_tol, 100000, iterations, nullptr, s, true);
  ADV_CUDA(adv::launch_basis_change(nn, u_new, 0, nc, false, s));
  ++h->launches;
  return rc;
}

} // extern "C"
