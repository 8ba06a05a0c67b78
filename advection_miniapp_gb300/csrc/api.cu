// C ABI of the GB300 advection operator (include/advection_gb300.h).
//
// Host side of AdvectionOperation (advection_solver.cc:329-818) and
// LowStorageRungeKuttaIntegrator (advection_solver.cc:822-944): set-up of
// mesh, tables and geometry on the device, and the stage sequencing with the
// buffer rotation that lets every fused stage kernel read r_in while writing
// its outputs to other buffers.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/advection_gb300.h"
#include "fdm.h"
#include "geometry.h"
#include "handle.h"
#include "batch_kernels.h"
#include "implicit_kernels.h"
#include "kernels.h"
#include "tables.h"

namespace
{
thread_local std::string g_last_error;
} // namespace

namespace adv
{
namespace detail
{
int fail(int code, const std::string &msg)
{
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *where)
{
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? ADV_ERR_OUT_OF_MEMORY : ADV_ERR_CUDA;
}
} // namespace detail
} // namespace adv

using adv::detail::cuda_fail;
using adv::detail::fail;

namespace
{

std::mutex g_table_mutex;
bool       g_tables_uploaded[256] = {};

// even-odd form of a reflection-(anti)symmetric n x n matrix M[q][i]
template <typename T>
void even_odd(int n, const double (&M)[adv::kMaxN][adv::kMaxN], bool anti, adv::EvenOdd<T> &eo)
{
  const int h = n / 2;
  std::memset(&eo, 0, sizeof(eo));
  for (int q = 0; q < h; ++q)
    {
      for (int i = 0; i < h; ++i)
        {
          eo.e[q][i] = (T)(0.5 * (M[q][i] + M[q][n - 1 - i]));
          eo.o[q][i] = (T)(0.5 * (M[q][i] - M[q][n - 1 - i]));
        }
      if (n % 2)
        eo.ce[q] = (T)M[q][h];
    }
  if (n % 2)
    {
      for (int i = 0; i < h; ++i)
        eo.mid[i] = (T)M[h][i];
      eo.cc = anti ? (T)0 : (T)M[h][h];
    }
}

int ensure_tables(int device)
{
  std::lock_guard<std::mutex> lock(g_table_mutex);
  if (device < 0 || device >= 256)
    return fail(ADV_ERR_INVALID, "device index out of range");
  if (g_tables_uploaded[device])
    return ADV_OK;
  static adv::DevTables<double> td[adv::kMaxNDev + 1];
  static adv::DevTables<float>  tf[adv::kMaxNDev + 1];
  std::memset(td, 0, sizeof(td));
  std::memset(tf, 0, sizeof(tf));
  for (int n = 2; n <= adv::kMaxNDev; ++n)
    {
      adv::Tables1D t;
      t.init(n - 1);
      for (int q = 0; q < n; ++q)
        {
          for (int i = 0; i < n; ++i)
            {
              td[n].S[q][i]  = t.S[q][i];
              td[n].Si[q][i] = t.Si[q][i];
              td[n].Dw[q][i] = t.Dw[q][i];
              td[n].D[q][i]  = t.D[q][i];
              tf[n].S[q][i]  = (float)t.S[q][i];
              tf[n].Si[q][i] = (float)t.Si[q][i];
              tf[n].Dw[q][i] = (float)t.Dw[q][i];
              tf[n].D[q][i]  = (float)t.D[q][i];
            }
          td[n].l0[q] = t.l0[q], td[n].l1[q] = t.l1[q];
          td[n].lw0[q] = t.lw0[q], td[n].lw1[q] = t.lw1[q], td[n].gw[q] = t.gw[q];
          tf[n].l0[q] = (float)t.l0[q], tf[n].l1[q] = (float)t.l1[q];
          tf[n].lw0[q] = (float)t.lw0[q], tf[n].lw1[q] = (float)t.lw1[q], tf[n].gw[q] = (float)t.gw[q];
          td[n].ld0[q] = t.ld0[q], td[n].ld1[q] = t.ld1[q], td[n].lwd0[q] = t.lwd0[q], td[n].lwd1[q] = t.lwd1[q];
          td[n].dphi0[q] = t.dphi0[q], td[n].dphi1[q] = t.dphi1[q];
          tf[n].ld0[q] = (float)t.ld0[q], tf[n].ld1[q] = (float)t.ld1[q];
          tf[n].lwd0[q] = (float)t.lwd0[q], tf[n].lwd1[q] = (float)t.lwd1[q];
          tf[n].dphi0[q] = (float)t.dphi0[q], tf[n].dphi1[q] = (float)t.dphi1[q];
        }
      for (int q = 0; q < n / 2; ++q)
        {
          const double e = 0.5 * (t.lw0[q] + t.lw0[n - 1 - q]), o = 0.5 * (t.lw0[q] - t.lw0[n - 1 - q]);
          td[n].lwe[q] = e, td[n].lwo[q] = o;
          tf[n].lwe[q] = (float)e, tf[n].lwo[q] = (float)o;
        }
      if (n % 2)
        td[n].lwe[n / 2] = t.lw0[n / 2], tf[n].lwe[n / 2] = (float)t.lw0[n / 2];
      for (int q = 0; q < n / 2; ++q)
        {
          const double e = 0.5 * (t.lwd0[q] + t.lwd0[n - 1 - q]), o = 0.5 * (t.lwd0[q] - t.lwd0[n - 1 - q]);
          td[n].lde[q] = e, td[n].ldo[q] = o;
          tf[n].lde[q] = (float)e, tf[n].ldo[q] = (float)o;
        }
      if (n % 2)
        td[n].lde[n / 2] = t.lwd0[n / 2], tf[n].lde[n / 2] = (float)t.lwd0[n / 2];
      double Si[adv::kMaxN][adv::kMaxN] = {};
      for (int i = 0; i < n; ++i)
        for (int q = 0; q < n; ++q)
          Si[i][q] = t.Si[i][q];
      double St[adv::kMaxN][adv::kMaxN] = {}, SiT[adv::kMaxN][adv::kMaxN] = {};
      for (int i = 0; i < n; ++i)
        for (int q = 0; q < n; ++q)
          {
            St[i][q]        = t.S[q][i];
            SiT[q][i]       = t.Si[i][q];
            td[n].St[i][q]  = t.S[q][i];
            td[n].SiT[q][i] = t.Si[i][q];
            tf[n].St[i][q]  = (float)t.S[q][i];
            tf[n].SiT[q][i] = (float)t.Si[i][q];
          }
      even_odd(n, St, false, td[n].St_eo);
      even_odd(n, SiT, false, td[n].SiT_eo);
      even_odd(n, St, false, tf[n].St_eo);
      even_odd(n, SiT, false, tf[n].SiT_eo);
      even_odd(n, t.S, false, td[n].S_eo);
      even_odd(n, Si, false, td[n].Si_eo);
      even_odd(n, t.Dw, true, td[n].Dw_eo);
      even_odd(n, t.D, true, td[n].D_eo);
      even_odd(n, t.S, false, tf[n].S_eo);
      even_odd(n, Si, false, tf[n].Si_eo);
      even_odd(n, t.Dw, true, tf[n].Dw_eo);
      even_odd(n, t.D, true, tf[n].D_eo);
    }
  ADV_CUDA(adv::upload_tables_stage64(td, tf));
  ADV_CUDA(adv::upload_tables_stage32(td, tf));
  ADV_CUDA(adv::upload_tables_diag(td, tf));
  ADV_CUDA(adv::upload_tables_implicit(td, tf));
  ADV_CUDA(adv::upload_tables_batch(td, tf));
  ADV_CUDA(adv::upload_tables_gauss64(td, tf));
  ADV_CUDA(adv::upload_tables_gauss32(td, tf));
  g_tables_uploaded[device] = true;
  return ADV_OK;
}

int validate(const adv_config &c)
{
  if (c.degree < 1 || c.degree > 6)
    return fail(ADV_ERR_INVALID, "degree must be in 1..6");
  if (c.fused_form < ADV_FORM_AUTO || c.fused_form > ADV_FORM_COLLOCATION_NO_TRACES)
    return fail(ADV_ERR_INVALID, "unknown fused_form");
  if (c.anchor_interval < 0 || c.anchor_interval > 64)
    return fail(ADV_ERR_INVALID, "anchor_interval must be in 0..64");
  for (int d = 0; d < 3; ++d)
    {
      if (c.n_cells[d] < 1)
        return fail(ADV_ERR_INVALID, "n_cells must be >= 1 in every direction");
      if (!(c.domain_hi[d] > c.domain_lo[d]))
        return fail(ADV_ERR_INVALID, "domain_hi must exceed domain_lo");
    }
  // vector indices are 64-bit everywhere (cell offset x points per cell),
  // cell indices are 32-bit: the cell count is the limit, device memory the
  // practical one
  const double nc = (double)c.n_cells[0] * c.n_cells[1] * c.n_cells[2];
  if (nc > 2.0e9)
    return fail(ADV_ERR_INVALID, "more than 2e9 cells are not supported");
  if (c.mesh_type != ADV_MESH_CARTESIAN && c.mesh_type != ADV_MESH_DEFORMED)
    return fail(ADV_ERR_INVALID, "unknown mesh_type");
  if (c.mesh_type == ADV_MESH_DEFORMED && !(std::fabs(c.deformation) < 0.1))
    return fail(ADV_ERR_INVALID, "|deformation| must be below 0.1 to keep the mapping invertible");
  if (c.velocity_type != ADV_VELOCITY_CONSTANT && c.velocity_type != ADV_VELOCITY_ROTATING)
    return fail(ADV_ERR_INVALID, "unknown velocity_type");
  if (c.velocity_type == ADV_VELOCITY_ROTATING && !(c.velocity_period > 0.0))
    return fail(ADV_ERR_INVALID, "velocity_period must be positive for the rotating field");
  if (c.initial_condition < ADV_IC_SINE_GAUSS || c.initial_condition > ADV_IC_WAVE)
    return fail(ADV_ERR_INVALID, "unknown initial_condition");
  if (c.initial_condition == ADV_IC_BLOB && !(c.ic_params[3] > 0.0))
    return fail(ADV_ERR_INVALID, "blob width ic_params[3] must be positive");
  if (c.precision != ADV_PRECISION_FP64 && c.precision != ADV_PRECISION_FP32_OPERATOR &&
      c.precision != ADV_PRECISION_FP32_INCREMENT)
    return fail(ADV_ERR_INVALID, "unknown precision");
  if (c.diffusion < 0.0)
    return fail(ADV_ERR_INVALID, "diffusion must be >= 0");
  if (c.diffusion != 0.0 && c.mesh_type != ADV_MESH_CARTESIAN)
    return fail(ADV_ERR_INVALID, "diffusion (SIPG) runs on affine meshes only");
  if (c.diffusion != 0.0 && !(c.penalty_factor > 0.0))
    return fail(ADV_ERR_INVALID, "penalty_factor must be positive with diffusion");
  if (!(c.flux_alpha >= 0.0 && c.flux_alpha <= 1.0))
    return fail(ADV_ERR_INVALID, "flux_alpha must be in [0, 1]");
  return ADV_OK;
}

template <typename T>
int upload_array(const std::vector<double> &src, void **dst, int64_t &bytes)
{
  std::vector<T> tmp(src.begin(), src.end());
  const size_t   nb = tmp.size() * sizeof(T);
  ADV_CUDA(cudaMalloc(dst, nb));
  ADV_CUDA(cudaMemcpy(*dst, tmp.data(), nb, cudaMemcpyHostToDevice));
  bytes += (int64_t)nb;
  return ADV_OK;
}

void fill_diag(adv_handle &h)
{
  adv::detail::make_diag(h.cfg, h.mesh, h.tb, h.diag);
}
} // namespace

void adv::detail::make_diag(const adv_config &cfg, const adv::Mesh &m, const adv::Tables1D &tb, adv::DiagArgs &g)
{
  struct
  {
    const adv_config    &cfg;
    const adv::Tables1D &tb;
  } h{cfg, tb};
  std::memset(&g, 0, sizeof(g));
  const int n = m.n;
  g.n                = n;
  for (int d = 0; d < 3; ++d)
    {
      g.nc[d] = m.nc[d];
      g.lo[d] = m.lo[d];
      g.L[d]  = m.L[d];
      g.h[d]  = m.h[d];
    }
  g.n_cells     = m.cell_end;
  g.cell_begin  = m.cell_begin;
  g.zoff        = m.zoff;
  g.curved      = m.curved;
  g.deformation = h.cfg.deformation;
  g.ex.type     = h.cfg.initial_condition;
  g.ex.constant_velocity = h.cfg.velocity_type == ADV_VELOCITY_CONSTANT;
  for (int d = 0; d < 3; ++d)
    {
      g.ex.velocity[d] = h.cfg.velocity[d];
      g.ex.lo[d]       = m.lo[d];
      g.ex.L[d]        = m.L[d];
    }
  for (int i = 0; i < 8; ++i)
    g.ex.p[i] = h.cfg.ic_params[i];
  for (int i = 0; i < n; ++i)
    g.gl[i] = h.tb.gl[i], g.gp[i] = h.tb.gp[i], g.gw[i] = h.tb.gw[i];
  adv::gauss_points(n + 1, g.ep, g.ew);
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i)
      {
        g.S[q * n + i]  = h.tb.S[q][i];
        g.Sd[q * n + i] = h.tb.Sd[q][i];
        g.Si[q * n + i] = h.tb.Si[q][i];
        g.Dc[q * n + i] = h.tb.D[q][i];
      }
  for (int p = 0; p < n + 1; ++p)
    for (int i = 0; i < n; ++i)
      {
        g.SE[p * n + i]  = adv::lagrange(h.tb.gl, n, i, g.ep[p]);
        g.SEd[p * n + i] = adv::lagrange_derivative(h.tb.gl, n, i, g.ep[p]);
      }
}

namespace
{

// velocity time factor of the rotating field at time t (1 for a constant velocity)
double time_factor(const adv_handle &h, double t)
{
  if (h.cfg.velocity_type == ADV_VELOCITY_CONSTANT)
    return 1.0;
  return std::cos(3.14159265358979323846 * t / h.cfg.velocity_period);
}

// precision of the operator kernels of a handle: FP64 (0) or FP32 (1)
int op_precision(const adv_handle &h)
{
  return h.cfg.precision == ADV_PRECISION_FP64 ? 0 : 1;
}

adv::StageArgs base_args(const adv_handle &h, double t, int prec = -1)
{
  adv::StageArgs A;
  std::memset(&A, 0, sizeof(A));
  const adv::Mesh &m = h.mesh;
  // the FP64 anchor stage of an FP32-increment handle uses the FP64 copy
  const bool geo64 = prec == 0 && op_precision(h) == 1;
  for (int d = 0; d < 3; ++d)
    {
      A.nc[d]   = m.nc[d];
      A.npos[d] = m.npos[d];
      A.cv[d]   = h.cv[d];
      A.P[d]    = h.P[d];
      A.M[d]    = h.M[d];
      A.cvf[d]  = (float)h.cv[d];
      A.Pf[d]   = (float)h.P[d];
      A.Mf[d]   = (float)h.M[d];
      A.face_geo[d] = geo64 ? (const void *)h.d_face_geo64[d] : h.d_face_geo[d];
      A.face_x[d]   = h.d_face_x[d];
    }
  A.n_cells    = m.cell_end;
  A.cell_begin = m.cell_begin;
  A.periodic   = m.pmask;
  A.uniform  = m.uniform;
  A.bc_exact = h.cfg.boundary_value == ADV_BOUNDARY_EXACT;
  A.skew     = h.cfg.factor_skew;
  A.skewf    = (float)h.cfg.factor_skew;
  A.has_skew = h.cfg.factor_skew != 0.0;
  A.cell_geo = geo64 ? (const void *)h.d_cell_geo64 : h.d_cell_geo;
  A.t        = t;
  A.ex       = h.diag.ex;
  const double s = time_factor(h, t);
  A.swap_pm      = s < 0.0;
  A.out_scale    = s;
  if (h.cfg.diffusion != 0.0)
    {
      // SIPG on the affine mesh: the velocity factor is applied in the kernel
      // (it does not scale the viscous terms), so outputs are not rescaled
      A.visc       = 1;
      A.adv_scale  = s;
      A.adv_scalef = (float)s;
      A.out_scale  = 1.0;
      const double nu = h.cfg.diffusion, V = m.h[0] * m.h[1] * m.h[2];
      for (int d = 0; d < 3; ++d)
        {
          const double sigma = h.cfg.penalty_factor * (h.cfg.degree + 1.0) * (h.cfg.degree + 1.0) / m.h[d];
          A.K1[d]     = nu * sigma * V / m.h[d];
          A.K2[d]     = nu * V / (2.0 * m.h[d] * m.h[d]);
          A.cdiff[d]  = nu * V / (m.h[d] * m.h[d]);
          A.K1f[d]    = (float)A.K1[d];
          A.K2f[d]    = (float)A.K2[d];
          A.cdifff[d] = (float)A.cdiff[d];
        }
    }
  return A;
}

int launch(adv_handle *h, const adv::StageArgs &A, cudaStream_t s, int prec = -1)
{
  const bool  fp64 = (prec < 0 ? op_precision(*h) : prec) == 0;
  cudaError_t e    = A.gauss ? (fp64 ? adv::launch_stage_gauss_fp64(h->mesh.n, A, s)
                                     : adv::launch_stage_gauss_fp32(h->mesh.n, A, s))
                             : (fp64 ? adv::launch_stage_fp64(h->mesh.n, A, s)
                                     : adv::launch_stage_fp32(h->mesh.n, A, s));
  if (e != cudaSuccess)
    return cuda_fail(e, "stage kernel launch");
  ++h->launches;
  return ADV_OK;
}

// Basis of the fused step loop: the collocation form wherever it is the
// faster one.  Measured on GB300: the FP64 operator (bound by the FP64 pipe,
// about 40 % fewer instructions; 1.68x at degree 4 on 64^3 curved cells) and
// the FP32 operator with diffusion (1.45x at degree 5); the FP32 advection
// operator is bound by memory latency and keeps the nodal form, whose
// neighbour reads are face layers rather than whole cells.
bool use_collocation(const adv_handle &h)
{
  if (h.cfg.fused_form == ADV_FORM_NODAL)
    return false;
  if (h.cfg.fused_form == ADV_FORM_COLLOCATION || h.cfg.fused_form == ADV_FORM_COLLOCATION_NO_TRACES)
    return true;
  return h.cfg.precision == ADV_PRECISION_FP64 || h.cfg.diffusion != 0.0;
}

// Face traces between the collocation stages: FP64 (with SIPG they carry
// the normal derivatives too).  Measured on GB300 at degree 4, 64^3
// curved cells: FP64 13.4 vs 12.3 GDoF/s without; the FP32 operator got
// slower with them (54.3 vs 61.0: one more barrier, more shared memory per
// CTA), so it does not use them.
bool use_traces(const adv_handle &h)
{
  return h.cfg.precision == ADV_PRECISION_FP64 && h.cfg.fused_form != ADV_FORM_COLLOCATION_NO_TRACES;
}

// trace values per face point: the value, and with SIPG its normal derivative
int trace_width(const adv_handle &h)
{
  return h.cfg.diffusion != 0.0 ? 2 : 1;
}

// Upwind traces (StageArgs::upwind_tr): each face point reads only the
// trace of its upwind cell.  Needs the upwind flux (flux_alpha 1: one of P, M
// is zero at every face point), a velocity constant in time (the pairs do
// not swap between the stage that writes a trace and the one that reads
// it), no skew term (it reads the own trace at every point), and field
// geometry without SIPG (the kernel variant that reads traces in its passes).
// Per cell-stage at degree 4 it saves 525 of 3,925 FP64 instructions (one
// trace contraction per pencil and direction instead of two, one product
// per face flux instead of two instructions) and 150 trace reads; measured
// on GB300 on 64^3 curved cells of degree 4: 1.717 instead of 2.107 ms per
// stage launch.
bool upwind_traces(const adv_handle &h)
{
  return h.cfg.flux_alpha == 1.0 && h.cfg.velocity_type == ADV_VELOCITY_CONSTANT && h.cfg.factor_skew == 0.0 &&
         !h.mesh.uniform && h.cfg.diffusion == 0.0;
}

int ensure_traces(adv_handle *h)
{
  const size_t nb = (size_t)h->mesh.n_cells * 6 * trace_width(*h) * h->mesh.n * h->mesh.n * sizeof(double);
  for (int i = 0; i < 2; ++i)
    if (!h->d_traces[i])
      {
        ADV_CUDA(cudaMalloc(&h->d_traces[i], nb));
        h->device_bytes += nb;
      }
  return ADV_OK;
}

int ensure_scratch(adv_handle *h, int i)
{
  if (!h->d_scratch[i])
    {
      ADV_CUDA(cudaMalloc(&h->d_scratch[i], h->mesh.n_dofs * sizeof(double)));
      h->device_bytes += h->mesh.n_dofs * sizeof(double);
    }
  return ADV_OK;
}

int check_device(const adv_handle *h)
{
  int dev = -1;
  ADV_CUDA(cudaGetDevice(&dev));
  if (dev != h->device)
    return fail(ADV_ERR_INVALID, "handle was created on another device than the current one");
  return ADV_OK;
}
} // namespace

// ---------------------------------------------------------------------------
// Static stage scratch of adv_perform_stage_noalloc.  Callers that cannot
// allocate device memory mid-solve (memory-budgeted serving, latency-critical
// loops, memory owned by another allocator) get the staging buffer for an
// output that aliases r_in from this file-scope array instead of a
// handle-owned vector.  In host code the array's name is a host-side shadow,
// not a device address: create_handle looks the device address up with the
// handle's device current and keeps it in the handle.  That lookup also
// loads this translation unit's module on the device (CUDA loads modules
// lazily), so the array's memory is committed when a handle is created and
// never inside a stage call; a handle lives no longer than the context its
// own buffers belong to, so its copy of the address cannot go stale.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double g_noalloc_stage_scratch[ADV_NOALLOC_MAX_DOFS];

namespace
{
int lookup_noalloc_scratch(double **out)
{
  void       *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_stage_scratch);
  if (e != cudaSuccess)
    return cuda_fail(e, "cudaGetSymbolAddress of the static stage scratch");
  *out = static_cast<double *>(p);
  return ADV_OK;
}
} // namespace

namespace adv
{
namespace detail
{
CallTrace::CallTrace(adv_handle *h, const char *name, cudaStream_t s) : h_(h), s_(s)
{
  nvtxRangePushA(name);
  // only the outermost traced call of a handle is timed (fgmres calls the
  // preconditioner, a BDF2 step calls fgmres)
  const bool outer = h_ && h_->trace_depth++ == 0;
  if (outer && h_->timing && cudaEventCreate(&e0_) == cudaSuccess && cudaEventRecord(e0_, s_) != cudaSuccess)
    {
      cudaEventDestroy(e0_);
      e0_ = nullptr;
    }
}

CallTrace::~CallTrace()
{
  if (e0_)
    {
      cudaEvent_t e1 = nullptr;
      if (cudaEventCreate(&e1) == cudaSuccess && cudaEventRecord(e1, s_) == cudaSuccess)
        h_->timed_events.emplace_back(e0_, e1);
      else
        {
          cudaEventDestroy(e0_);
          if (e1)
            cudaEventDestroy(e1);
        }
    }
  if (h_)
    --h_->trace_depth;
  nvtxRangePop();
}

adv::StageArgs base_args(const adv_handle &h, double t, int op_precision) { return ::base_args(h, t, op_precision); }
int            launch(adv_handle *h, const adv::StageArgs &A, cudaStream_t s) { return ::launch(h, A, s); }
int            check_device(const adv_handle *h) { return ::check_device(h); }
int            ensure_tables(int device) { return ::ensure_tables(device); }
} // namespace detail
} // namespace adv

extern "C" {

void adv_config_default(adv_config *c)
{
  std::memset(c, 0, sizeof(*c));
  c->degree = 3;
  for (int d = 0; d < 3; ++d)
    {
      c->n_cells[d]   = 8;
      c->domain_lo[d] = 0.0;
      c->domain_hi[d] = 1.0;
    }
  c->mesh_type         = ADV_MESH_CARTESIAN;
  c->periodic          = 1;
  c->velocity_type     = ADV_VELOCITY_CONSTANT;
  c->initial_condition = ADV_IC_SINE_GAUSS;
  c->velocity[0]       = 1.0;
  c->velocity[1]       = 0.15;
  c->velocity[2]       = -0.05;
  c->velocity_period   = 1.0;
  c->flux_alpha        = 1.0;
  c->penalty_factor    = 1.0;
  c->boundary_value    = ADV_BOUNDARY_EXACT;
  c->precision         = ADV_PRECISION_FP64;
}

const char *adv_last_error(void) { return g_last_error.c_str(); }

namespace
{
// z_end < 0: the whole mesh; else the slab of global z layers [z_begin, z_end)
int create_handle(const adv_config *cfg, int z_begin, int z_end, adv_handle **out)
{
  if (!cfg || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  *out = nullptr;
  if (int e = validate(*cfg))
    return e;
  if (z_end >= 0 && (z_begin < 0 || z_end > cfg->n_cells[2] || z_begin >= z_end))
    return fail(ADV_ERR_INVALID, "slab range must satisfy 0 <= z_begin < z_end <= n_cells[2]");
  auto *h = new adv_handle();
  h->cfg  = *cfg;
  int rc  = ADV_OK;
  do
    {
      cudaError_t e = cudaGetDevice(&h->device);
      if (e != cudaSuccess)
        {
          rc = cuda_fail(e, "cudaGetDevice");
          break;
        }
      if ((rc = ensure_tables(h->device)))
        break;
      if ((rc = lookup_noalloc_scratch(&h->noalloc_scratch)))
        break;
      if (z_end >= 0)
        adv::setup_slab(h->cfg, z_begin, z_end, h->mesh);
      else
        adv::setup_mesh(h->cfg, h->mesh);
      h->tb.init(h->cfg.degree);
      adv::HostGeometry g;
      adv::compute_geometry(h->cfg, h->mesh, h->tb, g);
      h->h_min = g.h_min;
      for (int d = 0; d < 3; ++d)
        h->cv[d] = g.cv[d], h->P[d] = g.P[d], h->M[d] = g.M[d];
      const bool fp64 = h->cfg.precision == ADV_PRECISION_FP64;
      const bool both = h->cfg.precision == ADV_PRECISION_FP32_INCREMENT;
      if (!g.cell.empty())
        {
          rc = fp64 ? upload_array<double>(g.cell, &h->d_cell_geo, h->device_bytes)
                    : upload_array<float>(g.cell, &h->d_cell_geo, h->device_bytes);
          if (rc == ADV_OK && both)
            rc = upload_array<double>(g.cell, (void **)&h->d_cell_geo64, h->device_bytes);
        }
      for (int d = 0; d < 3 && rc == ADV_OK; ++d)
        {
          if (!g.face[d].empty())
            {
              rc = fp64 ? upload_array<double>(g.face[d], &h->d_face_geo[d], h->device_bytes)
                        : upload_array<float>(g.face[d], &h->d_face_geo[d], h->device_bytes);
              if (rc == ADV_OK && both)
                rc = upload_array<double>(g.face[d], (void **)&h->d_face_geo64[d], h->device_bytes);
            }
          if (rc == ADV_OK && !g.face_x[d].empty())
            rc = upload_array<double>(g.face_x[d], (void **)&h->d_face_x[d], h->device_bytes);
        }
      if (rc)
        break;
      {
        std::vector<float> ff(g.fdm_cell.begin(), g.fdm_cell.end());
        const size_t       nb = g.fdm_cell.size();
        if ((e = cudaMalloc(&h->d_fdm_cell_d, nb * sizeof(double))) != cudaSuccess ||
            (e = cudaMalloc(&h->d_fdm_cell_f, nb * sizeof(float))) != cudaSuccess ||
            (e = cudaMemcpy(h->d_fdm_cell_d, g.fdm_cell.data(), nb * sizeof(double), cudaMemcpyHostToDevice)) !=
              cudaSuccess ||
            (e = cudaMemcpy(h->d_fdm_cell_f, ff.data(), nb * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
          {
            rc = cuda_fail(e, "FDM cell data");
            break;
          }
        h->device_bytes += nb * (sizeof(double) + sizeof(float));
      }
      e = cudaMalloc(&h->d_partials, 3 * 4096 * sizeof(double));
      if (e != cudaSuccess)
        {
          rc = cuda_fail(e, "cudaMalloc partials");
          break;
        }
      h->device_bytes += 3 * 4096 * sizeof(double);
      fill_diag(*h);
    }
  while (false);
  if (rc)
    {
      adv_destroy(h);
      return rc;
    }
  *out = h;
  return ADV_OK;
}
} // namespace

int adv_create(const adv_config *cfg, adv_handle **out)
{
  return create_handle(cfg, 0, -1, out);
}

int adv_create_slab(const adv_config *cfg, int z_begin, int z_end, adv_handle **out)
{
  return create_handle(cfg, z_begin, z_end, out);
}

int adv_slab_layout(const adv_config *cfg, int z_begin, int z_end, int64_t *out)
{
  if (!cfg || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  if (int e = validate(*cfg))
    return e;
  adv::Mesh m;
  if (adv::setup_slab(*cfg, z_begin, z_end, m))
    return fail(ADV_ERR_INVALID, "slab range must satisfy 0 <= z_begin < z_end <= n_cells[2]");
  const int64_t n3 = (int64_t)m.n * m.n * m.n;
  out[0] = m.n_dofs;
  out[1] = m.cell_begin * n3;
  out[2] = (m.cell_end - m.cell_begin) * n3;
  out[3] = (int64_t)m.nc[0] * m.nc[1];
  out[4] = n3;
  out[5] = m.ghost_lo;
  out[6] = m.ghost_hi;
  out[7] = cfg->diffusion != 0.0 ? n3 : (int64_t)m.n * m.n;
  out[8] = m.nc[2];
  out[9] = m.zoff;
  return ADV_OK;
}

int adv_set_timing(adv_handle *h, int enable)
{
  if (!h)
    return fail(ADV_ERR_INVALID, "null argument");
  h->timing = enable != 0;
  return ADV_OK;
}

int adv_timing(adv_handle *h, double *seconds, int64_t *calls)
{
  if (!h)
    return fail(ADV_ERR_INVALID, "null argument");
  for (auto &p : h->timed_events)
    {
      float ms = 0.0f;
      ADV_CUDA(cudaEventSynchronize(p.second));
      ADV_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
      h->timed_seconds += 1e-3 * ms;
      ++h->timed_calls;
      cudaEventDestroy(p.first);
      cudaEventDestroy(p.second);
    }
  h->timed_events.clear();
  if (seconds)
    *seconds = h->timed_seconds;
  if (calls)
    *calls = h->timed_calls;
  return ADV_OK;
}

int adv_destroy(adv_handle *h)
{
  if (!h)
    return ADV_OK;
  cudaFree(h->d_cell_geo);
  cudaFree(h->d_cell_geo64);
  for (int d = 0; d < 3; ++d)
    cudaFree(h->d_face_geo64[d]);
  for (int d = 0; d < 3; ++d)
    {
      cudaFree(h->d_face_geo[d]);
      cudaFree(h->d_face_x[d]);
    }
  cudaFree(h->d_partials);
  cudaFree(h->d_fdm_cell_d);
  cudaFree(h->d_fdm_cell_f);
  cudaFree(h->d_scratch[0]);
  cudaFree(h->d_scratch[1]);
  for (auto &p : h->timed_events)
    {
      cudaEventDestroy(p.first);
      cudaEventDestroy(p.second);
    }
  cudaFree(h->d_traces[0]);
  cudaFree(h->d_traces[1]);
  cudaFree(h->d_inc32);
  for (cudaEvent_t e : h->pipe_events)
    cudaEventDestroy(e);
  for (cudaStream_t cs : h->copy_stream)
    if (cs)
      cudaStreamDestroy(cs);
  delete h;
  return ADV_OK;
}

int adv_n_dofs(const adv_handle *h, int64_t *out)
{
  if (!h || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  *out = h->mesh.n_dofs;
  return ADV_OK;
}

int adv_n_cells(const adv_handle *h, int64_t *out)
{
  if (!h || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  *out = h->mesh.n_cells;
  return ADV_OK;
}

int adv_device_bytes(const adv_handle *h, int64_t *out)
{
  if (!h || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  *out = h->device_bytes;
  return ADV_OK;
}

int adv_launch_count(const adv_handle *h, int64_t *out)
{
  if (!h || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  *out = h->launches;
  return ADV_OK;
}

int adv_alloc_vector(adv_handle *h, double **out)
{
  if (!h || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  ADV_CUDA(cudaMalloc(out, h->mesh.n_dofs * sizeof(double)));
  ADV_CUDA(cudaMemset(*out, 0, h->mesh.n_dofs * sizeof(double)));
  return ADV_OK;
}

int adv_free_vector(adv_handle *h, double *vec)
{
  if (!h)
    return fail(ADV_ERR_INVALID, "null handle");
  ADV_CUDA(cudaFree(vec));
  return ADV_OK;
}

int adv_apply(adv_handle *h, const double *src, double *dst, double t, void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_apply", (cudaStream_t)stream);
  if (!h || !src || !dst)
    return fail(ADV_ERR_INVALID, "null argument");
  if (int e = check_device(h))
    return e;
  cudaStream_t   s = (cudaStream_t)stream;
  adv::StageArgs A = base_args(*h, t);
  A.mode           = adv::kModeApply;
  A.r_in           = src;
  double *target   = dst;
  if (src == dst)
    {
      if (int e = ensure_scratch(h, 0))
        return e;
      target = h->d_scratch[0];
    }
  A.r_out = target;
  if (int e = launch(h, A, s))
    return e;
  if (target != dst)
    ADV_CUDA(cudaMemcpyAsync(dst, target, h->mesh.n_dofs * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return ADV_OK;
}

int adv_perform_stage(adv_handle *h, double t, double b_dt, double a_dt, const double *r_in,
                      double *k, double *u, double *r_out, void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_perform_stage", (cudaStream_t)stream);
  if (!h || !r_in || !u || (a_dt != 0.0 && !r_out))
    return fail(ADV_ERR_INVALID, "null argument");
  if (a_dt != 0.0 && r_out == u)
    return fail(ADV_ERR_ALIASING, "r_out must not alias u");
  if (int e = check_device(h))
    return e;
  cudaStream_t   s   = (cudaStream_t)stream;
  const size_t   nb  = h->mesh.n_dofs * sizeof(double);
  adv::StageArgs A   = base_args(*h, t);
  const double   fac = A.out_scale;
  A.r_in             = r_in;
  A.u_in             = u;
  A.b                = b_dt * fac;
  A.a                = a_dt * fac;
  A.mode             = a_dt == 0.0 ? adv::kModeLastStage : adv::kModeStage;
  // outputs must not alias r_in, which neighbouring cells read concurrently
  double *u_target = u;
  if (u == r_in)
    {
      if (k && k != r_in && k != r_out && k != u)
        u_target = k;
      else
        {
          if (int e = ensure_scratch(h, 0))
            return e;
          u_target = h->d_scratch[0];
        }
    }
  double *r_target = r_out;
  if (a_dt != 0.0 && r_out == r_in)
    {
      if (k && k != r_in && k != u && k != u_target)
        r_target = k;
      else
        {
          if (int e = ensure_scratch(h, 1))
            return e;
          r_target = h->d_scratch[1];
        }
    }
  A.u_out = u_target;
  A.r_out = a_dt != 0.0 ? r_target : nullptr;
  if (int e = launch(h, A, s))
    return e;
  if (u_target != u)
    ADV_CUDA(cudaMemcpyAsync(u, u_target, nb, cudaMemcpyDeviceToDevice, s));
  if (a_dt != 0.0 && r_target != r_out)
    ADV_CUDA(cudaMemcpyAsync(r_out, r_target, nb, cudaMemcpyDeviceToDevice, s));
  return ADV_OK;
}

int adv_lsrk_coefficients(int scheme, double *a, double *b, int *n_stages)
{
  std::vector<double> av, bv;
  if (!adv::lsrk_coefficients(scheme, av, bv))
    return fail(ADV_ERR_INVALID, "unknown LSRK scheme");
  if (a)
    for (size_t i = 0; i < av.size(); ++i)
      a[i] = av[i];
  if (b)
    for (size_t i = 0; i < bv.size(); ++i)
      b[i] = bv[i];
  if (n_stages)
    *n_stages = (int)bv.size();
  return ADV_OK;
}

// Time steps of LowStorageRungeKuttaIntegrator::perform_time_step
// (advection_solver.cc:906-939) on caller buffers U (solution), R, K.
// Stage 0 reads U and writes u' to K and r to R; stage 1 reads R, writes u'
// back to U and r to K (each element of K is read as u before it is
// overwritten as r by the same thread); later stages read r from the buffer
// written by the previous stage, write the next r to the other one and
// update U in place.  No stage writes a buffer that neighbouring cells read,
// and the solution ends in U without copies.
extern "C++" {
namespace
{
// stage time of stage st of the step starting at t0 (the reference's
// accumulation order, advection_solver.cc:916-935)
double stage_time(const std::vector<double> &ai, const std::vector<double> &bi, double t0, double dt, int st)
{
  if (st == 0)
    return t0;
  double sum_previous_bi = 0.0;
  for (int j = 0; j + 1 < st; ++j)
    sum_previous_bi += bi[j];
  return t0 + (sum_previous_bi + ai[st - 1]) * dt;
}

// Stage st of step `step` of the plain step loop.  With face traces, stage g
// = step * n_stages + st reads the traces of its input from d_traces[g & 1]
// (the basis change writes those of u into d_traces[0]) and writes those of
// its output into the other buffer.
int plain_stage(adv_handle *h, const std::vector<double> &ai, const std::vector<double> &bi, double t, double dt,
                int step, int st, bool gauss, bool traces, double *u, double *r, double *k, adv::StageArgs &A,
                int &prec)
{
  const int ns = (int)bi.size();
  A            = base_args(*h, stage_time(ai, bi, t + step * dt, dt, st));
  prec         = -1;
  const double fac  = A.out_scale;
  const bool   last = st == ns - 1;
  A.gauss           = gauss;
  if (traces)
    {
      const long long g = (long long)step * ns + st;
      A.tr_in           = h->d_traces[g & 1];
      A.tr_out          = h->d_traces[(g + 1) & 1];
      A.upwind_tr       = upwind_traces(*h);
    }
  A.b    = bi[st] * dt * fac;
  A.a    = last ? 0.0 : ai[st] * dt * fac;
  A.mode = last ? adv::kModeLastStage : adv::kModeStage;
  if (st == 0)
    {
      A.r_in = u, A.u_in = u, A.u_out = k, A.r_out = r;
    }
  else if (st == 1)
    {
      A.r_in = r, A.u_in = k, A.u_out = u, A.r_out = k;
    }
  else
    {
      double *rin  = (st % 2 == 0) ? k : r;
      double *rout = (st % 2 == 0) ? r : k;
      A.r_in = rin, A.u_in = u, A.u_out = u, A.r_out = last ? nullptr : rout;
    }
  return ADV_OK;
}

// FP32 increments (ADV_PRECISION_FP32_INCREMENT).  Steps come in blocks of
// m = anchor_interval steps.  The first stage of a block's first step runs
// the FP64 operator on the block's start value B (= u) and writes K0 = L(B),
// E = b0 dt K0 and G = a0 dt K0, the increments u - B and r - B.  Every other
// stage of the block evaluates k = K0 + L32(G) with the FP32 operator and
// updates E and G in FP64.  The first stage of a later step of the block
// takes G = E (the step's start value relative to B).  The last stage of the
// block writes B + E + b dt k into u; the last stage of the block's other
// steps only updates E.  Buffers: u holds B, K0 a scratch vector, and E and
// the two G registers rotate over r, k and a second scratch vector: in the
// block's step j, E is in P[j % 3] and G in P[(j + 1) % 3], P[(j + 2) % 3].
int increment_stage(adv_handle *h, const std::vector<double> &ai, const std::vector<double> &bi, double t,
                    double dt, int n_steps, int step, int st, bool gauss, double *u, double *r, double *k,
                    adv::StageArgs &A, int &prec)
{
  const int ns = (int)bi.size();
  const int m  = h->cfg.anchor_interval > 0 ? h->cfg.anchor_interval : 4;
  const int j  = step % m;
  double   *P[3] = {r, k, h->d_scratch[0]}, *K0 = h->d_scratch[1];
  double   *E = P[j % 3], *Ga = P[(j + 1) % 3], *Gb = P[(j + 2) % 3];
  const bool anchor = j == 0 && st == 0;
  prec              = anchor ? 0 : 1;
  A                 = base_args(*h, stage_time(ai, bi, t + step * dt, dt, st), prec);
  const bool last   = st == ns - 1;
  A.gauss           = gauss;
  A.b               = bi[st] * dt * A.out_scale;
  A.a               = last ? 0.0 : ai[st] * dt * A.out_scale;
  A.mode            = last ? adv::kModeLastStage : adv::kModeStage;
  if (anchor)
    {
      A.r_in = u, A.u_in = nullptr, A.u_out = E, A.r_out = Ga, A.k_out = K0;
      return ADV_OK;
    }
  A.k_add = K0;
  if (st == 0)
    {
      // E of the previous step (in P[(j - 1) % 3] = Gb) is this step's start
      A.r_in = Gb, A.u_in = Gb, A.u_out = E, A.r_out = Ga;
      return ADV_OK;
    }
  A.r_in = (st % 2) ? Ga : Gb;
  A.u_in = E;
  if (!last)
    A.u_out = E, A.r_out = (st % 2) ? Gb : Ga;
  else if (j == m - 1 || step == n_steps - 1)
    A.u_out = u, A.u_base = u;
  else
    A.u_out = E;
  return ADV_OK;
}

// values per binary32 register of the increment form: n_dofs rounded up to 4,
// so that every register starts on 16 bytes
int64_t inc32_stride(const adv_handle &h)
{
  return (h.mesh.n_dofs + 3) / 4 * 4;
}

// FP32 increments in the collocation form, with the anchor's K0 folded out
// of the FP64 registers.  Within a block, with C the sum of the b dt of the
// stages since the anchor, the kernels carry e = u - u_a - C K0 (FP64) and
// the next operator input G = r - u_a only in binary32 (the FP32 operator
// reads nothing finer), which with k = K0 + kh, kh = L32(G), turns
//   E' = E + b k,  G' = E + a k    into    e' = e + b kh,  G' = e + (C + a) K0 + a kh
// with K0 read in binary32 for G' and in FP64 once, at the end of the block:
//   u = u_a + e + b kh + (C + b) K0.
// The anchor writes K0 (FP64 and binary32) and G = a0 dt K0; e starts at 0.
// A stage reads 4 + 8 + 4 and writes 8 + 4 bytes per DoF instead of 24 + 16,
// and issues one FP64 instruction per DoF instead of two.  The last stage of
// a step inside a block writes the next step's start G = e' + (C + b) K0.
// Buffers: u holds u_a, K0 lives in k and e in r; the two G registers and K0
// in binary32 share one allocation of 3 n_dofs floats.
// The anchor reads the face traces of u_a (field geometry without SIPG): the
// change of basis writes them for the first block, a traces-only launch for
// the later blocks of the call (750 FP64 FMAs per cell against the 1,500 the
// anchor saves; it writes no traces itself, another 750).
bool anchor_traces(const adv_handle &h)
{
  return !h.mesh.uniform && h.cfg.diffusion == 0.0;
}

int increment_stage_folded(adv_handle *h, const std::vector<double> &ai, const std::vector<double> &bi, double t,
                           double dt, int n_steps, int step, int st, double *u, double *r, double *k,
                           adv::StageArgs &A, int &prec, cudaStream_t s)
{
  const int ns     = (int)bi.size();
  const int m      = h->cfg.anchor_interval > 0 ? h->cfg.anchor_interval : 4;
  const int j      = step % m;
  const int q      = j * ns + st; // stage index inside the block
  const int64_t nd = inc32_stride(*h);
  float    *G[2]   = {h->d_inc32, h->d_inc32 + nd}, *K32 = h->d_inc32 + 2 * nd;
  double   *K0     = k;
  prec             = q == 0 ? 0 : 1;
  A                = base_args(*h, stage_time(ai, bi, t + step * dt, dt, st), prec);
  A.gauss          = true;
  A.inc32          = 1;
  A.mode           = adv::kModeStage;
  if (q == 0)
    {
      A.r_in  = u;
      A.a     = ai[0] * dt * A.out_scale;
      A.k_out = K0, A.k_out32 = K32, A.r_out32 = G[0];
      if (anchor_traces(*h))
        {
          double *tr = static_cast<double *>(h->d_traces[0]);
          if (step > 0)
            {
              const adv::StageArgs F = base_args(*h, 0.0, 0);
              ADV_CUDA(adv::launch_face_traces(h->mesh.n, u, h->mesh.cell_begin, h->mesh.cell_end, s, tr, 1,
                                               upwind_traces(*h) ? &F : nullptr));
              ++h->launches;
            }
          A.tr_in     = tr;
          A.upwind_tr = upwind_traces(*h);
        }
      return ADV_OK;
    }
  // C: the b dt of the stages since the anchor, summed in stage order
  double C = 0.0;
  for (int p = 0; p < q; ++p)
    C += bi[p % ns] * dt * A.out_scale;
  const bool last_of_step  = st == ns - 1;
  const bool last_of_block = last_of_step && (j == m - 1 || step == n_steps - 1);
  A.b       = bi[st] * dt * A.out_scale;
  A.r_in32  = G[(q - 1) & 1];
  A.u_in    = q == 1 ? nullptr : r;
  A.u_out   = r;
  if (last_of_block)
    {
      A.mode      = adv::kModeLastStage;
      A.inc_alpha = C + A.b;
      A.k_add     = K0;
      A.u_base    = u;
      A.u_out     = u;
      return ADV_OK;
    }
  // inside a step: G' = e + (C + a) K0 + a kh; at the end of a step: the
  // next step's start, e' + (C + b) K0 = e + (C + b) K0 + b kh
  const double a = last_of_step ? A.b : ai[st] * dt * A.out_scale;
  A.inc_af       = (float)a;
  A.inc_alphaf   = (float)(C + a);
  A.k_add32      = K32;
  A.r_out32      = G[q & 1];
  return ADV_OK;
}

int ensure_inc32(adv_handle *h)
{
  if (!h->d_inc32)
    {
      ADV_CUDA(cudaMalloc(&h->d_inc32, 3 * inc32_stride(*h) * sizeof(float)));
      h->device_bytes += 3 * inc32_stride(*h) * (int64_t)sizeof(float);
    }
  return ADV_OK;
}

// the increment form is exact for operators linear in u and independent of
// time: constant velocity, no inhomogeneous (exact) Dirichlet data
bool increment_form_applies(const adv_handle &h)
{
  return h.cfg.precision == ADV_PRECISION_FP32_INCREMENT && h.cfg.velocity_type == ADV_VELOCITY_CONSTANT &&
         (h.mesh.periodic || h.cfg.boundary_value != ADV_BOUNDARY_EXACT);
}

// Copies of a host solution in z-layer chunks (adv_lsrk_steps_host): chunk c
// holds the layers [z[c], z[c + 1]), a contiguous range of cells.
struct HostChunks
{
  std::vector<int> z;
  int64_t          layer_cells = 0, cell_dofs = 0;
  int              count() const { return (int)z.size() - 1; }
  int64_t          cell(int layer) const { return layer * layer_cells; }
  int64_t          dof(int layer) const { return layer * layer_cells * cell_dofs; }
};

HostChunks plan_chunks(const adv::Mesh &m)
{
  // 8 chunks at most, 2 MB at least.  Measured on GB300 with the 262 MB
  // solution of 64^3 degree-4 cells (FP64 step 13.6 ms without copies, each
  // copy 1.24-1.36 ms): 4 chunks 14.46 ms, 8 chunks 14.28 ms, 16 chunks
  // 14.37 ms, 32 chunks 14.85 ms per step with the copies
  HostChunks    c;
  const int     nz    = m.nc[2];
  c.layer_cells       = (int64_t)m.nc[0] * m.nc[1];
  c.cell_dofs         = (int64_t)m.n * m.n * m.n;
  const int64_t bytes = m.n_dofs * (int64_t)sizeof(double);
  int           k     = (int)std::min<int64_t>(std::min(nz, 8), std::max<int64_t>(1, bytes / (2 << 20)));
  // the last chunk is small (1/32 of the layers): its basis change after the
  // end of the copies in and its copy out after the end of the last stage are
  // the parts the pipeline cannot hide
  const int tail = k > 1 ? std::max(1, nz / 32) : 0;
  const int big  = tail ? k - 1 : k; // chunks before the tail
  for (int i = 0; i < big; ++i)
    c.z.push_back((int)((int64_t)(nz - tail) * i / big));
  if (tail)
    c.z.push_back(nz - tail);
  c.z.push_back(nz);
  c.z.erase(std::unique(c.z.begin(), c.z.end()), c.z.end()); // no empty chunk
  return c;
}

int ensure_copy_pipe(adv_handle *h, size_t n_events)
{
  for (cudaStream_t &cs : h->copy_stream)
    if (!cs)
      ADV_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  while (h->pipe_events.size() < n_events)
    {
      cudaEvent_t e = nullptr;
      ADV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      h->pipe_events.push_back(e);
    }
  return ADV_OK;
}

// The step loop shared by the plain and the increment forms.  stage(step, st,
// A, prec) fills the arguments of one whole-mesh stage launch.  With gauss
// the solution moves to the Gauss-point values before the steps and back
// afterwards (cell by cell; with traces the first change writes the face
// traces of u as well).
//
// With host != nullptr the solution comes from and goes back to host memory,
// in z-layer chunks on the handle's copy streams.  Chunk c's copy in is
// followed on the compute stream by its basis change (collocation form) or,
// in the nodal form, the first stage of the first step runs chunk by chunk as
// soon as a chunk and the layers next to it have arrived.  The last stage of
// the last step runs chunk by chunk, each chunk followed by its basis change
// back and its copy out.  Every cell gets the same arithmetic as in the
// whole-mesh launches, so the results are the same bit for bit.
//
// In the collocation form the first stage runs on the whole mesh after the
// copies: measured on GB300 (64^3 degree-4 cells, FP64) a chunked first stage
// overlapping the copies in was 0.15 ms slower per call (14.43 against 14.28
// ms; the copies write through the L2 the stage reads its neighbours from),
// while the basis change alone, cell-local streaming, hides most of the 1.24
// ms copy.
template <typename StageFn>
int run_steps(adv_handle *h, int n_steps, int ns, bool gauss, bool traces, double *u, double *host, cudaStream_t s,
              StageFn stage)
{
  const int64_t cb = h->mesh.cell_begin, ce = h->mesh.cell_end;
  const int     n  = h->mesh.n;
  double       *tr_basis = traces ? static_cast<double *>(h->d_traces[0]) : nullptr;
  // the traces the first stage reads: only the upwind ones where it reads those
  adv::StageArgs upw;
  if (traces && upwind_traces(*h))
    upw = base_args(*h, 0.0, 0);
  const adv::StageArgs *tr_upwind = traces && upwind_traces(*h) ? &upw : nullptr;
  HostChunks    ch;
  int           nch = 0;
  if (host)
    {
      ch  = plan_chunks(h->mesh);
      nch = ch.count();
      if (int e = ensure_copy_pipe(h, 2 * (size_t)nch + 2))
        return e;
    }
  cudaEvent_t *ev      = h->pipe_events.data();
  auto         launch_range = [&](adv::StageArgs A, int prec, int z0, int z1) {
    A.cell_begin = ch.cell(z0);
    A.n_cells    = ch.cell(z1);
    return launch(h, A, s, prec);
  };
  if (host)
    {
      // copy in: chunk c on copy stream 0 after the work already on s; with
      // the first stage run chunk by chunk (nodal form) on a periodic mesh the
      // top chunk goes first, so that the bottom chunk's first stage does not
      // wait for the end of the copies
      const int         nz   = h->mesh.nc[2];
      const bool        wrap = h->mesh.periodic;
      std::vector<int>  order;
      if (wrap && nch > 2 && !gauss)
        order.push_back(nch - 1);
      for (int c = 0; (int)order.size() < nch; ++c)
        order.push_back(c);
      cudaStream_t in = h->copy_stream[0];
      ADV_CUDA(cudaEventRecord(ev[0], s));
      ADV_CUDA(cudaStreamWaitEvent(in, ev[0], 0));
      for (int c : order)
        {
          const int64_t d0 = ch.dof(ch.z[c]), d1 = ch.dof(ch.z[c + 1]);
          ADV_CUDA(cudaMemcpyAsync(u + d0, host + d0, (d1 - d0) * sizeof(double), cudaMemcpyHostToDevice, in));
          ADV_CUDA(cudaEventRecord(ev[1 + c], in));
        }
      adv::StageArgs A0;
      int            prec0 = -1;
      if (n_steps > 0)
        if (int e = stage(0, 0, A0, prec0))
          return e;
      std::vector<char> arrived(nz, 0), staged(nch, 0);
      auto              ready = [&](int layer) {
        if (layer < 0 || layer >= nz)
          return wrap ? arrived[(layer + nz) % nz] != 0 : true;
        return arrived[layer] != 0;
      };
      for (int c : order)
        {
          ADV_CUDA(cudaStreamWaitEvent(s, ev[1 + c], 0));
          if (gauss)
            {
              ADV_CUDA(adv::launch_basis_change(n, u, ch.cell(ch.z[c]), ch.cell(ch.z[c + 1]), true, s, tr_basis,
                                                trace_width(*h), tr_upwind));
              ++h->launches;
            }
          for (int l = ch.z[c]; l < ch.z[c + 1]; ++l)
            arrived[l] = 1;
          if (n_steps == 0 || gauss)
            continue;
          // first stage of every chunk whose cells and neighbour layers are in
          for (int j = 0; j < nch; ++j)
            if (!staged[j] && ready(ch.z[j] - 1) && ready(ch.z[j + 1]))
              {
                bool all = true;
                for (int l = ch.z[j]; l < ch.z[j + 1]; ++l)
                  all = all && arrived[l];
                if (!all)
                  continue;
                if (int e = launch_range(A0, prec0, ch.z[j], ch.z[j + 1]))
                  return e;
                staged[j] = 1;
              }
        }
    }
  else if (gauss)
    {
      ADV_CUDA(adv::launch_basis_change(n, u, cb, ce, true, s, tr_basis, trace_width(*h), tr_upwind));
      ++h->launches;
    }
  for (int step = 0; step < n_steps; ++step)
    for (int st = 0; st < ns; ++st)
      {
        if (host && step == 0 && st == 0 && !gauss)
          continue; // ran chunk by chunk with the copies in
        adv::StageArgs A;
        int            prec = -1;
        if (int e = stage(step, st, A, prec))
          return e;
        if (!(host && step == n_steps - 1 && st == ns - 1))
          {
            if (int e = launch(h, A, s, prec))
              return e;
            continue;
          }
        // last stage with the copies out: chunk c on copy stream 1 after its
        // stage and basis change
        cudaStream_t out = h->copy_stream[1];
        for (int c = 0; c < nch; ++c)
          {
            if (int e = launch_range(A, prec, ch.z[c], ch.z[c + 1]))
              return e;
            if (gauss)
              {
                ADV_CUDA(adv::launch_basis_change(n, u, ch.cell(ch.z[c]), ch.cell(ch.z[c + 1]), false, s));
                ++h->launches;
              }
            const int64_t d0 = ch.dof(ch.z[c]), d1 = ch.dof(ch.z[c + 1]);
            ADV_CUDA(cudaEventRecord(ev[1 + nch + c], s));
            ADV_CUDA(cudaStreamWaitEvent(out, ev[1 + nch + c], 0));
            ADV_CUDA(cudaMemcpyAsync(host + d0, u + d0, (d1 - d0) * sizeof(double), cudaMemcpyDeviceToHost, out));
          }
        ADV_CUDA(cudaEventRecord(ev[1 + 2 * nch], out));
        ADV_CUDA(cudaStreamWaitEvent(s, ev[1 + 2 * nch], 0));
      }
  if (gauss && !host)
    {
      ADV_CUDA(adv::launch_basis_change(n, u, cb, ce, false, s));
      ++h->launches;
    }
  return ADV_OK;
}

int lsrk_steps_impl(adv_handle *h, int scheme, double t, double dt, int n_steps, double *u, double *r, double *k,
                    double *host, cudaStream_t s)
{
  if (!h || !u || !r || !k)
    return fail(ADV_ERR_INVALID, "null argument");
  if (u == r || u == k || r == k)
    return fail(ADV_ERR_ALIASING, "u, r and k must be distinct buffers");
  if (n_steps < 0)
    return fail(ADV_ERR_INVALID, "n_steps must be >= 0");
  if (h->mesh.slab)
    return fail(ADV_ERR_INVALID, "a slab needs its ghost layers exchanged before every stage: "
                                 "call adv_perform_stage per stage");
  if (int e = check_device(h))
    return e;
  std::vector<double> ai, bi;
  if (!adv::lsrk_coefficients(scheme, ai, bi))
    return fail(ADV_ERR_INVALID, "unknown LSRK scheme");
  const int ns = (int)bi.size();
  if (ns == 1)
    return fail(ADV_ERR_INVALID, "one-stage schemes are not supported");
  if (host && n_steps == 0)
    {
      ADV_CUDA(cudaMemcpyAsync(u, host, h->mesh.n_dofs * sizeof(double), cudaMemcpyHostToDevice, s));
      return ADV_OK;
    }
  if (increment_form_applies(*h))
    {
      const bool gauss = n_steps > 0 && h->cfg.fused_form != ADV_FORM_NODAL;
      if (gauss)
        {
          if (int e = ensure_inc32(h))
            return e;
          const bool tr = anchor_traces(*h);
          if (tr)
            if (int e = ensure_traces(h))
              return e;
          return run_steps(h, n_steps, ns, true, tr, u, host, s,
                           [&](int step, int st, adv::StageArgs &A, int &prec) {
                             return increment_stage_folded(h, ai, bi, t, dt, n_steps, step, st, u, r, k, A, prec,
                                                           s);
                           });
        }
      if (int e = ensure_scratch(h, 0))
        return e;
      if (int e = ensure_scratch(h, 1))
        return e;
      return run_steps(h, n_steps, ns, gauss, false, u, host, s,
                       [&](int step, int st, adv::StageArgs &A, int &prec) {
                         return increment_stage(h, ai, bi, t, dt, n_steps, step, st, gauss, u, r, k, A, prec);
                       });
    }
  // collocation form: the solution moves to the Gauss-point values for the
  // steps and back afterwards (r and k are scratch either way)
  const bool gauss  = n_steps > 0 && use_collocation(*h);
  const bool traces = gauss && use_traces(*h);
  if (traces)
    if (int e = ensure_traces(h))
      return e;
  return run_steps(h, n_steps, ns, gauss, traces, u, host, s, [&](int step, int st, adv::StageArgs &A, int &prec) {
    return plain_stage(h, ai, bi, t, dt, step, st, gauss, traces, u, r, k, A, prec);
  });
}
} // namespace
} // extern "C++"

int adv_lsrk_steps(adv_handle *h, int scheme, double t, double dt, int n_steps, double *u, double *r,
                   double *k, void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_lsrk_steps", (cudaStream_t)stream);
  return lsrk_steps_impl(h, scheme, t, dt, n_steps, u, r, k, nullptr, (cudaStream_t)stream);
}

int adv_lsrk_steps_host(adv_handle *h, int scheme, double t, double dt, int n_steps, double *u_host, double *u,
                        double *r, double *k, void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_lsrk_steps_host", (cudaStream_t)stream);
  if (!u_host)
    return fail(ADV_ERR_INVALID, "null argument");
  return lsrk_steps_impl(h, scheme, t, dt, n_steps, u, r, k, u_host, (cudaStream_t)stream);
}

int adv_lsrk_step(adv_handle *h, int scheme, double t, double dt, double *u, double *r, double *k,
                  void *stream)
{
  return adv_lsrk_steps(h, scheme, t, dt, 1, u, r, k, stream);
}

int adv_project(adv_handle *h, double t, double *dst, void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_project", (cudaStream_t)stream);
  if (!h || !dst)
    return fail(ADV_ERR_INVALID, "null argument");
  if (int e = check_device(h))
    return e;
  ADV_CUDA(adv::launch_project(h->diag, t, dst, (cudaStream_t)stream));
  ++h->launches;
  return ADV_OK;
}

int adv_mass_energy(adv_handle *h, const double *u, double out[3], void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_mass_energy", (cudaStream_t)stream);
  if (!h || !u || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  if (int e = check_device(h))
    return e;
  cudaStream_t s = (cudaStream_t)stream;
  int          nb = 0;
  ADV_CUDA(adv::launch_mass_energy(h->diag, u, h->d_partials, &nb, s));
  ++h->launches;
  std::vector<double> part(3 * nb);
  ADV_CUDA(cudaMemcpyAsync(part.data(), h->d_partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  ADV_CUDA(cudaStreamSynchronize(s));
  out[0] = out[1] = out[2] = 0.0;
  for (int b = 0; b < nb; ++b)
    for (int i = 0; i < 3; ++i)
      out[i] += part[3 * b + i];
  return ADV_OK;
}

int adv_l2_error(adv_handle *h, const double *u, double t, double out[2], void *stream)
{
  adv::detail::CallTrace trace_(h, "adv_l2_error", (cudaStream_t)stream);
  if (!h || !u || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  if (int e = check_device(h))
    return e;
  cudaStream_t s = (cudaStream_t)stream;
  int          nb = 0;
  ADV_CUDA(adv::launch_l2_error(h->diag, u, t, h->d_partials, &nb, s));
  ++h->launches;
  std::vector<double> part(3 * nb);
  ADV_CUDA(cudaMemcpyAsync(part.data(), h->d_partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  ADV_CUDA(cudaStreamSynchronize(s));
  double e2 = 0.0, n2 = 0.0;
  for (int b = 0; b < nb; ++b)
    e2 += part[3 * b], n2 += part[3 * b + 1];
  out[0] = std::sqrt(e2);
  out[1] = std::sqrt(n2);
  return ADV_OK;
}

int adv_time_step(adv_handle *h, double courant, double *dt)
{
  if (!h || !dt)
    return fail(ADV_ERR_INVALID, "null argument");
  const double *a    = h->cfg.velocity;
  const double  anrm = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double  nu   = h->cfg.diffusion;
  if (!(anrm > 0.0) && !(nu > 0.0))
    return fail(ADV_ERR_INVALID, "zero velocity");
  // advective limit of setup_dofs (advection_solver.cc:1155-1165)
  const double dt_a = courant * h->h_min / anrm / std::pow(std::max(1, h->cfg.degree), 1.5);
  // explicit SIPG: the spectral radius of M^{-1} A_diff is at most about
  // 7 nu (k+1)^4 / h^2 with the penalty (k+1)^2 / h (power iteration, k = 1..6),
  // LSRK(5,4) is stable on the negative real axis down to -4.8; the diffusive
  // limit 0.3 h^2 / (nu (k+1)^4) keeps its eigenvalues within -2.1 and is
  // combined harmonically with the advective one
  const double k1 = h->cfg.degree + 1.0;
  if (!(nu > 0.0))
    *dt = dt_a;
  else
    {
      const double dt_d = 0.3 * h->h_min * h->h_min / (nu * k1 * k1 * k1 * k1);
      *dt               = anrm > 0.0 ? 1.0 / (1.0 / dt_a + 1.0 / dt_d) : dt_d;
    }
  return ADV_OK;
}

int adv_copy_to_host(adv_handle *h, const double *dev, double *host, void *stream)
{
  if (!h || !dev || !host)
    return fail(ADV_ERR_INVALID, "null argument");
  ADV_CUDA(cudaMemcpyAsync(host, dev, h->mesh.n_dofs * sizeof(double), cudaMemcpyDeviceToHost,
                           (cudaStream_t)stream));
  return ADV_OK;
}

int adv_copy_from_host(adv_handle *h, const double *host, double *dev, void *stream)
{
  if (!h || !dev || !host)
    return fail(ADV_ERR_INVALID, "null argument");
  ADV_CUDA(cudaMemcpyAsync(dev, host, h->mesh.n_dofs * sizeof(double), cudaMemcpyHostToDevice,
                           (cudaStream_t)stream));
  return ADV_OK;
}

int adv_fdm_tables(int degree, double flux_alpha, int sign_index, double *lambda, double *V,
                   double *VinvW, double *A1, double *residual)
{
  if (degree < 1 || degree > 6 || (sign_index != 0 && sign_index != 1))
    return fail(ADV_ERR_INVALID, "degree must be in 1..6 and sign_index 0 or 1");
  adv::FdmTables t;
  if (!adv::fdm_tables(degree, flux_alpha, t))
    return fail(ADV_ERR_NOT_CONVERGED, "eigen-decomposition of the 1D operator did not converge");
  const int n = t.n;
  for (int i = 0; i < n; ++i)
    {
      if (lambda)
        lambda[2 * i] = t.lambda[sign_index][i].real(), lambda[2 * i + 1] = t.lambda[sign_index][i].imag();
      for (int j = 0; j < n; ++j)
        {
          if (V)
            V[2 * (i * n + j)] = t.V[sign_index][i * n + j].real(),
                          V[2 * (i * n + j) + 1] = t.V[sign_index][i * n + j].imag();
          if (VinvW)
            VinvW[2 * (i * n + j)] = t.VinvW[sign_index][i * n + j].real(),
                              VinvW[2 * (i * n + j) + 1] = t.VinvW[sign_index][i * n + j].imag();
          if (A1)
            A1[i * n + j] = t.A1[sign_index][i * n + j];
        }
    }
  if (residual)
    *residual = t.residual;
  return ADV_OK;
}

int adv_measure_fma_peak(int precision, double *tflops, void *stream)
{
  if (!tflops || precision < 0 || precision > 2)
    return fail(ADV_ERR_INVALID, "bad argument");
  cudaStream_t s   = (cudaStream_t)stream;
  int          dev = 0, sms = 0;
  ADV_CUDA(cudaGetDevice(&dev));
  ADV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8;
  double   *buf    = nullptr;
  ADV_CUDA(cudaMalloc(&buf, (size_t)blocks * 256 * sizeof(double)));
  const int   iters = precision == 1 ? 65536 : 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int   rc   = ADV_OK;
  for (int rep = 0; rep < 3 && rc == ADV_OK; ++rep)
    {
      cudaEventRecord(e0, s);
      cudaError_t e = adv::launch_fma_peak(precision, buf, iters, blocks, s);
      cudaEventRecord(e1, s);
      if (e == cudaSuccess)
        e = cudaEventSynchronize(e1);
      if (e != cudaSuccess)
        rc = cuda_fail(e, "fma peak kernel");
      else
        {
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          best = ms < best ? ms : best;
        }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (rc)
    return rc;
  // FMA-equivalent TFLOP/s: 2 x instructions per second
  *tflops = 2.0 * adv::fma_peak_chains(precision) * iters * (double)blocks * 256 / (best * 1e-3) / 1e12;
  return ADV_OK;
}

} // extern "C"

extern "C" int adv_perform_stage_noalloc(adv_handle *h, double t, double b_dt, double a_dt,
                                         const double *r_in, double *k, double *u, double *r_out,
                                         void *stream)
{
  (void)k; // scratch in the reference's semantics; this variant does not need it
  // NVTX range and optional call timing like every other entry point (event
  // records, no device memory)
  adv::detail::CallTrace trace_(h, "adv_perform_stage_noalloc", (cudaStream_t)stream);
  if (!h || !r_in || !u || (a_dt != 0.0 && !r_out))
    return fail(ADV_ERR_INVALID, "null argument");
  if (a_dt != 0.0 && r_out == u)
    return fail(ADV_ERR_ALIASING, "r_out must not alias u");
  if (h->mesh.n_dofs > (int64_t)ADV_NOALLOC_MAX_DOFS)
    return fail(ADV_ERR_INVALID, "adv_perform_stage_noalloc: the mesh has " + std::to_string(h->mesh.n_dofs) +
                                   " DoFs, more than the static scratch of ADV_NOALLOC_MAX_DOFS = " +
                                   std::to_string((long long)ADV_NOALLOC_MAX_DOFS) +
                                   "; use adv_perform_stage");
  if (int e = check_device(h))
    return e;
  double *scratch = h->noalloc_scratch;
  if (!scratch)
    return fail(ADV_ERR_INVALID, "handle has no static stage scratch address");
  cudaStream_t   s   = (cudaStream_t)stream;
  const size_t   nb  = h->mesh.n_dofs * sizeof(double);
  adv::StageArgs A   = base_args(*h, t);
  const double   fac = A.out_scale;
  A.r_in             = r_in;
  A.u_in             = u;
  A.b                = b_dt * fac;
  A.a                = a_dt * fac;
  A.mode             = a_dt == 0.0 ? adv::kModeLastStage : adv::kModeStage;
  // an output aliasing r_in (read by neighbouring cells during the kernel) is
  // staged in the static array; u == r_in and r_out == r_in cannot both hold
  // because r_out == u is rejected above
  double *u_target = u == r_in ? scratch : u;
  double *r_target = (a_dt != 0.0 && r_out == r_in) ? scratch : r_out;
  A.u_out          = u_target;
  A.r_out          = a_dt != 0.0 ? r_target : nullptr;
  if (int e = launch(h, A, s))
    return e;
  if (u_target != u)
    ADV_CUDA(cudaMemcpyAsync(u, u_target, nb, cudaMemcpyDeviceToDevice, s));
  if (a_dt != 0.0 && r_target != r_out)
    ADV_CUDA(cudaMemcpyAsync(r_out, r_target, nb, cudaMemcpyDeviceToDevice, s));
  return ADV_OK;
}

namespace adv
{
cudaError_t launch_stage(int n, int precision, const StageArgs &args, cudaStream_t stream)
{
  return precision == 0 ? launch_stage_fp64(n, args, stream) : launch_stage_fp32(n, args, stream);
}
int stage_cells_per_block(int n, int precision)
{
  return precision == 0 ? stage_cells_per_block_fp64(n) : stage_cells_per_block_fp32(n);
}
} // namespace adv
