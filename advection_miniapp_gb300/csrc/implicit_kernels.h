// Launch interface of the implicit-solver kernels (implicit_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "device_common.cuh"

namespace adv
{
struct FdmArgs
{
  const double *src;
  double       *dst;
  long long     n_cells;
  double        mass_factor; // c in (c M + A)
  double        time_factor; // velocity factor s of the rotating field (1 for constant)
  int           gauss;       // residual and result on the Gauss-point basis (no S^{-T}, S^{-1} transforms)
};

struct MassArgs
{
  const double *src;
  double       *dst;
  long long     n_cells;
  int           uniform;
  double        vol;      // uniform case: cell volume
  const double *cell_geo; // field case: [vt0|vt1|vt2|idet] blocks (FP64)
};

cudaError_t upload_tables_implicit(const DevTables<double> *d, const DevTables<float> *f);
// tables: per sign [VWr VWi Vr Vi lr li] in the preconditioner's precision;
// cell_data: per cell (v0, v1, v2, 1/|K|) in the same precision
cudaError_t launch_fdm(int n, int precision, const FdmArgs &a, const void *tables, const void *cell_data,
                       cudaStream_t s);
cudaError_t launch_mass(int n, const MassArgs &a, cudaStream_t s);
int         vec_partial_blocks(long long n);
// out[i] = V_i . w for i < m (V_i = V + i * ld), partials: vec_partial_blocks(n) * m doubles
cudaError_t launch_multi_dot(const double *V, long long ld, int m, const double *w, long long n, double *partials,
                             double *out, cudaStream_t s);
// w += sign * sum_i coef[i] V_i (coef on the device, m <= 64)
cudaError_t launch_multi_axpy(double *w, const double *V, long long ld, int m, const double *coef, double sign,
                              long long n, cudaStream_t s);
cudaError_t launch_lincomb(double *dst, double a, const double *x, double b, const double *y, long long n,
                           cudaStream_t s);
// dst = JxW (a x + b y) at the Gauss points of every cell (y may be null): the
// mass matrix on the Gauss-point basis, diagonal; cell_geo holds idet = 1 /
// det J per point (field case) or is null for a uniform mesh of cell volume vol
cudaError_t launch_gauss_mass_lincomb(int n, double *dst, double a, const double *x, double b, const double *y,
                                      long long n_cells, const double *cell_geo, double vol, cudaStream_t s);
} // namespace adv
