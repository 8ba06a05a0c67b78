// Set-up and diagnostics kernels: L2 projection of the initial data
// (project_initial, advection_solver.cc:760-784), mass/energy/H1 seminorm
// (compute_mass_and_energy, advection_solver.cc:787-818), the L2 error
// against the analytic solution (output_results, advection_solver.cc:1183-1208)
// and an FMA throughput probe for roofline denominators.  These run once per
// output, not per stage; they favour simplicity (direct sums per point, one
// CTA per cell) over speed.
#include "kernels.h"

namespace adv
{
namespace
{
constexpr int kDiagThreads = 128;
constexpr int kMaxNQ       = 343; // 7^3

__device__ __forceinline__ void cell_origin(const DiagArgs &g, long long c, double lo[3])
{
  const int ix = (int)(c % g.nc[0]), iy = (int)((c / g.nc[0]) % g.nc[1]),
            iz = (int)(c / ((long long)g.nc[0] * g.nc[1]));
  lo[0] = g.lo[0] + ix * g.h[0];
  lo[1] = g.lo[1] + iy * g.h[1];
  lo[2] = g.lo[2] + iz * g.h[2];
}

// support points of the curved mapping into X (3 per node)
__device__ void load_support_points(const DiagArgs &g, const double lo[3], double *X)
{
  const int n = g.n, nq = n * n * n;
  for (int i = threadIdx.x; i < nq; i += blockDim.x)
    {
      const int    a = i % n, b = (i / n) % n, c = i / (n * n);
      const double p[3] = {lo[0] + g.h[0] * g.gl[a], lo[1] + g.h[1] * g.gl[b], lo[2] + g.h[2] * g.gl[c]};
      deform_dev(g.deformation, g.lo, g.L, p, X + 3 * i);
    }
}

// position and Jacobian at a reference point given 1D basis values V[d][a]
// and derivatives W[d][a] (curved: sums over the support points)
__device__ void map_at(const DiagArgs &g, const double lo[3], const double *X, const double *V0,
                       const double *V1, const double *V2, const double *W0, const double *W1,
                       const double *W2, const double xi[3], double x[3], double J[9])
{
  const int n = g.n;
  if (!g.curved)
    {
      for (int d = 0; d < 3; ++d)
        x[d] = lo[d] + g.h[d] * xi[d];
      for (int i = 0; i < 9; ++i)
        J[i] = 0.0;
      J[0] = g.h[0], J[4] = g.h[1], J[8] = g.h[2];
      return;
    }
  for (int d = 0; d < 3; ++d)
    x[d] = 0.0;
  for (int i = 0; i < 9; ++i)
    J[i] = 0.0;
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a)
        {
          const double *y  = X + 3 * (a + n * (b + n * c));
          const double  w  = V0[a] * V1[b] * V2[c];
          const double  w0 = W0[a] * V1[b] * V2[c];
          const double  w1 = V0[a] * W1[b] * V2[c];
          const double  w2 = V0[a] * V1[b] * W2[c];
          for (int d = 0; d < 3; ++d)
            {
              x[d] += w * y[d];
              J[3 * d + 0] += w0 * y[d];
              J[3 * d + 1] += w1 * y[d];
              J[3 * d + 2] += w2 * y[d];
            }
        }
}

__device__ double det_inv3(const double *J, double *Ji)
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

// in-place 1D sweep along direction d of an n^3 shared array with matrix M[q*n+i]
__device__ void sweep_smem(int n, const double *M, double *a, int d)
{
  const int stride = d == 0 ? 1 : d == 1 ? n : n * n;
  for (int w = threadIdx.x; w < n * n; w += blockDim.x)
    {
      const int r    = w % n, s = w / n;
      const int base = d == 0 ? n * (r + n * s) : d == 1 ? r + n * n * s : r + n * s;
      double    in[kMaxNDev];
      for (int i = 0; i < n; ++i)
        in[i] = a[base + i * stride];
      for (int q = 0; q < n; ++q)
        {
          double s2 = 0.0;
          for (int i = 0; i < n; ++i)
            s2 += M[q * n + i] * in[i];
          a[base + q * stride] = s2;
        }
    }
  __syncthreads();
}

__device__ void block_reduce3(double v0, double v1, double v2, double *out)
{
  __shared__ double red[3][kDiagThreads / 32];
  for (int o = 16; o > 0; o >>= 1)
    {
      v0 += __shfl_down_sync(0xffffffffu, v0, o);
      v1 += __shfl_down_sync(0xffffffffu, v1, o);
      v2 += __shfl_down_sync(0xffffffffu, v2, o);
    }
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0)
    red[0][warp] = v0, red[1][warp] = v1, red[2][warp] = v2;
  __syncthreads();
  if (threadIdx.x == 0)
    {
      double s0 = 0, s1 = 0, s2 = 0;
      for (int w = 0; w < kDiagThreads / 32; ++w)
        s0 += red[0][w], s1 += red[1][w], s2 += red[2][w];
      out[0] = s0, out[1] = s1, out[2] = s2;
    }
}

__global__ void __launch_bounds__(kDiagThreads) project_kernel(const DiagArgs g, double t, double *dst)
{
  __shared__ double X[3 * kMaxNQ];
  __shared__ double V[kMaxNQ];
  __shared__ double S[kMaxNDev * kMaxNDev], Si[kMaxNDev * kMaxNDev];
  const int n = g.n, nq = n * n * n;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x)
    S[i] = g.S[i], Si[i] = g.Si[i];
  for (long long c = blockIdx.x; c < g.n_cells; c += gridDim.x)
    {
      double lo[3];
      cell_origin(g, c, lo);
      __syncthreads();
      if (g.curved)
        load_support_points(g, lo, X);
      __syncthreads();
      for (int q = threadIdx.x; q < nq; q += blockDim.x)
        {
          const int    q0 = q % n, q1 = (q / n) % n, q2 = q / (n * n);
          const double xi[3] = {g.gp[q0], g.gp[q1], g.gp[q2]};
          double       x[3], J[9];
          map_at(g, lo, X, S + q0 * n, S + q1 * n, S + q2 * n, S, S, S, xi, x, J);
          V[q] = exact_value(g.ex, x[0], x[1], x[2], t);
        }
      __syncthreads();
      sweep_smem(n, Si, V, 0);
      sweep_smem(n, Si, V, 1);
      sweep_smem(n, Si, V, 2);
      for (int i = threadIdx.x; i < nq; i += blockDim.x)
        dst[c * nq + i] = V[i];
    }
}

__global__ void __launch_bounds__(kDiagThreads)
  mass_energy_kernel(const DiagArgs g, const double *u, double *partials)
{
  __shared__ double X[3 * kMaxNQ];
  __shared__ double U[kMaxNQ];
  __shared__ double S[kMaxNDev * kMaxNDev], Sd[kMaxNDev * kMaxNDev];
  const int n = g.n, nq = n * n * n;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x)
    S[i] = g.S[i], Sd[i] = g.Sd[i];
  double m = 0.0, e = 0.0, hs = 0.0;
  for (long long c = blockIdx.x; c < g.n_cells; c += gridDim.x)
    {
      double lo[3];
      cell_origin(g, c, lo);
      __syncthreads();
      if (g.curved)
        load_support_points(g, lo, X);
      for (int i = threadIdx.x; i < nq; i += blockDim.x)
        U[i] = u[c * nq + i];
      __syncthreads();
      for (int q = threadIdx.x; q < nq; q += blockDim.x)
        {
          const int    q0 = q % n, q1 = (q / n) % n, q2 = q / (n * n);
          const double xi[3] = {g.gp[q0], g.gp[q1], g.gp[q2]};
          double       x[3], J[9], Ji[9];
          map_at(g, lo, X, S + q0 * n, S + q1 * n, S + q2 * n, Sd + q0 * n, Sd + q1 * n,
                 Sd + q2 * n, xi, x, J);
          const double det = det_inv3(J, Ji);
          double       v = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
          for (int cc = 0; cc < n; ++cc)
            for (int b = 0; b < n; ++b)
              for (int a = 0; a < n; ++a)
                {
                  const double ua = U[a + n * (b + n * cc)];
                  v += S[q0 * n + a] * S[q1 * n + b] * S[q2 * n + cc] * ua;
                  g0 += Sd[q0 * n + a] * S[q1 * n + b] * S[q2 * n + cc] * ua;
                  g1 += S[q0 * n + a] * Sd[q1 * n + b] * S[q2 * n + cc] * ua;
                  g2 += S[q0 * n + a] * S[q1 * n + b] * Sd[q2 * n + cc] * ua;
                }
          const double JxW = det * g.gw[q0] * g.gw[q1] * g.gw[q2];
          double       gg  = 0.0;
          for (int i = 0; i < 3; ++i)
            {
              const double gi = Ji[0 * 3 + i] * g0 + Ji[1 * 3 + i] * g1 + Ji[2 * 3 + i] * g2;
              gg += gi * gi;
            }
          m += v * JxW;
          e += v * v * JxW;
          hs += gg * JxW;
        }
    }
  __syncthreads();
  block_reduce3(m, e, hs, partials + 3 * blockIdx.x);
}

__global__ void __launch_bounds__(kDiagThreads)
  l2_error_kernel(const DiagArgs g, const double *u, double t, double *partials)
{
  __shared__ double X[3 * kMaxNQ];
  __shared__ double U[kMaxNQ];
  __shared__ double S[kMaxNDev * kMaxNDev], Sd[kMaxNDev * kMaxNDev];
  __shared__ double SE[8 * kMaxNDev], SEd[8 * kMaxNDev];
  const int n = g.n, nq = n * n * n, m = n + 1, meq = m * m * m;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x)
    S[i] = g.S[i], Sd[i] = g.Sd[i];
  for (int i = threadIdx.x; i < m * n; i += blockDim.x)
    SE[i] = g.SE[i], SEd[i] = g.SEd[i];
  double err = 0.0, nrm = 0.0;
  for (long long c = blockIdx.x; c < g.n_cells; c += gridDim.x)
    {
      double lo[3];
      cell_origin(g, c, lo);
      __syncthreads();
      if (g.curved)
        load_support_points(g, lo, X);
      for (int i = threadIdx.x; i < nq; i += blockDim.x)
        U[i] = u[c * nq + i];
      __syncthreads();
      for (int p = threadIdx.x; p < meq; p += blockDim.x)
        {
          const int    p0 = p % m, p1 = (p / m) % m, p2 = p / (m * m);
          const double xi[3] = {g.ep[p0], g.ep[p1], g.ep[p2]};
          double       x[3], J[9], Ji[9];
          map_at(g, lo, X, SE + p0 * n, SE + p1 * n, SE + p2 * n, SEd + p0 * n, SEd + p1 * n,
                 SEd + p2 * n, xi, x, J);
          const double det = det_inv3(J, Ji);
          double       uh  = 0.0;
          for (int cc = 0; cc < n; ++cc)
            for (int b = 0; b < n; ++b)
              {
                const double w = SE[p1 * n + b] * SE[p2 * n + cc];
                for (int a = 0; a < n; ++a)
                  uh += w * SE[p0 * n + a] * U[a + n * (b + n * cc)];
              }
          const double d = uh - exact_value(g.ex, x[0], x[1], x[2], t);
          err += d * d * det * g.ew[p0] * g.ew[p1] * g.ew[p2];
        }
      for (int q = threadIdx.x; q < nq; q += blockDim.x)
        {
          const int    q0 = q % n, q1 = (q / n) % n, q2 = q / (n * n);
          const double xi[3] = {g.gp[q0], g.gp[q1], g.gp[q2]};
          double       x[3], J[9], Ji[9];
          map_at(g, lo, X, S + q0 * n, S + q1 * n, S + q2 * n, Sd + q0 * n, Sd + q1 * n,
                 Sd + q2 * n, xi, x, J);
          const double det = det_inv3(J, Ji);
          const double ue  = exact_value(g.ex, x[0], x[1], x[2], t);
          nrm += ue * ue * det * g.gw[q0] * g.gw[q1] * g.gw[q2];
        }
    }
  __syncthreads();
  block_reduce3(err, nrm, 0.0, partials + 3 * blockIdx.x);
}

template <typename T>
__global__ void fma_peak_kernel(T *out, int iters, T a, T b)
{
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
    x7 = x0 + 7;
  for (int i = 0; i < iters; ++i)
    {
      x0 = fma(x0, a, b), x1 = fma(x1, a, b), x2 = fma(x2, a, b), x3 = fma(x3, a, b);
      x4 = fma(x4, a, b), x5 = fma(x5, a, b), x6 = fma(x6, a, b), x7 = fma(x7, a, b);
    }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
} // namespace

cudaError_t upload_tables_diag(const DevTables<double> *d, const DevTables<float> *f)
{
  return upload_tables_local(d, f);
}

int diag_max_blocks(long long n_cells)
{
  return (int)(n_cells < 4096 ? n_cells : 4096);
}

cudaError_t launch_project(const DiagArgs &g, double t, double *dst, cudaStream_t s)
{
  project_kernel<<<diag_max_blocks(g.n_cells), kDiagThreads, 0, s>>>(g, t, dst);
  return cudaGetLastError();
}

cudaError_t launch_mass_energy(const DiagArgs &g, const double *u, double *partials, int *n_blocks,
                               cudaStream_t s)
{
  *n_blocks = diag_max_blocks(g.n_cells);
  mass_energy_kernel<<<*n_blocks, kDiagThreads, 0, s>>>(g, u, partials);
  return cudaGetLastError();
}

cudaError_t launch_l2_error(const DiagArgs &g, const double *u, double t, double *partials,
                            int *n_blocks, cudaStream_t s)
{
  *n_blocks = diag_max_blocks(g.n_cells);
  l2_error_kernel<<<*n_blocks, kDiagThreads, 0, s>>>(g, u, t, partials);
  return cudaGetLastError();
}

// out must hold blocks * 256 values of the precision's type
cudaError_t launch_fma_peak(int precision, double *out, int iters, int blocks, cudaStream_t s)
{
  if (precision == 0)
    fma_peak_kernel<double><<<blocks, 256, 0, s>>>(out, iters, 1.0000001, 1e-9);
  else
    fma_peak_kernel<float><<<blocks, 256, 0, s>>>(reinterpret_cast<float *>(out), iters, 1.0000001f,
                                                   1e-9f);
  return cudaGetLastError();
}
} // namespace adv
