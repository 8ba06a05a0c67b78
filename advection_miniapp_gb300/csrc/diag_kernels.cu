// Set-up and diagnostics kernels: L2 projection of the initial data
// (project_initial, advection_solver.cc:760-784), mass/energy/H1 seminorm
// (compute_mass_and_energy, advection_solver.cc:787-818), the L2 error
// against the analytic solution (output_results, advection_solver.cc:1183-1208)
// and an FMA throughput probe for roofline denominators.
//
// FP64, one CTA per cell at a time (grid-stride), every evaluation by sum
// factorization: 1D matrices applied direction by direction in shared memory,
// one thread per output entry.  The curved mapping is evaluated from its
// support points (the analytic deformation at the Gauss-Lobatto nodes), so
// no geometry is stored for the diagnostics.  Reductions are deterministic:
// per-CTA partials, summed by the caller.
#include "kernels.h"

namespace adv
{
namespace
{
constexpr int kDiagThreads = 128;
constexpr int kMaxP        = 8; // points per direction (error quadrature: n + 1 <= 8)
constexpr int kMaxP3       = kMaxP * kMaxP * kMaxP;
constexpr int kMaxN3       = 343;

__device__ __forceinline__ void cell_origin(const DiagArgs &g, long long c, double lo[3])
{
  const int ix = (int)(c % g.nc[0]), iy = (int)((c / g.nc[0]) % g.nc[1]),
            iz = (int)(c / ((long long)g.nc[0] * g.nc[1])) + g.zoff;
  lo[0] = g.lo[0] + ix * g.h[0];
  lo[1] = g.lo[1] + iy * g.h[1];
  lo[2] = g.lo[2] + iz * g.h[2];
}

// out = A applied along direction d of `in` (dims d0 x d1 x d2, first fastest);
// A is mo x ni row-major (A[q * ni + k]); the output has mo entries along d.
// Ends with a barrier.
__device__ void tsweep(const double *A, int mo, int ni, int d, int d0, int d1, int d2, const double *in,
                       double *out)
{
  const int o0 = d == 0 ? mo : d0, o1 = d == 1 ? mo : d1, o2 = d == 2 ? mo : d2;
  const int total = o0 * o1 * o2;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x)
    {
      const int i0 = idx % o0, i1 = (idx / o0) % o1, i2 = idx / (o0 * o1);
      const int q  = d == 0 ? i0 : d == 1 ? i1 : i2;
      const int st = d == 0 ? 1 : d == 1 ? d0 : d0 * d1;
      const int b  = (d == 0 ? 0 : i0) + d0 * ((d == 1 ? 0 : i1) + d1 * (d == 2 ? 0 : i2));
      double    s  = 0.0;
      for (int k = 0; k < ni; ++k)
        s += A[q * ni + k] * in[b + k * st];
      out[idx] = s;
    }
  __syncthreads();
}

// K sweeps with the same shape at once (one barrier): outs[k] = As[k]
// applied along d of ins[k]
template <int K>
__device__ void tsweep_n(const double *const (&As)[K], const double *const (&ins)[K], double *const (&outs)[K],
                         int mo, int ni, int d, int d0, int d1, int d2)
{
  const int o0 = d == 0 ? mo : d0, o1 = d == 1 ? mo : d1, o2 = d == 2 ? mo : d2;
  const int total = o0 * o1 * o2;
  const int st    = d == 0 ? 1 : d == 1 ? d0 : d0 * d1;
  for (int idx = threadIdx.x; idx < K * total; idx += blockDim.x)
    {
      const int kk = idx / total, r = idx % total;
      const int i0 = r % o0, i1 = (r / o0) % o1, i2 = r / (o0 * o1);
      const int q  = d == 0 ? i0 : d == 1 ? i1 : i2;
      const int b  = (d == 0 ? 0 : i0) + d0 * ((d == 1 ? 0 : i1) + d1 * (d == 2 ? 0 : i2));
      const double *A = As[kk], *in = ins[kk];
      double        s = 0.0;
      for (int k = 0; k < ni; ++k)
        s = fma(A[q * ni + k], in[b + k * st], s);
      outs[kk][r] = s;
    }
  __syncthreads();
}

// support points of a curved cell, the three components X[c * n^3 + i]; each
// sine of the deformation depends on one coordinate, so the 3n values
// sin(2 pi s_d) at the nodes along each direction (sn) serve all n^3 points
// (the same arithmetic as deform_dev)
__device__ void support_points(const DiagArgs &g, const double lo[3], double *X, double *sn)
{
  const int n = g.n, nq = n * n * n;
  for (int i = threadIdx.x; i < 3 * n; i += blockDim.x)
    {
      const int    d = i / n, a = i % n;
      const double x = lo[d] + g.h[d] * g.gl[a];
      sn[i]          = sinpi(2.0 * ((x - g.lo[d]) / g.L[d]));
    }
  __syncthreads();
  for (int i = threadIdx.x; i < nq; i += blockDim.x)
    {
      const int a[3] = {i % n, (i / n) % n, i / (n * n)};
#pragma unroll
      for (int c = 0; c < 3; ++c)
        {
          const int    c1 = (c + 1) % 3, c2 = (c + 2) % 3;
          const double p  = lo[c] + g.h[c] * g.gl[a[c]];
          X[c * nq + i]   = p + g.deformation * g.L[c] * sn[c1 * n + a[c1]] * sn[c2 * n + a[c2]];
        }
    }
  __syncthreads();
}

struct Scratch
{
  double *X, *A, *Az, *B, *By, *Bz, *sn;
};

// position x[c][p] and Jacobian J[3c + j][p] at the m^3 points of the 1D rule
// with nodal-basis values V and derivatives W (m x n), from the support
// points in s.X; curved cells only
__device__ void map_points(const DiagArgs &g, int m, const double *V, const double *W, double *x, double *J,
                           const Scratch &s)
{
  const int n = g.n, m3 = m * m * m, nq = n * n * n;
  for (int c = 0; c < 3; ++c)
    {
      const double *X = s.X + c * nq;
      tsweep_n<2>({V, W}, {X, X}, {s.A, s.Az}, m, n, 2, n, n, n);
      tsweep_n<3>({V, W, V}, {s.A, s.A, s.Az}, {s.B, s.By, s.Bz}, m, n, 1, n, n, m);
      tsweep_n<4>({V, W, V, V}, {s.B, s.B, s.By, s.Bz},
                  {x + c * m3, J + (3 * c + 0) * m3, J + (3 * c + 1) * m3, J + (3 * c + 2) * m3}, m, n, 0, n, m,
                  m);
    }
}

// J at point p from the component arrays, or the affine Jacobian
__device__ void jacobian_at(const DiagArgs &g, const double *J, int m3, int p, double Jp[9])
{
  if (!g.curved)
    {
      for (int i = 0; i < 9; ++i)
        Jp[i] = 0.0;
      Jp[0] = g.h[0], Jp[4] = g.h[1], Jp[8] = g.h[2];
      return;
    }
  for (int i = 0; i < 9; ++i)
    Jp[i] = J[i * m3 + p];
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

__device__ void point_position(const DiagArgs &g, const double lo[3], const double *pts, int m, int p,
                               const double *x, double xp[3])
{
  if (g.curved)
    {
      const int m3 = m * m * m;
      xp[0] = x[p], xp[1] = x[m3 + p], xp[2] = x[2 * m3 + p];
      return;
    }
  const int i0 = p % m, i1 = (p / m) % m, i2 = p / (m * m);
  xp[0] = lo[0] + g.h[0] * pts[i0];
  xp[1] = lo[1] + g.h[1] * pts[i1];
  xp[2] = lo[2] + g.h[2] * pts[i2];
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

// shared-memory layout (doubles) for n points per direction and P = n + 1
// (the most points of any rule used): X[3][n^3], A, Az [n n P], B, By, Bz
// [n P P], x[3][P^3], J[9][P^3], U[n^3], T1, T2, T3 [P^3], sn[3n]
__host__ __device__ inline int diag_smem_doubles(int n)
{
  const int P = n + 1, P3 = P * P * P, N3 = n * n * n;
  return 3 * N3 + 2 * n * n * P + 3 * n * P * P + 12 * P3 + N3 + 3 * P3 + 3 * n;
}
constexpr int kSmemDoubles = 3 * kMaxN3 + 2 * 7 * 7 * kMaxP + 3 * 7 * kMaxP * kMaxP + 12 * kMaxP3 + kMaxN3 +
                             3 * kMaxP3 + 3 * 7;

struct Layout
{
  Scratch s;
  double *x, *J, *U, *T1, *T2, *T3;
  __device__ Layout(double *base, int n)
  {
    const int P = n + 1, P3 = P * P * P, N3 = n * n * n;
    s.X  = base;
    s.A  = s.X + 3 * N3;
    s.Az = s.A + n * n * P;
    s.B  = s.Az + n * n * P;
    s.By = s.B + n * P * P;
    s.Bz = s.By + n * P * P;
    x    = s.Bz + n * P * P;
    J    = x + 3 * P3;
    U    = J + 9 * P3;
    T1   = U + N3;
    T2   = T1 + P3;
    T3   = T2 + P3;
    s.sn = T3 + P3;
  }
};

__global__ void __launch_bounds__(kDiagThreads) project_kernel(const DiagArgs g, double t, double *dst)
{
  extern __shared__ __align__(16) double smem[];
  Layout    L(smem, g.n);
  const int n = g.n, nq = n * n * n;
  for (long long c = g.cell_begin + blockIdx.x; c < g.n_cells; c += gridDim.x)
    {
      double lo[3];
      cell_origin(g, c, lo);
      if (g.curved)
        {
          support_points(g, lo, L.s.X, L.s.sn);
          map_points(g, n, g.S, g.Sd, L.x, L.J, L.s);
        }
      for (int q = threadIdx.x; q < nq; q += blockDim.x)
        {
          double xp[3];
          point_position(g, lo, g.gp, n, q, L.x, xp);
          L.T1[q] = exact_value(g.ex, xp[0], xp[1], xp[2], t);
        }
      __syncthreads();
      // transform_from_q_points_to_basis: S^{-1} in every direction
      tsweep(g.Si, n, n, 0, n, n, n, L.T1, L.T2);
      tsweep(g.Si, n, n, 1, n, n, n, L.T2, L.T3);
      tsweep(g.Si, n, n, 2, n, n, n, L.T3, L.T1);
      for (int i = threadIdx.x; i < nq; i += blockDim.x)
        dst[c * nq + i] = L.T1[i];
      __syncthreads();
    }
}

__global__ void __launch_bounds__(kDiagThreads)
  mass_energy_kernel(const DiagArgs g, const double *u, double *partials)
{
  extern __shared__ __align__(16) double smem[];
  Layout    L(smem, g.n);
  const int n = g.n, nq = n * n * n;
  double    m = 0.0, e = 0.0, hs = 0.0;
  double   *G[3] = {L.s.A, L.s.B, L.s.By}; // reuse scratch for the three gradients
  for (long long c = g.cell_begin + blockIdx.x; c < g.n_cells; c += gridDim.x)
    {
      double lo[3];
      cell_origin(g, c, lo);
      if (g.curved)
        {
          support_points(g, lo, L.s.X, L.s.sn);
          map_points(g, n, g.S, g.Sd, L.x, L.J, L.s);
        }
      for (int i = threadIdx.x; i < nq; i += blockDim.x)
        L.U[i] = u[c * nq + i];
      __syncthreads();
      tsweep(g.S, n, n, 0, n, n, n, L.U, L.T1);
      tsweep(g.S, n, n, 1, n, n, n, L.T1, L.T2);
      tsweep(g.S, n, n, 2, n, n, n, L.T2, L.T3); // values at the Gauss points
      for (int d = 0; d < 3; ++d)
        tsweep(g.Dc, n, n, d, n, n, n, L.T3, G[d]);
      for (int q = threadIdx.x; q < nq; q += blockDim.x)
        {
          double Jp[9], Ji[9];
          jacobian_at(g, L.J, nq, q, Jp);
          const double det = det_inv3(Jp, Ji);
          const int    q0 = q % n, q1 = (q / n) % n, q2 = q / (n * n);
          const double JxW = det * g.gw[q0] * g.gw[q1] * g.gw[q2];
          const double v   = L.T3[q];
          double       gg  = 0.0;
          for (int i = 0; i < 3; ++i)
            {
              const double gi = Ji[0 * 3 + i] * G[0][q] + Ji[1 * 3 + i] * G[1][q] + Ji[2 * 3 + i] * G[2][q];
              gg += gi * gi;
            }
          m += v * JxW;
          e += v * v * JxW;
          hs += gg * JxW;
        }
      __syncthreads();
    }
  block_reduce3(m, e, hs, partials + 3 * blockIdx.x);
}

__global__ void __launch_bounds__(kDiagThreads)
  l2_error_kernel(const DiagArgs g, const double *u, double t, double *partials)
{
  extern __shared__ __align__(16) double smem[];
  Layout    L(smem, g.n);
  const int n = g.n, nq = n * n * n, m = n + 1, m3 = m * m * m;
  double    err = 0.0, nrm = 0.0;
  for (long long c = g.cell_begin + blockIdx.x; c < g.n_cells; c += gridDim.x)
    {
      double lo[3];
      cell_origin(g, c, lo);
      for (int i = threadIdx.x; i < nq; i += blockDim.x)
        L.U[i] = u[c * nq + i];
      __syncthreads();
      // u_h at the QGauss(k+2) points
      tsweep(g.SE, m, n, 0, n, n, n, L.U, L.T1);
      tsweep(g.SE, m, n, 1, m, n, n, L.T1, L.T2);
      tsweep(g.SE, m, n, 2, m, m, n, L.T2, L.T3);
      if (g.curved)
        {
          support_points(g, lo, L.s.X, L.s.sn);
          map_points(g, m, g.SE, g.SEd, L.x, L.J, L.s);
        }
      for (int p = threadIdx.x; p < m3; p += blockDim.x)
        {
          double xp[3], Jp[9], Ji[9];
          point_position(g, lo, g.ep, m, p, L.x, xp);
          jacobian_at(g, L.J, m3, p, Jp);
          const double det = det_inv3(Jp, Ji);
          const int    p0 = p % m, p1 = (p / m) % m, p2 = p / (m * m);
          const double d   = L.T3[p] - exact_value(g.ex, xp[0], xp[1], xp[2], t);
          err += d * d * det * g.ew[p0] * g.ew[p1] * g.ew[p2];
        }
      __syncthreads();
      // norm of the exact solution with QGauss(k+1) (same support points)
      if (g.curved)
        map_points(g, n, g.S, g.Sd, L.x, L.J, L.s);
      for (int q = threadIdx.x; q < nq; q += blockDim.x)
        {
          double xp[3], Jp[9], Ji[9];
          point_position(g, lo, g.gp, n, q, L.x, xp);
          jacobian_at(g, L.J, nq, q, Jp);
          const double det = det_inv3(Jp, Ji);
          const int    q0 = q % n, q1 = (q / n) % n, q2 = q / (n * n);
          const double ue  = exact_value(g.ex, xp[0], xp[1], xp[2], t);
          nrm += ue * ue * det * g.gw[q0] * g.gw[q1] * g.gw[q2];
        }
      __syncthreads();
    }
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

// FP64 with the stage kernel's mix of FP64 instructions: per iteration 14
// independent chains, 7 FMA, 4 MUL and 3 ADD (the collocation stage with
// upwind traces issues about 51 % FMA, 28 % MUL and 21 % ADD)
constexpr int kMixF = 7, kMixM = 4, kMixA = 3;
__global__ void fp64_mix_kernel(double *out, int iters, double a, double b)
{
  double f[kMixF], m[kMixM], d[kMixA];
#pragma unroll
  for (int i = 0; i < kMixF; ++i)
    f[i] = threadIdx.x + i;
#pragma unroll
  for (int i = 0; i < kMixM; ++i)
    m[i] = threadIdx.x + kMixF + i;
#pragma unroll
  for (int i = 0; i < kMixA; ++i)
    d[i] = threadIdx.x + kMixF + kMixM + i;
  for (int it = 0; it < iters; ++it)
    {
#pragma unroll
      for (int i = 0; i < kMixF; ++i)
        f[i] = fma(f[i], a, b);
#pragma unroll
      for (int i = 0; i < kMixM; ++i)
        m[i] = m[i] * a;
#pragma unroll
      for (int i = 0; i < kMixA; ++i)
        d[i] = d[i] + b;
    }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kMixF; ++i)
    s += f[i];
#pragma unroll
  for (int i = 0; i < kMixM; ++i)
    s += m[i];
#pragma unroll
  for (int i = 0; i < kMixA; ++i)
    s += d[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

constexpr size_t kSmemBytes = kSmemDoubles * sizeof(double);

template <typename K>
cudaError_t opt_in(K kernel)
{
  static std::atomic<unsigned long long> configured{0};
  return opt_in_smem(kernel, (int)kSmemBytes, configured);
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
  if (cudaError_t e = opt_in(project_kernel))
    return e;
  project_kernel<<<diag_max_blocks(g.n_cells - g.cell_begin), kDiagThreads,
                   diag_smem_doubles(g.n) * sizeof(double), s>>>(g, t, dst);
  return cudaGetLastError();
}

cudaError_t launch_mass_energy(const DiagArgs &g, const double *u, double *partials, int *n_blocks,
                               cudaStream_t s)
{
  if (cudaError_t e = opt_in(mass_energy_kernel))
    return e;
  *n_blocks = diag_max_blocks(g.n_cells - g.cell_begin);
  mass_energy_kernel<<<*n_blocks, kDiagThreads, diag_smem_doubles(g.n) * sizeof(double), s>>>(g, u, partials);
  return cudaGetLastError();
}

cudaError_t launch_l2_error(const DiagArgs &g, const double *u, double t, double *partials,
                            int *n_blocks, cudaStream_t s)
{
  if (cudaError_t e = opt_in(l2_error_kernel))
    return e;
  *n_blocks = diag_max_blocks(g.n_cells - g.cell_begin);
  l2_error_kernel<<<*n_blocks, kDiagThreads, diag_smem_doubles(g.n) * sizeof(double), s>>>(g, u, t, partials);
  return cudaGetLastError();
}

// out must hold blocks * 256 values of the precision's type
int fma_peak_chains(int precision)
{
  return precision == 2 ? kMixF + kMixM + kMixA : 8;
}

cudaError_t launch_fma_peak(int precision, double *out, int iters, int blocks, cudaStream_t s)
{
  if (precision == 2)
    fp64_mix_kernel<<<blocks, 256, 0, s>>>(out, iters, 1.0000001, 1e-9);
  else if (precision == 0)
    fma_peak_kernel<double><<<blocks, 256, 0, s>>>(out, iters, 1.0000001, 1e-9);
  else
    fma_peak_kernel<float><<<blocks, 256, 0, s>>>(reinterpret_cast<float *>(out), iters, 1.0000001f,
                                                   1e-9f);
  return cudaGetLastError();
}
} // namespace adv
