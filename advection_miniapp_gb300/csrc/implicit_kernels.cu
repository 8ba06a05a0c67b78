// Kernels of the implicit solver: the cellwise mass matrix, the block-Jacobi
// fast-diagonalization (FDM) preconditioner and the FP64 vector kernels of
// FGMRES.  The implicit operator itself (M/dt + A) is a mode of the fused
// stage kernel.
//
// FDM (CellwisePreconditionerFDM, advection_solver_implicit.cc:490-646, inside
// precondition_block_jacobi, :1283-1340): per cell, the residual is moved to
// the collocation basis on the Gauss points (S^{-T}), V^{-1}W^{-1} is applied
// in every direction, each point is scaled by
//   (1/|K|) / (c + s sum_d v_d lambda_d(i_d))
// (v = cell average of J^{-1} a, s the velocity time factor, tables of the
// sign of s v_d), V is applied in every direction and the real part is moved
// back to the nodal basis (S^{-1}).  Complex sweeps run in the
// preconditioner's precision (FP32 by default) in shared memory.
#include "implicit_kernels.h"

#include <algorithm>

namespace adv
{
namespace
{
template <int N>
struct FdmShape
{
  static constexpr int C       = N == 2 ? 32 : N == 3 ? 14 : N == 4 ? 8 : N == 5 ? 5 : N == 6 ? 7 : 5;
  static constexpr int NQ      = N * N * N;
  static constexpr int NF      = N * N;
  static constexpr int THREADS = ((C * NF + 31) / 32) * 32;
};

template <int N, typename T>
__device__ __forceinline__ void rsweep(const T (&M)[kMaxNDev][kMaxNDev], const T (&in)[N], T (&out)[N])
{
#pragma unroll
  for (int q = 0; q < N; ++q)
    {
      T s = M[q][0] * in[0];
#pragma unroll
      for (int i = 1; i < N; ++i)
        s = fma(M[q][i], in[i], s);
      out[q] = s;
    }
}

// complex matrix (Mr + i Mi) times complex vector (xr + i xi)
template <int N, typename T>
__device__ __forceinline__ void csweep(const T *Mr, const T *Mi, const T (&xr)[N], const T (&xi)[N], T (&yr)[N],
                                       T (&yi)[N])
{
#pragma unroll
  for (int q = 0; q < N; ++q)
    {
      T sr = T(0), si = T(0);
#pragma unroll
      for (int k = 0; k < N; ++k)
        {
          const T mr = Mr[q * N + k], mi = Mi[q * N + k];
          sr         = fma(mr, xr[k], fma(-mi, xi[k], sr));
          si         = fma(mr, xi[k], fma(mi, xr[k], si));
        }
      yr[q] = sr, yi[q] = si;
    }
}

// GAUSS: the residual and the result are on the Gauss-point basis (the
// residual as dual coefficients, the result as values at the points): the
// transforms S^{-T} on entry and S^{-1} on exit drop out.
template <int N, typename T, bool GAUSS>
__global__ void __launch_bounds__(FdmShape<N>::THREADS)
  fdm_kernel(const FdmArgs A, const T *__restrict__ tables, const T *__restrict__ cell_data)
{
  using SH         = FdmShape<N>;
  constexpr int C  = SH::C, NQ = SH::NQ, NF = SH::NF, NT = SH::THREADS;
  constexpr int TB = 2 * (2 * N * N + 2 * N * N + 2 * N); // [sign][VWr VWi Vr Vi lr li]
  __shared__ T    tab_s[TB];
  __shared__ T    R[C * NQ], Xi[C * NQ];
  __shared__ T    cinfo[C * 4];
  __shared__ int  sgn[C * 3];
  const DevTables<T> &tb    = tab<T>(N);
  const int           tid   = threadIdx.x;
  const long long     cell0 = (long long)blockIdx.x * C;
  const int           ncell = (int)min((long long)C, A.n_cells - cell0);
  for (int i = tid; i < TB; i += NT)
    tab_s[i] = tables[i];
  for (int i = tid; i < ncell * 4; i += NT)
    cinfo[i] = cell_data[cell0 * 4 + i];
  __syncthreads();
  for (int i = tid; i < ncell * 3; i += NT)
    sgn[i] = (T(A.time_factor) * cinfo[(i / 3) * 4 + i % 3] < T(0)) ? 1 : 0;
  auto VWr = [&](int s) { return tab_s + s * (TB / 2); };
  auto VWi = [&](int s) { return tab_s + s * (TB / 2) + N * N; };
  auto Vr  = [&](int s) { return tab_s + s * (TB / 2) + 2 * N * N; };
  auto Vi  = [&](int s) { return tab_s + s * (TB / 2) + 3 * N * N; };
  auto Lr  = [&](int s) { return tab_s + s * (TB / 2) + 4 * N * N; };
  auto Li  = [&](int s) { return tab_s + s * (TB / 2) + 4 * N * N + N; };

  // phase 1: residual as z-pencils, S^{-T} along z
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int     cl = w / NF, r = w % NF;
      const double *g  = A.src + (cell0 + cl) * NQ + r;
      T             in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = (T)__ldg(g + k * NF);
      if (GAUSS)
        for (int k = 0; k < N; ++k)
          out[k] = in[k];
      else
        rsweep<N, T>(tb.SiT, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        R[cl * NQ + r + k * NF] = out[k];
    }
  __syncthreads();
  // phase 2: S^{-T} along y
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int r = w % NF;
      T        *p = R + (w / NF) * NQ + (r % N) + NF * (r / N);
      T         in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * N];
      if (GAUSS)
        for (int k = 0; k < N; ++k)
          out[k] = in[k];
      else
        rsweep<N, T>(tb.SiT, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k * N] = out[k];
    }
  __syncthreads();
  // phase 3: S^{-T} along x, then V^{-1} W^{-1} along x (real input)
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      T        *p  = R + cl * NQ + N * r;
      T        *pi = Xi + cl * NQ + N * r;
      T         in[N], xr[N], xi[N], yr[N], yi[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k];
      if (GAUSS)
        for (int k = 0; k < N; ++k)
          xr[k] = in[k];
      else
        rsweep<N, T>(tb.SiT, in, xr);
#pragma unroll
      for (int k = 0; k < N; ++k)
        xi[k] = T(0);
      const int s = sgn[cl * 3 + 0];
      csweep<N, T>(VWr(s), VWi(s), xr, xi, yr, yi);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k] = yr[k], pi[k] = yi[k];
    }
  __syncthreads();
  // phase 4: V^{-1} W^{-1} along y
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const int off = cl * NQ + (r % N) + NF * (r / N);
      T         xr[N], xi[N], yr[N], yi[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        xr[k] = R[off + k * N], xi[k] = Xi[off + k * N];
      const int s = sgn[cl * 3 + 1];
      csweep<N, T>(VWr(s), VWi(s), xr, xi, yr, yi);
#pragma unroll
      for (int k = 0; k < N; ++k)
        R[off + k * N] = yr[k], Xi[off + k * N] = yi[k];
    }
  __syncthreads();
  // phase 5: V^{-1} W^{-1} along z, eigenvalue scaling, V along z
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const int off = cl * NQ + r;
      T         xr[N], xi[N], yr[N], yi[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        xr[k] = R[off + k * NF], xi[k] = Xi[off + k * NF];
      const int sx = sgn[cl * 3 + 0], sy = sgn[cl * 3 + 1], sz = sgn[cl * 3 + 2];
      csweep<N, T>(VWr(sz), VWi(sz), xr, xi, yr, yi);
      const T  tf  = T(A.time_factor);
      const T *ci  = cinfo + cl * 4;
      const int i0 = r % N, i1 = r / N;
      // c + s (v_x lambda_x(i0) + v_y lambda_y(i1)), then + s v_z lambda_z(k)
      const T br = T(A.mass_factor) + tf * (ci[0] * Lr(sx)[i0] + ci[1] * Lr(sy)[i1]);
      const T bi = tf * (ci[0] * Li(sx)[i0] + ci[1] * Li(sy)[i1]);
#pragma unroll
      for (int k = 0; k < N; ++k)
        {
          const T dr = br + tf * ci[2] * Lr(sz)[k], di = bi + tf * ci[2] * Li(sz)[k];
          const T f  = ci[3] / (dr * dr + di * di); // (1/|K|) / (dr + i di)
          const T ar = yr[k], ai = yi[k];
          yr[k]      = f * (ar * dr + ai * di);
          yi[k]      = f * (ai * dr - ar * di);
        }
      csweep<N, T>(Vr(sz), Vi(sz), yr, yi, xr, xi);
#pragma unroll
      for (int k = 0; k < N; ++k)
        R[off + k * NF] = xr[k], Xi[off + k * NF] = xi[k];
    }
  __syncthreads();
  // phase 6: V along y
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const int off = cl * NQ + (r % N) + NF * (r / N);
      T         xr[N], xi[N], yr[N], yi[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        xr[k] = R[off + k * N], xi[k] = Xi[off + k * N];
      const int s = sgn[cl * 3 + 1];
      csweep<N, T>(Vr(s), Vi(s), xr, xi, yr, yi);
#pragma unroll
      for (int k = 0; k < N; ++k)
        R[off + k * N] = yr[k], Xi[off + k * N] = yi[k];
    }
  __syncthreads();
  // phase 7: V along x, real part, S^{-1} along x
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      T        *p  = R + cl * NQ + N * r;
      const T  *pi = Xi + cl * NQ + N * r;
      T         xr[N], xi[N], yr[N], yi[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        xr[k] = p[k], xi[k] = pi[k];
      const int s = sgn[cl * 3 + 0];
      csweep<N, T>(Vr(s), Vi(s), xr, xi, yr, yi);
      if (GAUSS)
        for (int k = 0; k < N; ++k)
          out[k] = yr[k];
      else
        rsweep<N, T>(tb.Si, yr, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k] = out[k];
    }
  __syncthreads();
  // phase 8: S^{-1} along y
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int r = w % NF;
      T        *p = R + (w / NF) * NQ + (r % N) + NF * (r / N);
      T         in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * N];
      if (GAUSS)
        for (int k = 0; k < N; ++k)
          out[k] = in[k];
      else
        rsweep<N, T>(tb.Si, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k * N] = out[k];
    }
  __syncthreads();
  // phase 9: S^{-1} along z, write the nodal result (coalesced over (x, y))
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const T  *p  = R + cl * NQ + r;
      T         in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * NF];
      if (GAUSS)
        for (int k = 0; k < N; ++k)
          out[k] = in[k];
      else
        rsweep<N, T>(tb.Si, in, out);
      double *d = A.dst + (cell0 + cl) * NQ + r;
#pragma unroll
      for (int k = 0; k < N; ++k)
        d[k * NF] = (double)out[k];
    }
}

// cellwise mass matrix S^T diag(JxW) S, FP64; JxW = w / idet (field) or w V (uniform)
template <int N>
__global__ void __launch_bounds__(FdmShape<N>::THREADS) mass_kernel(const MassArgs A)
{
  using SH        = FdmShape<N>;
  constexpr int C = SH::C, NQ = SH::NQ, NF = SH::NF, NT = SH::THREADS;
  __shared__ double        R[C * NQ];
  const DevTables<double> &tb    = tab<double>(N);
  const int                tid   = threadIdx.x;
  const long long          cell0 = (long long)blockIdx.x * C;
  const int                ncell = (int)min((long long)C, A.n_cells - cell0);
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int     cl = w / NF, r = w % NF;
      const double *g  = A.src + (cell0 + cl) * NQ + r;
      double        in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = __ldg(g + k * NF);
      rsweep<N, double>(tb.S, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        R[cl * NQ + r + k * NF] = out[k];
    }
  __syncthreads();
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int r = w % NF;
      double   *p = R + (w / NF) * NQ + (r % N) + NF * (r / N);
      double    in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * N];
      rsweep<N, double>(tb.S, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k * N] = out[k];
    }
  __syncthreads();
  // S along x, JxW, S^T along x
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      double   *p  = R + cl * NQ + N * r;
      double    in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k];
      rsweep<N, double>(tb.S, in, out);
      const double wyz = tb.gw[r % N] * tb.gw[r / N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        {
          const double wq = wyz * tb.gw[k];
          out[k] *= A.uniform ? wq * A.vol : wq / __ldg(A.cell_geo + (cell0 + cl) * 4 * NQ + 3 * NQ + N * r + k);
        }
      rsweep<N, double>(tb.St, out, in);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k] = in[k];
    }
  __syncthreads();
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int r = w % NF;
      double   *p = R + (w / NF) * NQ + (r % N) + NF * (r / N);
      double    in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * N];
      rsweep<N, double>(tb.St, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k * N] = out[k];
    }
  __syncthreads();
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int     cl = w / NF, r = w % NF;
      const double *p  = R + cl * NQ + r;
      double        in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * NF];
      rsweep<N, double>(tb.St, in, out);
      double *d = A.dst + (cell0 + cl) * NQ + r;
#pragma unroll
      for (int k = 0; k < N; ++k)
        d[k * NF] = out[k];
    }
}

// ---------------------------------------------------------------- FP64 vectors
constexpr int kVecThreads = 256;

// partials[b * m + i] = sum over block b's elements of V_i . w (V_i = V +
// i * ld), one basis vector at a time: each is a plain coalesced stream
// (evict-first loads), four elements per thread in flight per step, and w,
// read once per vector, stays in L2 while the basis vectors stream past.
// Per vector one block reduction in a fixed order, so results repeat.
__global__ void __launch_bounds__(kVecThreads)
  multi_dot_kernel(const double *__restrict__ V, long long ld, int m, const double *__restrict__ w, long long n,
                   double *partials)
{
  __shared__ double red[kVecThreads / 32];
  const int         lane = threadIdx.x % 32, warp = threadIdx.x / 32;
  const long long   stride = (long long)gridDim.x * blockDim.x;
  const long long   first  = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  for (int i = 0; i < m; ++i)
    {
      const double *v  = V + i * ld;
      double        s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      long long     e  = first;
      for (; e + 3 * stride < n; e += 4 * stride)
        {
          s0 = fma(__ldcs(v + e), __ldg(w + e), s0);
          s1 = fma(__ldcs(v + e + stride), __ldg(w + e + stride), s1);
          s2 = fma(__ldcs(v + e + 2 * stride), __ldg(w + e + 2 * stride), s2);
          s3 = fma(__ldcs(v + e + 3 * stride), __ldg(w + e + 3 * stride), s3);
        }
      for (; e < n; e += stride)
        s0 = fma(__ldcs(v + e), __ldg(w + e), s0);
      double t = (s0 + s1) + (s2 + s3);
      for (int o = 16; o > 0; o >>= 1)
        t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0)
        red[warp] = t;
      __syncthreads();
      if (threadIdx.x == 0)
        {
          double b = 0.0;
          for (int k = 0; k < kVecThreads / 32; ++k)
            b += red[k];
          partials[blockIdx.x * m + i] = b;
        }
      __syncthreads();
    }
}

// out[i] = sum_b partials[b * m + i]: block i, strided partial sums per
// thread and a tree over the threads (a fixed order, so results repeat)
__global__ void __launch_bounds__(kVecThreads) reduce_partials_kernel(const double *partials, int blocks, int m,
                                                                      double *out)
{
  __shared__ double red[kVecThreads / 32];
  const int         i = blockIdx.x;
  double            s = 0.0;
  for (int b = threadIdx.x; b < blocks; b += blockDim.x)
    s += partials[b * m + i];
  for (int o = 16; o > 0; o >>= 1)
    s += __shfl_down_sync(0xffffffffu, s, o);
  if (threadIdx.x % 32 == 0)
    red[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0)
    {
      double t = 0.0;
      for (int k = 0; k < kVecThreads / 32; ++k)
        t += red[k];
      out[i] = t;
    }
}

// w += sign * sum_i coef[i] V_i
__global__ void __launch_bounds__(kVecThreads)
  multi_axpy_kernel(double *w, const double *__restrict__ V, long long ld, int m, const double *__restrict__ coef,
                    double sign, long long n)
{
  __shared__ double c[64];
  if (threadIdx.x < m)
    c[threadIdx.x] = sign * coef[threadIdx.x];
  __syncthreads();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    {
      double s = w[e];
      for (int i = 0; i < m; ++i)
        s = fma(c[i], __ldcs(V + i * ld + e), s);
      w[e] = s;
    }
}

// dst = a x + b y (y may be null: dst = a x)
__global__ void __launch_bounds__(kVecThreads)
  lincomb_kernel(double *dst, double a, const double *x, double b, const double *y, long long n)
{
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    dst[e] = y ? fma(a, x[e], b * y[e]) : a * x[e];
}

int vec_blocks(long long n)
{
  const long long b = (n + kVecThreads - 1) / kVecThreads;
  return (int)(b < 2048 ? b : 2048);
}
} // namespace

cudaError_t upload_tables_implicit(const DevTables<double> *d, const DevTables<float> *f)
{
  return upload_tables_local(d, f);
}

cudaError_t launch_fdm(int n, int precision, const FdmArgs &a, const void *tables, const void *cell_data,
                       cudaStream_t s)
{
#define ADV_FDM_CASE(NN)                                                                                       \
  case NN:                                                                                                     \
    {                                                                                                          \
      const unsigned blocks = (unsigned)((a.n_cells + FdmShape<NN>::C - 1) / FdmShape<NN>::C);               \
      const double *td = static_cast<const double *>(tables), *cd = static_cast<const double *>(cell_data);    \
      const float  *tf = static_cast<const float *>(tables), *cf = static_cast<const float *>(cell_data);      \
      if (precision == 0 && a.gauss)                                                                           \
        fdm_kernel<NN, double, true><<<blocks, FdmShape<NN>::THREADS, 0, s>>>(a, td, cd);                     \
      else if (precision == 0)                                                                                 \
        fdm_kernel<NN, double, false><<<blocks, FdmShape<NN>::THREADS, 0, s>>>(a, td, cd);                    \
      else if (a.gauss)                                                                                        \
        fdm_kernel<NN, float, true><<<blocks, FdmShape<NN>::THREADS, 0, s>>>(a, tf, cf);                      \
      else                                                                                                     \
        fdm_kernel<NN, float, false><<<blocks, FdmShape<NN>::THREADS, 0, s>>>(a, tf, cf);                     \
      break;                                                                                                   \
    }
  switch (n)
    {
      ADV_FDM_CASE(2)
      ADV_FDM_CASE(3)
      ADV_FDM_CASE(4)
      ADV_FDM_CASE(5)
      ADV_FDM_CASE(6)
      ADV_FDM_CASE(7)
      default:
        return cudaErrorInvalidValue;
    }
#undef ADV_FDM_CASE
  return cudaGetLastError();
}

cudaError_t launch_mass(int n, const MassArgs &a, cudaStream_t s)
{
#define ADV_MASS_CASE(NN)                                                                                      \
  case NN:                                                                                                     \
    mass_kernel<NN><<<(unsigned)((a.n_cells + FdmShape<NN>::C - 1) / FdmShape<NN>::C), FdmShape<NN>::THREADS, 0, \
                      s>>>(a);                                                                                 \
    break;
  switch (n)
    {
      ADV_MASS_CASE(2)
      ADV_MASS_CASE(3)
      ADV_MASS_CASE(4)
      ADV_MASS_CASE(5)
      ADV_MASS_CASE(6)
      ADV_MASS_CASE(7)
      default:
        return cudaErrorInvalidValue;
    }
#undef ADV_MASS_CASE
  return cudaGetLastError();
}

int vec_partial_blocks(long long n)
{
  return vec_blocks(n);
}

cudaError_t launch_multi_dot(const double *V, long long ld, int m, const double *w, long long n, double *partials,
                             double *out, cudaStream_t s)
{
  // about 16 elements per thread and vector between two block reductions
  // (at most vec_blocks(n) blocks, the size of the partials)
  const long long want   = (n + 16 * kVecThreads - 1) / (16 * kVecThreads);
  const int       blocks = (int)std::max<long long>(1, std::min<long long>(want, std::min(vec_blocks(n), 152 * 6)));
  multi_dot_kernel<<<blocks, kVecThreads, 0, s>>>(V, ld, m, w, n, partials);
  reduce_partials_kernel<<<m, kVecThreads, 0, s>>>(partials, blocks, m, out);
  return cudaGetLastError();
}

cudaError_t launch_multi_axpy(double *w, const double *V, long long ld, int m, const double *coef, double sign,
                              long long n, cudaStream_t s)
{
  multi_axpy_kernel<<<vec_blocks(n), kVecThreads, 0, s>>>(w, V, ld, m, coef, sign, n);
  return cudaGetLastError();
}

cudaError_t launch_lincomb(double *dst, double a, const double *x, double b, const double *y, long long n,
                           cudaStream_t s)
{
  lincomb_kernel<<<vec_blocks(n), kVecThreads, 0, s>>>(dst, a, x, b, y, n);
  return cudaGetLastError();
}

namespace
{
// dst = JxW (a x + b y) at every Gauss point (y may be null), grid-stride over
// the points; JxW = w_q / idet_q from the cell geometry, or w_q V (uniform)
template <int N>
__global__ void __launch_bounds__(kVecThreads)
  gauss_mass_lincomb_kernel(double *dst, double a, const double *x, double b, const double *y, long long n_cells,
                            const double *cell_geo, double vol)
{
  constexpr int            NQ = N * N * N;
  const DevTables<double> &tb = tab<double>(N);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_cells * NQ;
       e += (long long)gridDim.x * blockDim.x)
    {
      const long long c   = e / NQ;
      const int       q   = (int)(e - c * NQ);
      const double    w   = tb.gw[q % N] * tb.gw[(q / N) % N] * tb.gw[q / (N * N)];
      const double    jxw = cell_geo ? w / __ldg(cell_geo + c * 4 * NQ + 3 * NQ + q) : w * vol;
      double          v   = a * __ldg(x + e);
      if (y)
        v = fma(b, __ldg(y + e), v);
      dst[e] = jxw * v;
    }
}
} // namespace

cudaError_t launch_gauss_mass_lincomb(int n, double *dst, double a, const double *x, double b, const double *y,
                                      long long n_cells, const double *cell_geo, double vol, cudaStream_t s)
{
  const long long total  = n_cells * n * n * n;
  const unsigned  blocks = (unsigned)std::min<long long>((total + kVecThreads - 1) / kVecThreads, 152 * 16);
  switch (n)
    {
      case 2: gauss_mass_lincomb_kernel<2><<<blocks, kVecThreads, 0, s>>>(dst, a, x, b, y, n_cells, cell_geo, vol); break;
      case 3: gauss_mass_lincomb_kernel<3><<<blocks, kVecThreads, 0, s>>>(dst, a, x, b, y, n_cells, cell_geo, vol); break;
      case 4: gauss_mass_lincomb_kernel<4><<<blocks, kVecThreads, 0, s>>>(dst, a, x, b, y, n_cells, cell_geo, vol); break;
      case 5: gauss_mass_lincomb_kernel<5><<<blocks, kVecThreads, 0, s>>>(dst, a, x, b, y, n_cells, cell_geo, vol); break;
      case 6: gauss_mass_lincomb_kernel<6><<<blocks, kVecThreads, 0, s>>>(dst, a, x, b, y, n_cells, cell_geo, vol); break;
      case 7: gauss_mass_lincomb_kernel<7><<<blocks, kVecThreads, 0, s>>>(dst, a, x, b, y, n_cells, cell_geo, vol); break;
      default: return cudaErrorInvalidValue;
    }
  return cudaGetLastError();
}
} // namespace adv
