// Device-side helpers shared by the kernels: 1D tables in constant memory,
// integer-pipe conversions between IEEE binary64 and binary32, and the
// analytic solutions used for initial data, Dirichlet data and errors.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/advection_gb300.h"

namespace adv
{
constexpr int kMaxNDev = 7;

// Even-odd form of an n x n matrix M that is symmetric (M[n-1-q][n-1-i] =
// M[q][i]) or antisymmetric (= -M[q][i]) under reflection of both indices:
// with e_i = x_i + x_{n-1-i}, o_i = x_i - x_{n-1-i} (i < n/2) and the middle
// entry c (odd n), out_q = E_q + O_q and out_{n-1-q} = E_q - O_q
// (antisymmetric: O_q - E_q), E_q = sum e[q][i] e_i + ce[q] c,
// O_q = sum o[q][i] o_i; the middle output is sum mid[i] e_i + cc c
// (antisymmetric: sum mid[i] o_i).  For n = 5 a sweep costs 21 instead of 25
// operations.
template <typename T>
struct EvenOdd
{
  T e[4][4], o[4][4], ce[4], mid[4], cc;
};

template <typename T>
struct DevTables
{
  T S[kMaxNDev][kMaxNDev];  // nodal -> Gauss values
  T Si[kMaxNDev][kMaxNDev]; // Gauss values -> nodal (S^{-1})
  T Dw[kMaxNDev][kMaxNDev]; // weighted collocation derivative (integration by parts)
  T D[kMaxNDev][kMaxNDev];  // collocation derivative on the Gauss points
  T l0[kMaxNDev], l1[kMaxNDev];   // Gauss-Lagrange basis at xi = 0, 1
  T lw0[kMaxNDev], lw1[kMaxNDev]; // the same divided by the Gauss weights
  T gw[kMaxNDev];                 // Gauss weights
  EvenOdd<T> S_eo, Si_eo, Dw_eo, D_eo;  // S, S^-1 symmetric; Dw, D antisymmetric
  T St[kMaxNDev][kMaxNDev], SiT[kMaxNDev][kMaxNDev]; // transposes of S and S^-1
  EvenOdd<T> St_eo, SiT_eo;
  // viscous (SIPG) terms: Gauss-Lagrange derivatives at the faces, the same
  // divided by the weights, nodal-basis derivatives at the faces
  T ld0[kMaxNDev], ld1[kMaxNDev], lwd0[kMaxNDev], lwd1[kMaxNDev], dphi0[kMaxNDev], dphi1[kMaxNDev];
  // lift vectors split by the mirror symmetry lw1[q] = lw0[n-1-q]:
  // lwe[q] = (lw0[q] + lw0[n-1-q]) / 2, lwo[q] = (lw0[q] - lw0[n-1-q]) / 2
  // for q < n/2, lwe[n/2] = lw0[n/2] for odd n
  T lwe[kMaxNDev], lwo[kMaxNDev];
  // the same split of the derivative lifts (lwd1[q] = -lwd0[n-1-q]):
  // lde[q] = (lwd0[q] + lwd0[n-1-q]) / 2, ldo[q] = (lwd0[q] - lwd0[n-1-q]) / 2,
  // lde[n/2] = lwd0[n/2] for odd n
  T lde[kMaxNDev], ldo[kMaxNDev];
};

// Index [n] holds the tables of n points per direction.  The library is
// built without relocatable device code, so every translation unit that
// includes this header owns a copy, filled by its own upload function.
static __constant__ DevTables<double> c_tab_d[kMaxNDev + 1];
static __constant__ DevTables<float>  c_tab_f[kMaxNDev + 1];

static inline cudaError_t upload_tables_local(const DevTables<double> *d, const DevTables<float> *f)
{
  cudaError_t e = cudaMemcpyToSymbol(c_tab_d, d, sizeof(c_tab_d));
  if (e != cudaSuccess)
    return e;
  return cudaMemcpyToSymbol(c_tab_f, f, sizeof(c_tab_f));
}

// One-time opt-in of a kernel's dynamic shared-memory size on the current
// device (a per-device function attribute).  The mask of configured devices
// is atomic because handles on different host threads may launch the same
// kernel concurrently; two threads that both see the bit clear both set the
// attribute, which is harmless.  Devices 64 and up set it on every launch.
template <typename K>
inline cudaError_t opt_in_smem(K kernel, int bytes, std::atomic<unsigned long long> &configured)
{
  int         dev = 0;
  cudaError_t e   = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return e;
  if (dev < 64 && ((configured.load(std::memory_order_acquire) >> dev) & 1ull))
    return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && dev < 64)
    configured.fetch_or(1ull << dev, std::memory_order_acq_rel);
  return e;
}

template <typename T>
__device__ __forceinline__ const DevTables<T> &tab(int n);
template <>
__device__ __forceinline__ const DevTables<double> &tab<double>(int n)
{
  return c_tab_d[n];
}
template <>
__device__ __forceinline__ const DevTables<float> &tab<float>(int n)
{
  return c_tab_f[n];
}

// binary64 -> binary32 by integer arithmetic (round half away from zero in
// magnitude; |x| below the smallest normal binary32 flushes to a signed
// zero; |x| >= 2^128 and infinities give a signed infinity, as does a
// rounding that carries past the largest binary32; NaN gives a quiet NaN).
// On this GPU F2F conversions issue on the FP64 pipe, which the FP32-operator
// path otherwise reserves for the FP64 vector updates.
__device__ __forceinline__ float d2f_int(double x)
{
  const long long b   = __double_as_longlong(x);
  const unsigned  hi  = (unsigned)((unsigned long long)b >> 32);
  const unsigned  lo  = (unsigned)b;
  const unsigned  ahi = hi & 0x7FFFFFFFu;
  // exponent and top 23 mantissa bits, exponent rebased from 1023 to 127
  const unsigned mag = __funnelshift_l(lo, hi, 3) + ((lo >> 28) & 1u) - 0xC0000000u;
  unsigned       r   = ahi < 0x38100000u ? 0u : mag;
  // binary64 exponent >= 1151 (|x| >= 2^128), infinity or NaN
  if (ahi >= 0x47F00000u)
    r = (ahi > 0x7FF00000u || (ahi == 0x7FF00000u && lo != 0u)) ? 0x7FC00000u : 0x7F800000u;
  return __uint_as_float(r | (hi & 0x80000000u));
}

// binary32 -> binary64, exact for normal numbers, infinities and NaN (the
// payload keeps its leading bits); subnormals become zero.
__device__ __forceinline__ double f2d_int(float f)
{
  const unsigned b    = __float_as_uint(f);
  const unsigned a    = b & 0x7FFFFFFFu;
  const unsigned sign = b & 0x80000000u;
  const bool     zero = a < 0x00800000u;
  unsigned       hi   = zero ? sign : (sign | ((a >> 3) + 0x38000000u));
  if (a >= 0x7F800000u)
    hi = sign | 0x7FF00000u | ((a >> 3) & 0x000FFFFFu);
  const unsigned lo = zero ? 0u : (b << 29);
  return __hiloint2double((int)hi, (int)lo);
}

template <typename T>
__device__ __forceinline__ T from_double(double x);
template <>
__device__ __forceinline__ double from_double<double>(double x)
{
  return x;
}
template <>
__device__ __forceinline__ float from_double<float>(double x)
{
  return d2f_int(x);
}

template <typename T>
__device__ __forceinline__ double to_double(T x);
template <>
__device__ __forceinline__ double to_double<double>(double x)
{
  return x;
}
template <>
__device__ __forceinline__ double to_double<float>(float x)
{
  return f2d_int(x);
}

// Parameters of the analytic solution (initial data / Dirichlet data).
struct ExactParams
{
  int    type;          // ADV_IC_*
  int    constant_velocity;
  double velocity[3];
  double lo[3], L[3];
  double p[8];
};

// The initial condition translated with the constant velocity (for the
// rotating field: the initial condition).  Mirrors ExactSolution::value
// (advection_solver.cc:149-172) for the workloads' initial data.
__host__ __device__ __forceinline__ double exact_value(const ExactParams &e, double x0, double x1, double x2,
                                              double t)
{
  const double kPi = 3.14159265358979323846;
  const double tt  = e.constant_velocity ? t : 0.0;
  const double x[3] = {x0, x1, x2};
  if (e.type == ADV_IC_SINE_GAUSS)
    {
      double s[3], r2 = 0.0;
      for (int d = 0; d < 3; ++d)
        {
          const double y = (x[d] - e.velocity[d] * tt - e.lo[d]) / e.L[d] - e.p[d];
          s[d]           = y - floor(y);
          r2 += (s[d] - 0.5) * (s[d] - 0.5);
        }
#ifdef __CUDA_ARCH__
      // sin(2 pi s) as sinpi(2 s): exact argument reduction, no product with pi
      return sinpi(2.0 * s[0]) * sinpi(2.0 * s[1]) * sinpi(2.0 * s[2]) + exp(-50.0 * r2);
#else
      return sin(2.0 * kPi * s[0]) * sin(2.0 * kPi * s[1]) * sin(2.0 * kPi * s[2]) + exp(-50.0 * r2);
#endif
    }
  if (e.type == ADV_IC_BLOB)
    {
      double r2 = 0.0;
      for (int d = 0; d < 3; ++d)
        {
          const double y = x[d] - e.velocity[d] * tt - e.p[d];
          r2 += y * y;
        }
      return exp(-r2 / (e.p[3] * e.p[3]));
    }
#ifdef __CUDA_ARCH__
  double r = sinpi(4.0 * (x[0] - tt * e.velocity[0]));
  r *= cospi(4.0 * (x[1] - tt * e.velocity[1]));
  r *= cospi(4.0 * (x[2] - tt * e.velocity[2]));
#else
  double r = sin(4.0 * kPi * (x[0] - tt * e.velocity[0]));
  r *= cos(4.0 * kPi * (x[1] - tt * e.velocity[1]));
  r *= cos(4.0 * kPi * (x[2] - tt * e.velocity[2]));
#endif
  return r;
}

// position of the deformed box (ADV_MESH_DEFORMED)
__device__ __forceinline__ void deform_dev(double A, const double lo[3], const double L[3],
                                           const double x[3], double y[3])
{
  double s[3];
  for (int d = 0; d < 3; ++d)
    s[d] = (x[d] - lo[d]) / L[d];
  for (int d = 0; d < 3; ++d)
    y[d] = x[d] + A * L[d] * sinpi(2.0 * s[(d + 1) % 3]) * sinpi(2.0 * s[(d + 2) % 3]);
}
} // namespace adv
