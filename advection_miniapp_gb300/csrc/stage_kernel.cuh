// Fused matrix-free DG advection stage for sm_103a.
//
// One launch evaluates, for every cell, k = M^{-1} L(r_in) and applies the
// low-storage Runge-Kutta update, replacing the reference's data.loop
// (cell / inner-face / boundary-face workers, advection_solver.cc:469-631,
// 710-718) followed by the inverse-mass cell_loop with its vector-update
// lambda (advection_solver.cc:635-657, 722-752).
//
// Formulation (all in the space of the (k+1)^3 Gauss points of a cell):
//   U   = (S x S x S) u                     values at the Gauss points
//   Z   = idet * [ sum_d Dw_d (vt_d . U)    volume term, integrated by parts
//                 + sum_faces lw(s) phi ]   face fluxes lifted to the points
//   k   = (S^-1 x S^-1 x S^-1) Z            inverse mass matrix
// Because the Gauss-Lobatto nodal basis and the Gauss points share the
// tensor structure, S^-T cancels the transposed interpolation of the
// integration step, so the exact cellwise inverse mass matrix of the
// reference (CellwiseInverseMassMatrix, S^-1 diag(1/JxW) S^-T) costs one set
// of three sweeps.  Face values of the own cell are contractions of the
// Gauss-point values with l_q(0), l_q(1); neighbour values are its nodal face
// layer (Gauss-Lobatto nodes include the end points) interpolated to the face
// Gauss points.  Each face flux is computed from both sides, so no atomics
// are needed and every cell is independent.
//
// Threads: one thread per 1D pencil of a cell, C cells per CTA; phases are
// separated by __syncthreads.  The data of a CTA's cells stay in shared
// memory from the load of r_in to the final sweep, whose output goes straight
// from registers into the LSRK update.
#pragma once

#include <cuda_pipeline.h>

#include <type_traits>

#include "kernels.h"

namespace adv
{
template <int N, typename T, bool UNI, bool VISC = false>
struct StageShape
{
  // cells per CTA: about 128 (or 256) threads with few idle lanes, so that
  // several CTAs share an SM and their load and compute phases overlap
  static constexpr int cells() { return N == 2 ? 32 : N == 3 ? 14 : N == 4 ? 8 : N == 5 ? 5 : N == 6 ? 7 : 5; }
  static constexpr int C       = cells();
  static constexpr int NQ      = N * N * N;
  static constexpr int NF      = N * N;
  static constexpr int WORK    = C * NF;
  static constexpr int THREADS = ((WORK + 31) / 32) * 32;
  // shared memory (values of T): Ub, Qb [C][NQ]; Nb [C][6][NF]; field case:
  // Gb [C][4][NQ] cell geometry, Fb [C][6][2][NF] face coefficients
  // viscous terms: Nd [C][6][NF] neighbour normal derivatives at the face points
  static constexpr int VALUES =
    2 * C * NQ + 6 * C * NF + (UNI ? 0 : 4 * C * NQ + 12 * C * NF) + (VISC ? 6 * C * NF : 0);
  static constexpr int SMEM   = VALUES * (int)sizeof(T) + 12 * C * (int)sizeof(int);
  // the nodal kernel with the binary32 operator on field geometry reads the
  // face coefficients from global memory instead of staging them: one more
  // resident CTA per SM for a latency-bound kernel
  static constexpr bool FACES_GLOBAL = sizeof(T) == sizeof(float) && !UNI && !VISC;
  static constexpr int  SMEM_NODAL   = SMEM - (FACES_GLOBAL ? 12 * C * NF * (int)sizeof(T) : 0);
  // the cell geometry Gb (after Ub, Qb, Nb) is filled by 16-byte cp.async
  static_assert((2 * C * NQ + 6 * C * NF) * (int)sizeof(T) % 16 == 0, "cp.async destinations need 16-byte alignment");
};

// index of the point with coordinate a along direction d and (b, c) along
// the sorted tangential directions of d
template <int N>
__device__ __forceinline__ int idx3(int d, int a, int b, int c)
{
  return d == 0 ? a + N * (b + N * c) : d == 1 ? b + N * (a + N * c) : b + N * (c + N * a);
}

// uniform-case constants in the operator's precision
template <typename T>
struct Consts;
template <>
struct Consts<double>
{
  static __device__ __forceinline__ double cv(const StageArgs &A, int d) { return A.cv[d]; }
  static __device__ __forceinline__ double P(const StageArgs &A, int d) { return A.P[d]; }
  static __device__ __forceinline__ double M(const StageArgs &A, int d) { return A.M[d]; }
  static __device__ __forceinline__ double skew(const StageArgs &A) { return A.skew; }
  static __device__ __forceinline__ double K1(const StageArgs &A, int d) { return A.K1[d]; }
  static __device__ __forceinline__ double K2(const StageArgs &A, int d) { return A.K2[d]; }
  static __device__ __forceinline__ double cdiff(const StageArgs &A, int d) { return A.cdiff[d]; }
  static __device__ __forceinline__ double sa(const StageArgs &A) { return A.adv_scale; }
  static __device__ __forceinline__ double mass(const StageArgs &A) { return A.mass_factor; }
  static __device__ __forceinline__ double out(const StageArgs &A) { return A.out_scale; }
  static __device__ __forceinline__ double vol(const StageArgs &A) { return A.vol; }
};
template <>
struct Consts<float>
{
  static __device__ __forceinline__ float cv(const StageArgs &A, int d) { return A.cvf[d]; }
  static __device__ __forceinline__ float P(const StageArgs &A, int d) { return A.Pf[d]; }
  static __device__ __forceinline__ float M(const StageArgs &A, int d) { return A.Mf[d]; }
  static __device__ __forceinline__ float skew(const StageArgs &A) { return A.skewf; }
  static __device__ __forceinline__ float K1(const StageArgs &A, int d) { return A.K1f[d]; }
  static __device__ __forceinline__ float K2(const StageArgs &A, int d) { return A.K2f[d]; }
  static __device__ __forceinline__ float cdiff(const StageArgs &A, int d) { return A.cdifff[d]; }
  static __device__ __forceinline__ float sa(const StageArgs &A) { return A.adv_scalef; }
  static __device__ __forceinline__ float mass(const StageArgs &A) { return A.mass_factorf; }
  static __device__ __forceinline__ float out(const StageArgs &A) { return (float)A.out_scale; }
  static __device__ __forceinline__ float vol(const StageArgs &A) { return A.volf; }
};

template <int N, typename T>
__device__ __forceinline__ void sweep(const T (&M)[kMaxNDev][kMaxNDev], const T (&in)[N], T (&out)[N])
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

// The same product through the even-odd form (fewer operations for n >= 5).
template <int N, typename T, bool ANTI>
__device__ __forceinline__ void sweep_eo(const EvenOdd<T> &M, const T (&in)[N], T (&out)[N])
{
  constexpr int H = N / 2;
  T             e[H > 0 ? H : 1], o[H > 0 ? H : 1];
#pragma unroll
  for (int i = 0; i < H; ++i)
    {
      e[i] = in[i] + in[N - 1 - i];
      o[i] = in[i] - in[N - 1 - i];
    }
#pragma unroll
  for (int q = 0; q < H; ++q)
    {
      T E = M.e[q][0] * e[0], O = M.o[q][0] * o[0];
#pragma unroll
      for (int i = 1; i < H; ++i)
        {
          E = fma(M.e[q][i], e[i], E);
          O = fma(M.o[q][i], o[i], O);
        }
      if (N % 2)
        E = fma(M.ce[q], in[H], E);
      out[q]         = E + O;
      out[N - 1 - q] = ANTI ? O - E : E - O;
    }
  if (N % 2)
    {
      T m = ANTI ? M.mid[0] * o[0] : fma(M.mid[0], e[0], M.cc * in[H]);
#pragma unroll
      for (int i = 1; i < H; ++i)
        m = fma(M.mid[i], ANTI ? o[i] : e[i], m);
      out[H] = m;
    }
}

// out = Dw-type (antisymmetric) even-odd product of `in` plus the lifted face
// fluxes lw0 phlo + lw1 phhi, folded into the recombination of the even and
// odd halves: with ps = phlo + phhi, pd = phlo - phhi, the lift of point q is
// lwe[q] ps + lwo[q] pd and of point n-1-q lwe[q] ps - lwo[q] pd, so the
// pair costs two FMAs instead of four.
// DL adds the SIPG derivative lifts lwd0 dlo + lwd1 dhi the same way (by
// the symmetry lwd1[q] = -lwd0[n-1-q]: lde[q] (dlo - dhi) + ldo[q] (dlo + dhi)
// at q, lde[q] (dlo - dhi) - ldo[q] (dlo + dhi) at n-1-q).
// The sweep from the even and odd parts e[i] = in[i] + in[n-1-i],
// o[i] = in[i] - in[n-1-i] and the middle value in[n/2] (odd n).
template <int N, typename T, bool DL = false>
__device__ __forceinline__ void sweep_eo_anti_lift_parts(const EvenOdd<T> &M, const T (&e)[N / 2],
                                                         const T (&o)[N / 2], T mid, T phlo, T phhi, const T *lwe,
                                                         const T *lwo, T (&out)[N], T dlo = T(0), T dhi = T(0),
                                                         const T *lde = nullptr, const T *ldo = nullptr)
{
  constexpr int H  = N / 2;
  const T       ps = phlo + phhi, pd = phlo - phhi;
  const T       ds = dlo - dhi, dd = dlo + dhi;
#pragma unroll
  for (int q = 0; q < H; ++q)
    {
      T E = M.e[q][0] * e[0], O = M.o[q][0] * o[0];
#pragma unroll
      for (int i = 1; i < H; ++i)
        {
          E = fma(M.e[q][i], e[i], E);
          O = fma(M.o[q][i], o[i], O);
        }
      if (N % 2)
        E = fma(M.ce[q], mid, E);
      T a = fma(lwe[q], ps, O);
      T b = fma(lwo[q], pd, E);
      if (DL)
        {
          a = fma(lde[q], ds, a);
          b = fma(ldo[q], dd, b);
        }
      out[q]         = a + b;
      out[N - 1 - q] = a - b;
    }
  if (N % 2)
    {
      T m = M.mid[0] * o[0];
#pragma unroll
      for (int i = 1; i < H; ++i)
        m = fma(M.mid[i], o[i], m);
      m = fma(lwe[H], ps, m);
      if (DL)
        m = fma(lde[H], ds, m);
      out[H] = m;
    }
}

template <int N, typename T, bool DL = false>
__device__ __forceinline__ void sweep_eo_anti_lift(const EvenOdd<T> &M, const T (&in)[N], T phlo, T phhi,
                                                   const T *lwe, const T *lwo, T (&out)[N], T dlo = T(0),
                                                   T dhi = T(0), const T *lde = nullptr, const T *ldo = nullptr)
{
  constexpr int H = N / 2;
  T             e[H], o[H];
#pragma unroll
  for (int i = 0; i < H; ++i)
    {
      e[i] = in[i] + in[N - 1 - i];
      o[i] = in[i] - in[N - 1 - i];
    }
  sweep_eo_anti_lift_parts<N, T, DL>(M, e, o, N % 2 ? in[H] : T(0), phlo, phhi, lwe, lwo, out, dlo, dhi, lde,
                                     ldo);
}

// Sweep with the cheaper of the two forms: even-odd pays off from n = 5.
template <int N, typename T, bool ANTI>
__device__ __forceinline__ void sweep2(const T (&M)[kMaxNDev][kMaxNDev], const EvenOdd<T> &Meo,
                                       const T (&in)[N], T (&out)[N])
{
  if (N >= 5)
    sweep_eo<N, T, ANTI>(Meo, in, out);
  else
    sweep<N, T>(M, in, out);
}

// Face terms and volume term of one direction d for one pencil of Gauss-point
// values U along d; returns the pencil's contribution to Z (without 1/det J).
// Flo / Fhi: (P, M) pairs of the low / high face (field case);
// vt: det J (J^{-1} a)_d along the pencil (field case).  VISC adds the SIPG
// terms of an affine mesh (advection_diffusion_solver.cc:531-613 in the
// right-hand-side sign convention): dnlo / dnhi are the neighbour's reference
// normal derivatives at the face points, blo / bhi mark Dirichlet faces
// (mirror data u+ = 2g - u-, grad u+ = grad u-).
// The own face values of the pencil: ulo = sum_q l_q(0) U_q, uhi = sum_q l_q(1) U_q.
template <int N, typename T>
__device__ __forceinline__ void pencil_traces(const DevTables<T> &tb, const T (&U)[N], T &ulo, T &uhi)
{
  ulo = tb.l0[0] * U[0], uhi = tb.l1[0] * U[0];
#pragma unroll
  for (int q = 1; q < N; ++q)
    {
      ulo = fma(tb.l0[q], U[q], ulo);
      uhi = fma(tb.l1[q], U[q], uhi);
    }
}

// The own reference normal derivatives at the faces of the pencil:
// sum_q l'_q(0) U_q and sum_q l'_q(1) U_q.
template <int N, typename T>
__device__ __forceinline__ void pencil_dtraces(const DevTables<T> &tb, const T (&U)[N], T &dlo, T &dhi)
{
  dlo = tb.ld0[0] * U[0], dhi = tb.ld1[0] * U[0];
#pragma unroll
  for (int q = 1; q < N; ++q)
    {
      dlo = fma(tb.ld0[q], U[q], dlo);
      dhi = fma(tb.ld1[q], U[q], dhi);
    }
}

// OWN_TR: the own face values come precomputed (tr_lo, tr_hi), and with
// VISC the own reference normal derivatives at the faces (dtr_lo, dtr_hi)
// Upwind coefficients (P, M) of the low and high face of a pencil at one
// face point, after the exchange for a negative velocity time factor.
template <typename T>
struct FacePM
{
  T Plo, Mlo, Phi, Mhi;
};

// Flo / Fhi: (P, M) pairs of the low / high face (field case), read at face point fq
template <typename T, bool UNI, int D>
__device__ __forceinline__ FacePM<T> face_pm(const StageArgs &A, const T *Flo, const T *Fhi, int fq)
{
  FacePM<T> c;
  if (UNI)
    {
      c.Plo = c.Phi = Consts<T>::P(A, D);
      c.Mlo = c.Mhi = Consts<T>::M(A, D);
    }
  else
    {
      // (P, M) pairs per face point, 2 sizeof(T)-aligned
      using T2      = typename std::conditional<sizeof(T) == sizeof(double), double2, float2>::type;
      const T2 pmlo = *reinterpret_cast<const T2 *>(Flo + 2 * fq);
      const T2 pmhi = *reinterpret_cast<const T2 *>(Fhi + 2 * fq);
      c.Plo = pmlo.x, c.Mlo = pmlo.y;
      c.Phi = pmhi.x, c.Mhi = pmhi.y;
    }
  if (A.swap_pm)
    {
      T tmp = c.Plo;
      c.Plo = c.Mlo, c.Mlo = tmp;
      tmp   = c.Phi;
      c.Phi = c.Mhi, c.Mhi = tmp;
    }
  return c;
}

// The pass with the face coefficients given (face_pm).  UPW (upwind flux,
// one of P, M zero at every face point, no skew term): pm.Plo / pm.Phi hold
// the nonzero coefficient of the low / high face (or zero) and nlo / nhi the
// value on the upwind side there, own or neighbour; the flux is then one
// product per face, with the same value as the general form.
template <int N, typename T, bool UNI, bool VISC, int D, bool OWN_TR = false, bool UPW = false>
__device__ __forceinline__ void direction_pass_pm(const StageArgs &A, const DevTables<T> &tb,
                                                  const T (&U)[N], T nlo, T nhi, T dnlo, T dnhi, bool blo,
                                                  bool bhi, const FacePM<T> &pm, const T *vt, int vstride,
                                                  T (&out)[N], T tr_lo = T(0), T tr_hi = T(0),
                                                  T dtr_lo = T(0), T dtr_hi = T(0))
{
  constexpr int NF = N * N;
  static_assert(!UPW || (OWN_TR && !VISC), "the upwind form takes its face values from the caller");
  T ulo, uhi;
  if (OWN_TR)
    ulo = tr_lo, uhi = tr_hi;
  else
    pencil_traces<N, T>(tb, U, ulo, uhi);
  const T Plo = pm.Plo, Mlo = pm.Mlo, Phi = pm.Phi, Mhi = pm.Mhi;
  // numerical flux from the cell's point of view (outward normal):
  //   low face (cell is the "plus" side):  phi = M u_own + P u_nbr
  //   high face (cell is the "minus" side): phi = -P u_own - M u_nbr
  // plus the skew-symmetric correction -+ skew c u_own, c = P + M
  // (advection_solver.cc:554-574, 615-626)
  T phlo, phhi;
  if constexpr (UPW)
    {
      phlo = Plo * nlo;
      phhi = -(Phi * nhi);
    }
  else
    {
      phlo = fma(Mlo, ulo, Plo * nlo);
      phhi = -fma(Phi, uhi, Mhi * nhi);
    }
  if (!UPW && A.has_skew)
    {
      const T sk = Consts<T>::skew(A);
      phlo       = fma(-sk * (Plo + Mlo), ulo, phlo);
      phhi       = fma(sk * (Phi + Mhi), uhi, phhi);
    }
  // with diffusion the velocity time factor is applied here (it does not
  // scale the viscous terms); otherwise the caller folds it into b and a
  const T sa = VISC ? Consts<T>::sa(A) : T(1);
  if (VISC)
    {
      phlo *= sa;
      phhi *= sa;
    }
  // volume term: (1 - skew) (a u, grad v) - skew (a . grad u, v) - nu (grad u, grad v)
  // (advection_solver.cc:500-507); with vt = det J J^{-1} a per Gauss point
  if constexpr (!VISC && N >= 5)
    {
      // (1 - skew) Dw (c U) + lifts - skew c D U with c = a_d / h_d (uniform)
      // or vt (field); the lifts ride on the even-odd recombination
      const T cvd = Consts<T>::cv(A, D);
      const T sk  = A.has_skew ? Consts<T>::skew(A) : T(0);
      if (!UNI && !A.has_skew && sizeof(T) == sizeof(double))
        {
          // field, conservative form: the even and odd parts of vt U as
          // c_i U_i +- c_j U_j with one product and two FMAs per mirrored
          // pair (instead of two products and two additions)
          constexpr int H = N / 2;
          T             e[H], o[H];
#pragma unroll
          for (int i = 0; i < H; ++i)
            {
              const T p = vt[(N - 1 - i) * vstride] * U[N - 1 - i];
              e[i]      = fma(vt[i * vstride], U[i], p);
              o[i]      = fma(vt[i * vstride], U[i], -p);
            }
          sweep_eo_anti_lift_parts<N, T>(tb.Dw_eo, e, o, N % 2 ? vt[H * vstride] * U[H] : T(0), phlo, phhi,
                                         tb.lwe, tb.lwo, out);
          return;
        }
      T w[N], du[N];
#pragma unroll
      for (int q = 0; q < N; ++q)
        {
          const T c = UNI ? cvd : vt[q * vstride];
          w[q]      = A.has_skew ? (T(1) - sk) * (c * U[q]) : c * U[q];
        }
      sweep_eo_anti_lift<N, T>(tb.Dw_eo, w, phlo, phhi, tb.lwe, tb.lwo, out);
      if (A.has_skew)
        {
          sweep2<N, T, true>(tb.D, tb.D_eo, U, du);
#pragma unroll
          for (int q = 0; q < N; ++q)
            out[q] = fma(-sk * (UNI ? cvd : vt[q * vstride]), du[q], out[q]);
        }
      return;
    }
  // SIPG face terms: value coefficients join the flux, normal-derivative
  // coefficients are lifted with l'(s) / w
  T dlo = T(0), dhi = T(0);
  if (VISC)
    {
      T duo_lo, duo_hi;
      if (OWN_TR)
        duo_lo = dtr_lo, duo_hi = dtr_hi;
      else
        {
          duo_lo = tb.ld0[0] * U[0], duo_hi = tb.ld1[0] * U[0];
#pragma unroll
          for (int q = 1; q < N; ++q)
            {
              duo_lo = fma(tb.ld0[q], U[q], duo_lo);
              duo_hi = fma(tb.ld1[q], U[q], duo_hi);
            }
        }
      const T un_lo  = blo ? T(2) * nlo - ulo : nlo;
      const T un_hi  = bhi ? T(2) * nhi - uhi : nhi;
      const T dun_lo = blo ? duo_lo : dnlo;
      const T dun_hi = bhi ? duo_hi : dnhi;
      const T K1 = Consts<T>::K1(A, D), K2 = Consts<T>::K2(A, D);
      const T jl = un_lo - ulo, jh = uhi - un_hi; // jumps u- - u+ across the low / high face
      phlo       = fma(K1, jl, fma(-K2, dun_lo + duo_lo, phlo));
      phhi       = fma(-K1, jh, fma(K2, duo_hi + dun_hi, phhi));
      dlo        = K2 * jl;
      dhi        = K2 * jh;
    }
  if constexpr (VISC && N >= 5)
    {
      // (1 - skew) sa Dw (vt U) - nu Dw (D U) + lifts of values and
      // derivatives on the even-odd recombination - skew sa vt D U
      const T sk  = A.has_skew ? Consts<T>::skew(A) : T(0);
      const T adv = (T(1) - sk) * sa;
      const T cd  = Consts<T>::cdiff(A, D);
      T       w[N], du[N];
      sweep2<N, T, true>(tb.D, tb.D_eo, U, du);
#pragma unroll
      for (int q = 0; q < N; ++q)
        w[q] = fma(adv, vt[q * vstride] * U[q], -cd * du[q]);
      sweep_eo_anti_lift<N, T, true>(tb.Dw_eo, w, phlo, phhi, tb.lwe, tb.lwo, out, dlo, dhi, tb.lde, tb.ldo);
      if (A.has_skew)
        {
#pragma unroll
          for (int q = 0; q < N; ++q)
            out[q] = fma(-sk * sa, vt[q * vstride] * du[q], out[q]);
        }
      return;
    }
  T vtv[N], w[N], du[N];
  const bool need_du = VISC || A.has_skew;
  if (need_du)
    sweep2<N, T, true>(tb.D, tb.D_eo, U, du);
  const T sk  = A.has_skew ? Consts<T>::skew(A) : T(0);
  const T adv = VISC ? (T(1) - sk) * sa : T(1) - sk;
#pragma unroll
  for (int q = 0; q < N; ++q)
    {
      vtv[q] = UNI ? T(1) : vt[q * vstride];
      w[q]   = UNI ? U[q] : vtv[q] * U[q];
      if (VISC)
        w[q] = fma(adv, w[q], -Consts<T>::cdiff(A, D) * du[q]);
    }
  sweep2<N, T, true>(tb.Dw, tb.Dw_eo, w, out);
  if (A.has_skew)
    {
#pragma unroll
      for (int q = 0; q < N; ++q)
        out[q] = VISC ? fma(-sk * sa, vtv[q] * du[q], out[q])
                      : fma(T(1) - sk, out[q], -sk * (UNI ? du[q] : vtv[q] * du[q]));
    }
  const T cv = Consts<T>::cv(A, D);
#pragma unroll
  for (int q = 0; q < N; ++q)
    {
      T o = UNI ? cv * out[q] : out[q];
      o   = fma(tb.lw0[q], phlo, o);
      o   = fma(tb.lw1[q], phhi, o);
      if (VISC)
        {
          o = fma(tb.lwd0[q], dlo, o);
          o = fma(tb.lwd1[q], dhi, o);
        }
      out[q] = o;
    }
}

template <int N, typename T, bool UNI, bool VISC, int D, bool OWN_TR = false>
__device__ __forceinline__ void direction_pass(const StageArgs &A, const DevTables<T> &tb,
                                               const T (&U)[N], T nlo, T nhi, T dnlo, T dnhi, bool blo,
                                               bool bhi, int fq, const T *Flo, const T *Fhi, const T *vt,
                                               int vstride, T (&out)[N], T tr_lo = T(0), T tr_hi = T(0),
                                               T dtr_lo = T(0), T dtr_hi = T(0))
{
  direction_pass_pm<N, T, UNI, VISC, D, OWN_TR>(A, tb, U, nlo, nhi, dnlo, dnhi, blo, bhi,
                                                face_pm<T, UNI, D>(A, Flo, Fhi, fq), vt, vstride, out, tr_lo,
                                                tr_hi, dtr_lo, dtr_hi);
}

// Neighbour cells (-1 on boundary faces) and face ids of the cells
// cell0 .. cell0 + ncell - 1: s_nbr / s_face [cell][6] with faces ordered
// (x low, x high, y low, y high, z low, z high).
__device__ __forceinline__ void cell_neighbours(const StageArgs &A, long long cell0, int ncell, int *s_nbr,
                                                int *s_face, int tid, int nthreads)
{
  for (int i = tid; i < ncell * 6; i += nthreads)
    {
      const int       cl = i / 6, j = i % 6, d = j >> 1, s = j & 1;
      const long long c  = cell0 + cl;
      const int       nx = A.nc[0], ny = A.nc[1], nz = A.nc[2];
      const int       ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((long long)nx * ny));
      // coordinate along d, its extent, and the sorted tangential coordinates
      const int id  = d == 0 ? ix : d == 1 ? iy : iz;
      const int nd  = d == 0 ? nx : d == 1 ? ny : nz;
      const int j1  = d == 0 ? iy : ix;
      const int j2  = d == 2 ? iy : iz;
      const int n1  = d == 0 ? ny : nx;
      const int npd = d == 0 ? A.npos[0] : d == 1 ? A.npos[1] : A.npos[2];
      const bool wrap = (A.periodic >> d) & 1;
      int        pos  = id + s;
      if (wrap && pos == nd)
        pos = 0;
      s_face[i] = pos + npd * (j1 + n1 * j2);
      int nb    = id + (s ? 1 : -1);
      if (wrap)
        nb = (nb + nd) % nd;
      if (nb < 0 || nb >= nd)
        s_nbr[i] = -1;
      else
        {
          const int jx = d == 0 ? nb : ix, jy = d == 1 ? nb : iy, jz = d == 2 ? nb : iz;
          s_nbr[i] = (int)(jx + (long long)nx * (jy + (long long)ny * jz));
        }
    }
}

// Field case: asynchronous copies of the cell geometry (16-byte chunks) and
// the face coefficients (8-byte chunks) into shared memory, committed as one
// group; the caller waits with __pipeline_wait_prior(0) before using them.
template <int N, typename T>
__device__ __forceinline__ void geometry_async(const StageArgs &A, long long cell0, int ncell, const int *s_face,
                                               T *Gb, T *Fb, int tid, int nthreads, bool faces = true,
                                               bool cells = true)
{
  constexpr int NQ  = N * N * N;
  constexpr int NF  = N * N;
  const char   *geo = reinterpret_cast<const char *>(static_cast<const T *>(A.cell_geo) + cell0 * 4 * NQ);
  const int     n16 = cells ? ncell * 4 * NQ * (int)sizeof(T) / 16 : 0;
  for (int i = tid; i < n16; i += nthreads)
    __pipeline_memcpy_async(reinterpret_cast<char *>(Gb) + 16 * i, geo + 16 * i, 16);
  constexpr int F8 = 2 * NF * (int)sizeof(T) / 8; // 8-byte chunks per cell-face
  for (int i = tid; faces && i < ncell * 6 * F8; i += nthreads)
    {
      const int cf = i / F8, e = i % F8;
      const int d  = (cf % 6) >> 1;
      const T  *F  = static_cast<const T *>(d == 0 ? A.face_geo[0] : d == 1 ? A.face_geo[1] : A.face_geo[2]);
      __pipeline_memcpy_async(reinterpret_cast<char *>(Fb + cf * 2 * NF) + 8 * e,
                              reinterpret_cast<const char *>(F + (size_t)s_face[cf] * 2 * NF) + 8 * e, 8);
    }
  __pipeline_commit();
}

// One CTA's work: cells cell0 .. cell0 + C - 1 of the mesh described by A,
// with the dynamic shared memory of the launch.  Shared by the single-mesh
// kernel and the batched multi-mesh kernel of the serving loop.
template <int N, typename T, bool UNI, bool VISC>
__device__ __forceinline__ void stage_cta(const StageArgs &A, const long long cell0, unsigned char *smem_raw)
{
  using SH         = StageShape<N, T, UNI, VISC>;
  constexpr int C  = SH::C;
  constexpr int NQ = SH::NQ;
  constexpr int NF = SH::NF;
  constexpr int NT = SH::THREADS;
  T   *Ub     = reinterpret_cast<T *>(smem_raw); // [C][NQ] nodal -> Gauss values
  T   *Qb     = Ub + C * NQ;                     // [C][NQ] accumulated Z, then k
  T   *Nb     = Qb + C * NQ;                     // [C][6][NF] neighbour face values
  T   *Gb     = Nb + C * 6 * NF;                 // field: [C][4][NQ] cell geometry
  constexpr bool FG = SH::FACES_GLOBAL;
  T   *Fb     = Gb + (UNI ? 0 : C * 4 * NQ);     // field: [C][6][2][NF] face coefficients (staged unless FG)
  T   *Nd     = Fb + (UNI || FG ? 0 : C * 12 * NF); // viscous: [C][6][NF] neighbour normal derivatives
  int *s_nbr  = reinterpret_cast<int *>(Nd + (VISC ? C * 6 * NF : 0)); // [C][6] neighbour or -1
  int *s_face = s_nbr + C * 6;                                          // [C][6] face id

  const DevTables<T> &tb    = tab<T>(N);
  const int           tid   = threadIdx.x;
  const int           ncell = (int)min((long long)C, A.n_cells - cell0);

  // ---- phase 0a: neighbour cells and face ids of the CTA's cells; the
  //      binary32 operator also asks L2 for the CTA's range of u_in, which
  //      the update reads only after the seven barriers of the stage
  if (sizeof(T) == sizeof(float) && A.u_in && (A.mode == kModeStage || A.mode == kModeLastStage))
    {
      const char *ub    = reinterpret_cast<const char *>(A.u_in + cell0 * NQ);
      const int   lines = (ncell * NQ * (int)sizeof(double) + 127) / 128;
      for (int i = tid; i < lines; i += NT)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(ub + 128 * i));
    }
  cell_neighbours(A, cell0, ncell, s_nbr, s_face, tid, NT);
  __syncthreads();

  // ---- phase 0b: curved meshes / variable velocity: start the asynchronous
  //      copies of the geometry; they land while the sweeps below run
  if (!UNI)
    geometry_async<N, T>(A, cell0, ncell, s_face, Gb, Fb, tid, NT, !FG);
  // face coefficients, (P, M) pairs, of face j of local cell cl: staged or global
  auto faces = [&](int cl, int j) -> const T * {
    if (FG)
      {
        const int d = j >> 1;
        const T  *F = static_cast<const T *>(d == 0 ? A.face_geo[0] : d == 1 ? A.face_geo[1] : A.face_geo[2]);
        return F + (size_t)s_face[cl * 6 + j] * 2 * NF;
      }
    return Fb + (cl * 6 + j) * 2 * NF;
  };

  // ---- phase 1: own values loaded as z-pencils and interpolated along z;
  //      neighbour face layers loaded as rows along their first tangential
  //      direction and interpolated along it
  {
    const double *src = A.r_in + cell0 * NQ;
    for (int w = tid; w < ncell * NF; w += NT)
      {
        const int     cl = w / NF, r = w % NF;
        const double *g  = src + cl * NQ + r;
        T             in[N], out[N];
#pragma unroll
        for (int k = 0; k < N; ++k)
          in[k] = from_double<T>(__ldg(g + k * NF));
        sweep2<N, T, false>(tb.S, tb.S_eo, in, out);
        T *p = Ub + cl * NQ + r;
#pragma unroll
        for (int k = 0; k < N; ++k)
          p[k * NF] = out[k];
      }
    for (int w = tid; w < ncell * 6 * N; w += NT)
      {
        const int cf = w / N, b = w % N;
        const int nb = s_nbr[cf];
        if (nb < 0)
          continue; // boundary face: phase 2 writes the Dirichlet data
        const int j = cf % 6, d = j >> 1, layer = (j & 1) ? 0 : N - 1;
        // nodal index of (layer along d, a along t1, b along t2) = base + a * stride
        const int     base   = d == 0 ? layer + NF * b : d == 1 ? N * layer + NF * b : N * b + NF * layer;
        const int     stride = d == 0 ? N : 1;
        const double *g      = A.r_in + (long long)nb * NQ + base;
        T             in[N], out[N];
        if (!VISC)
          {
#pragma unroll
            for (int a = 0; a < N; ++a)
              in[a] = from_double<T>(__ldg(g + a * stride));
          }
        else
          {
            // whole pencils through the neighbour along d: the face value and
            // the reference normal derivative at the face (xi_d = 1 for the
            // neighbour below, 0 for the one above)
            const int     sd   = d == 0 ? 1 : d == 1 ? N : NF;
            const double *g0   = g - layer * sd;
            const T      *dphi = (j & 1) ? tb.dphi0 : tb.dphi1;
            T             der[N], dout[N];
#pragma unroll
            for (int a = 0; a < N; ++a)
              {
                T v[N];
#pragma unroll
                for (int i = 0; i < N; ++i)
                  v[i] = from_double<T>(__ldg(g0 + a * stride + i * sd));
                in[a] = v[layer];
                T dv  = dphi[0] * v[0];
#pragma unroll
                for (int i = 1; i < N; ++i)
                  dv = fma(dphi[i], v[i], dv);
                der[a] = dv;
              }
            sweep2<N, T, false>(tb.S, tb.S_eo, der, dout);
            T *pd = Nd + cf * NF + N * b;
#pragma unroll
            for (int a = 0; a < N; ++a)
              pd[a] = dout[a];
          }
        sweep2<N, T, false>(tb.S, tb.S_eo, in, out);
        T *p = Nb + cf * NF + N * b;
#pragma unroll
        for (int a = 0; a < N; ++a)
          p[a] = out[a];
      }
  }
  __syncthreads();

  // ---- phase 2: S along y; neighbour layers along the second tangential
  //      direction, or Dirichlet data on boundary faces
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int r = w % NF;
      T        *p = Ub + (w / NF) * NQ + (r % N) + NF * (r / N);
      T         in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * N];
      sweep2<N, T, false>(tb.S, tb.S_eo, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k * N] = out[k];
    }
  for (int w = tid; w < ncell * 6 * N; w += NT)
    {
      const int cf = w / N, q1 = w % N;
      T        *p  = Nb + cf * NF + q1;
      if (s_nbr[cf] >= 0)
        {
          T in[N], out[N];
#pragma unroll
          for (int k = 0; k < N; ++k)
            in[k] = p[k * N];
          sweep2<N, T, false>(tb.S, tb.S_eo, in, out);
#pragma unroll
          for (int k = 0; k < N; ++k)
            p[k * N] = out[k];
          if (VISC)
            {
              T *pd = Nd + cf * NF + q1;
#pragma unroll
              for (int k = 0; k < N; ++k)
                in[k] = pd[k * N];
              sweep2<N, T, false>(tb.S, tb.S_eo, in, out);
#pragma unroll
              for (int k = 0; k < N; ++k)
                pd[k * N] = out[k];
            }
        }
      else
        {
          const int d = (cf % 6) >> 1;
          for (int k = 0; k < N; ++k)
            {
              double g = 0.0;
              if (A.bc_exact)
                {
                  const double *fx = d == 0 ? A.face_x[0] : d == 1 ? A.face_x[1] : A.face_x[2];
                  const double *x  = fx + ((size_t)s_face[cf] * NF + q1 + N * k) * 3;
                  g                = exact_value(A.ex, x[0], x[1], x[2], A.t);
                }
              p[k * N] = from_double<T>(g);
            }
        }
    }
  if (!UNI)
    __pipeline_wait_prior(0);
  __syncthreads();

  // ---- phase 3: S along x gives the Gauss-point values; x-direction terms
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      T        *p  = Ub + cl * NQ + N * r;
      T         in[N], U[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k];
      sweep2<N, T, false>(tb.S, tb.S_eo, in, U);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k] = U[k];
      const T *F = faces(cl, 0), *Fh = faces(cl, 1);
      direction_pass<N, T, UNI, VISC, 0>(A, tb, U, Nb[(cl * 6 + 0) * NF + r], Nb[(cl * 6 + 1) * NF + r],
                                         VISC ? Nd[(cl * 6 + 0) * NF + r] : T(0),
                                         VISC ? Nd[(cl * 6 + 1) * NF + r] : T(0),
                                         s_nbr[cl * 6 + 0] < 0, s_nbr[cl * 6 + 1] < 0, r,
                                   F, Fh, Gb + cl * 4 * NQ + N * r, 1, out);
      T *z = Qb + cl * NQ + N * r;
#pragma unroll
      for (int k = 0; k < N; ++k)
        z[k] = out[k];
    }
  __syncthreads();

  // ---- phase 4: y-direction terms
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const int off = (r % N) + NF * (r / N);
      const T  *p   = Ub + cl * NQ + off;
      T         U[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        U[k] = p[k * N];
      const T *F = faces(cl, 2), *Fh = faces(cl, 3);
      direction_pass<N, T, UNI, VISC, 1>(A, tb, U, Nb[(cl * 6 + 2) * NF + r], Nb[(cl * 6 + 3) * NF + r],
                                         VISC ? Nd[(cl * 6 + 2) * NF + r] : T(0),
                                         VISC ? Nd[(cl * 6 + 3) * NF + r] : T(0),
                                         s_nbr[cl * 6 + 2] < 0, s_nbr[cl * 6 + 3] < 0, r,
                                   F, Fh, Gb + (cl * 4 + 1) * NQ + off, N, out);
      T *z = Qb + cl * NQ + off;
#pragma unroll
      for (int k = 0; k < N; ++k)
        z[k * N] += out[k];
    }
  __syncthreads();

  // ---- phase 5: z-direction terms, 1/det J, S^-1 along z
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const T  *p  = Ub + cl * NQ + r;
      T         U[N], out[N], zz[N], kk[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        U[k] = p[k * NF];
      const T *F = faces(cl, 4), *Fh = faces(cl, 5);
      const T *G = Gb + cl * 4 * NQ;
      direction_pass<N, T, UNI, VISC, 2>(A, tb, U, Nb[(cl * 6 + 4) * NF + r], Nb[(cl * 6 + 5) * NF + r],
                                         VISC ? Nd[(cl * 6 + 4) * NF + r] : T(0),
                                         VISC ? Nd[(cl * 6 + 5) * NF + r] : T(0),
                                         s_nbr[cl * 6 + 4] < 0, s_nbr[cl * 6 + 5] < 0, r,
                                   F, Fh, G + 2 * NQ + r, NF, out);
      T *z = Qb + cl * NQ + r;
      if (A.mode != kModeVmult)
        {
#pragma unroll
          for (int k = 0; k < N; ++k)
            {
              zz[k] = z[k * NF] + out[k];
              if (!UNI)
                zz[k] *= G[3 * NQ + r + k * NF];
            }
          sweep2<N, T, false>(tb.Si, tb.Si_eo, zz, kk);
        }
      else
        {
          // implicit operator in weak form: S^T [JxW (c U - Z)], with
          // JxW Z = w B (field) or w V B (uniform) for the bracket B
          const T cm = Consts<T>::mass(A), sc = Consts<T>::out(A);
          const T wxy = tb.gw[r % N] * tb.gw[r / N];
#pragma unroll
          for (int k = 0; k < N; ++k)
            {
              const T bracket = sc * (z[k * NF] + out[k]);
              const T wq      = wxy * tb.gw[k];
              zz[k] = UNI ? wq * Consts<T>::vol(A) * (cm * U[k] - bracket)
                          : wq * (cm * U[k] / G[3 * NQ + r + k * NF] - bracket);
            }
          sweep2<N, T, false>(tb.St, tb.St_eo, zz, kk);
        }
#pragma unroll
      for (int k = 0; k < N; ++k)
        z[k * NF] = kk[k];
    }
  __syncthreads();

  // ---- phase 6: S^-1 along y
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int r = w % NF;
      T        *p = Qb + (w / NF) * NQ + (r % N) + NF * (r / N);
      T         in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k * N];
      if (A.mode != kModeVmult)
        sweep2<N, T, false>(tb.Si, tb.Si_eo, in, out);
      else
        sweep2<N, T, false>(tb.St, tb.St_eo, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k * N] = out[k];
    }
  __syncthreads();

  // ---- phase 7: S^-1 along x
  for (int w = tid; w < ncell * NF; w += NT)
    {
      T *p = Qb + (w / NF) * NQ + N * (w % NF);
      T  in[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        in[k] = p[k];
      if (A.mode != kModeVmult)
        sweep2<N, T, false>(tb.Si, tb.Si_eo, in, out);
      else
        sweep2<N, T, false>(tb.St, tb.St_eo, in, out);
#pragma unroll
      for (int k = 0; k < N; ++k)
        p[k] = out[k];
    }
  __syncthreads();

  // ---- phase 8: Runge-Kutta update over the CTA's contiguous DoF range
  //      (the post-operation lambda of advection_solver.cc:728-752)
  const long long g0 = cell0 * NQ;
  if (A.mode == kModeVmult)
    {
      for (int i = tid; i < ncell * NQ; i += NT)
        A.r_out[g0 + i] = to_double<T>(Qb[i]);
    }
  else if (A.mode == kModeApply)
    {
      for (int i = tid; i < ncell * NQ; i += NT)
        A.r_out[g0 + i] = A.out_scale * to_double<T>(Qb[i]);
    }
  else if (A.mode == kModeStage)
    {
      for (int i = tid; i < ncell * NQ; i += NT)
        {
          double kd = to_double<T>(Qb[i]);
          if (A.k_add)
            kd += __ldcs(A.k_add + g0 + i);
          const double u  = A.u_in ? __ldcs(A.u_in + g0 + i) : 0.0;
          A.u_out[g0 + i] = fma(A.b, kd, u);
          A.r_out[g0 + i] = fma(A.a, kd, u);
          if (A.k_out)
            A.k_out[g0 + i] = kd;
        }
    }
  else
    {
      for (int i = tid; i < ncell * NQ; i += NT)
        {
          double kd = to_double<T>(Qb[i]);
          if (A.k_add)
            kd += __ldcs(A.k_add + g0 + i);
          double v = fma(A.b, kd, __ldcs(A.u_in + g0 + i));
          if (A.u_base)
            v += A.u_base[g0 + i];
          A.u_out[g0 + i] = v;
        }
    }
}

template <int N, typename T, bool UNI, bool VISC>
__global__ void __launch_bounds__(StageShape<N, T, UNI, VISC>::THREADS)
  stage_kernel(const StageArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_cta<N, T, UNI, VISC>(A, A.cell_begin + (long long)blockIdx.x * StageShape<N, T, UNI, VISC>::C, smem_raw);
}

template <int N, typename T, bool UNI, bool VISC>
cudaError_t launch_stage_t(const StageArgs &args, cudaStream_t stream)
{
  using SH = StageShape<N, T, UNI, VISC>;
  // the shared-memory opt-in is a per-device function attribute
  static std::atomic<unsigned long long> configured{0};
  cudaError_t                            e = opt_in_smem(stage_kernel<N, T, UNI, VISC>, SH::SMEM, configured);
  if (e != cudaSuccess)
    return e;
  const long long blocks = (args.n_cells - args.cell_begin + SH::C - 1) / SH::C;
  stage_kernel<N, T, UNI, VISC><<<(unsigned)blocks, SH::THREADS, SH::SMEM_NODAL, stream>>>(args);
  return cudaGetLastError();
}

template <int N, typename T>
cudaError_t launch_stage_n(const StageArgs &args, cudaStream_t stream)
{
  if (args.visc)
    return launch_stage_t<N, T, false, true>(args, stream);
  return args.uniform ? launch_stage_t<N, T, true, false>(args, stream)
                      : launch_stage_t<N, T, false, false>(args, stream);
}

template <int N, typename T>
int stage_cells()
{
  return StageShape<N, T, true>::C;
}
} // namespace adv
