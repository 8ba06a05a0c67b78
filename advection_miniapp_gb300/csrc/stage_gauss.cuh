// Fused DG advection stage in collocation form for sm_103a.
//
// The vectors hold, per cell, the values at the (k+1)^3 Gauss points: the
// nodal basis of the Lagrange polynomials on the Gauss points spans the same
// space as the reference's FE_DGQ basis on Gauss-Lobatto nodes, and the two
// coefficient vectors are related by U = (S x S x S) u.  In this basis the
// stage of the nodal kernel (stage_kernel.cuh) loses its interpolation and
// inverse-mass sweeps:
//   Z = idet * [ sum_d Dw_d (vt_d . U) + sum_faces lw(s) phi ]
// is already the Gauss-point representation of k = M^{-1} L(u)
// (advection_solver.cc:469-657), because M^{-1} = S^{-1} diag(1/JxW) S^{-T}
// and the S^{-T} cancels against the transposed interpolation of the
// integration.  Face values of a neighbour are contractions of its pencil
// through the face point with its Lagrange basis at the shared face, so each
// cell reads whole neighbour cells (n^3 values, from L2) instead of their
// Gauss-Lobatto face layers.  Per cell and stage at degree 4 this removes 6 of
// the 9 n^4 sweeps and replaces the 2D interpolation of the neighbour layers
// by n^3 contractions: about 4.9k instead of 8.4k FP64 instructions.
//
// The fused LSRK loop changes the basis of the solution once on entry and
// once on exit (launch_basis_change); the stages in between run here.
//
// Face traces (TR, FP64): a stage also writes the values at the face points
// of its output that the next stage reads (r_out, or u_out on a last stage),
// [6][n^2] per cell, and with SIPG also the reference normal derivatives
// there ([6][2][n^2]); the next stage then reads its own and its neighbours'
// face data, one global read per face point in the direction passes,
// instead of contracting pencils.  Per cell-stage at degree 4 the producer
// adds 750 FMAs and the consumer saves 1500; the traces are the same
// contractions in the same order, so results are bit-identical to the
// variant without them.
#pragma once

#include "stage_kernel.cuh"

namespace adv
{
template <int N, typename T, bool UNI, bool VISC, bool TR>
struct GaussShape
{
  using SH                     = StageShape<N, T, UNI, VISC>;
  static constexpr int C       = SH::C;
  static constexpr int THREADS = SH::THREADS;
  // traces per face point: the value, and with SIPG the reference normal derivative
  static constexpr int TRW = VISC ? 2 : 1;
  // TG: traces read from global memory in the direction passes, one read per
  // face point, instead of being staged (field geometry without SIPG, where
  // shared memory limits the resident CTAs: 12 C n^2 values less per CTA,
  // 7 instead of 5 CTAs per SM in FP64 at degree 4, 2.2 % faster on GB300);
  // the other variants are limited by registers and stage them
  static constexpr bool TG = TR && !UNI && !VISC;
  // staged: neighbour values Nb [C][6][NF], own traces Tb [C][6][TRW][NF],
  // padded so that the cell geometry Gb after them starts on 16 bytes (it is
  // filled by 16-byte cp.async)
  static constexpr int NB_VALUES = TG ? 0 : 6 * C * N * N;
  static constexpr int TB_VALUES =
    ((2 * C * N * N * N + NB_VALUES + (TR && !TG ? TRW * 6 * C * N * N : 0)) * (int)sizeof(T) + 15) / 16 * 16 /
      (int)sizeof(T) -
    (2 * C * N * N * N + NB_VALUES);
  // field geometry with traces: the face coefficients are read from global
  // memory in the direction passes (one read per face point) instead of being
  // staged, which frees 12 C n^2 values of shared memory per CTA.
  // Cell geometry [vt0|vt1|vt2|idet] read from global memory in the passes
  // (one read per point and direction) instead of staged by cp.async:
  // with SIPG (staged it would take 4 C n^3 + 12 C n^2 values, at degree 5 in
  // FP64 72 KB of a 145 KB CTA: +15 % FP64, +19 % FP32) and in the FP64
  // kernel with traces (the CTA starts its passes without waiting for 20 KB
  // of geometry: +3.6 % on 64^3 curved cells of degree 4 at 7 CTAs per SM).
  // The other advection kernels keep staging it (measured 7 % / 4 % slower
  // without).
  static constexpr bool GEO_GLOBAL   = VISC || (TR && !UNI && sizeof(T) == sizeof(double));
  static constexpr bool FACES_GLOBAL = !UNI && (TR || VISC || sizeof(T) == sizeof(float));
  static constexpr int  FB_VALUES    = UNI || FACES_GLOBAL ? 0 : 12 * C * N * N;
  static constexpr int  GB_VALUES    = UNI || GEO_GLOBAL ? 0 : 4 * C * N * N * N;
  // viscous: Nd [C][6][NF] neighbour normal derivatives
  static constexpr int  ND_VALUES    = VISC ? 6 * C * N * N : 0;
  // upwind traces (StageArgs::upwind_tr): per face point of the CTA's cells
  // whether its own trace there is read, one byte each, then a count and a
  // list of the pencils whose high trace is deferred (at most 3 C n^2)
  static constexpr int  NEED_FLAGS   = (6 * C * N * N + 3) / 4 * 4;
  static constexpr int  NEED_BYTES   = TG ? NEED_FLAGS + 4 * (1 + 3 * C * N * N) : 0;
  static constexpr int  SMEM         = (2 * C * N * N * N + NB_VALUES + TB_VALUES + GB_VALUES + FB_VALUES + ND_VALUES) *
                                    (int)sizeof(T) + 12 * C * (int)sizeof(int) + NEED_BYTES;
  // byte offset of the cell geometry Gb in the layout of stage_gauss_cta
  static constexpr int GB_OFFSET = (2 * C * N * N * N + NB_VALUES + TB_VALUES) * (int)sizeof(T);
  static_assert(GB_OFFSET % 16 == 0, "cp.async destinations need 16-byte alignment");
};

__device__ __forceinline__ double or_bits(double a, double b)
{
  return __longlong_as_double(__double_as_longlong(a) | __double_as_longlong(b));
}
__device__ __forceinline__ float or_bits(float a, float b)
{
  return __int_as_float(__float_as_int(a) | __float_as_int(b));
}
// x != 0 on the integer pipe (a floating-point comparison of doubles issues
// on the FP64 pipe, the kernel's bottleneck)
__device__ __forceinline__ bool nonzero(double x)
{
  return (__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFll) != 0;
}
__device__ __forceinline__ bool nonzero(float x)
{
  return (__float_as_int(x) & 0x7FFFFFFF) != 0;
}

// Upwind traces of a pencil x: the trace at the face whose flux reads it
// (need_lo / need_hi; the low one where neither is read), one contraction
// with the coefficients of either face picked per thread (a pointer into
// the tables, so a warp whose pencils need different faces runs one chain),
// the same sum in the same order as pencil_traces.  Returns whether the
// high trace is read as well (a diverging flow at a point of a curved cell,
// rare): the caller defers that one.
template <int N, typename T>
__device__ __forceinline__ bool upwind_pencil_traces(const DevTables<T> &tb, const T (&x)[N], bool need_lo,
                                                     bool need_hi, T *to_lo, T *to_hi)
{
  const bool lo = need_lo || !need_hi;
  const T   *c  = lo ? tb.l0 : tb.l1;
  T          s  = c[0] * x[0];
#pragma unroll
  for (int q = 1; q < N; ++q)
    s = fma(c[q], x[q], s);
  *(lo ? to_lo : to_hi) = s;
  return need_lo && need_hi;
}

// INC: FP32 increments with the anchor's K0 folded out (StageArgs::inc32).
// Binary32 operator: the input comes from r_in32 and the update is the
// increment form's.  FP64 operator: the block's anchor (writes K0 and the
// first G).
template <int N, typename T, bool UNI, bool VISC, bool TR = false, bool INC = false, bool UPW = false>
__device__ __forceinline__ void stage_gauss_cta(const StageArgs &A, const long long cell0,
                                                unsigned char *smem_raw)
{
  using SH         = StageShape<N, T, UNI, VISC>;
  constexpr int C  = SH::C;
  constexpr int NQ = SH::NQ;
  constexpr int NF = SH::NF;
  constexpr int NT = SH::THREADS;
  T   *Ub     = reinterpret_cast<T *>(smem_raw); // [C][NQ] Gauss-point values of r_in
  T   *Qb     = Ub + C * NQ;                     // [C][NQ] x and y contributions to Z
  using GS                 = GaussShape<N, T, UNI, VISC, TR>;
  constexpr bool FG        = GS::FACES_GLOBAL;
  constexpr int  TRW       = GS::TRW;
  constexpr bool TG        = GS::TG;
  T   *Nb     = Qb + C * NQ;                     // staged: [C][6][NF] neighbour values at the face points
  T   *Tb     = Nb + GS::NB_VALUES;              // staged traces: [C][6][TRW][NF] own values (and derivatives)
  T   *Gb     = Tb + GS::TB_VALUES;              // field: [C][4][NQ] cell geometry
  T   *Fb     = Gb + GS::GB_VALUES;              // field: [C][6][2][NF] face coefficients (staged unless FG)
  T   *Nd     = Fb + GS::FB_VALUES;              // viscous: [C][6][NF] neighbour normal derivatives
  int *s_nbr  = reinterpret_cast<int *>(Nd + GS::ND_VALUES);
  int *s_face = s_nbr + C * 6;
  unsigned char *s_need = reinterpret_cast<unsigned char *>(s_face + C * 6); // upwind traces: [C][6][NF]
  int *s_nboth = reinterpret_cast<int *>(s_need + GS::NEED_FLAGS);           // deferred high traces: count,
  int *s_both  = s_nboth + 1;                                                 // [3 C NF] (d C + cl) NF + r

  const DevTables<T> &tb    = tab<T>(N);
  const int           tid   = threadIdx.x;
  const int           ncell = (int)min((long long)C, A.n_cells - cell0);

  // binary32 operator: ask L2 for the CTA's ranges of u_in and k_add, read
  // by the update after the three passes
  if (sizeof(T) == sizeof(float) && (A.mode == kModeStage || A.mode == kModeLastStage))
    {
      const int lines = (ncell * NQ * (int)sizeof(double) + 127) / 128;
      for (int i = tid; i < 2 * lines; i += NT)
        {
          const double *base = i < lines ? A.u_in : A.k_add;
          if (base)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char *>(base + cell0 * NQ) +
                                                          128 * (i % lines)));
        }
      if (INC && sizeof(T) == sizeof(float) && A.k_add32)
        for (int i = tid; i < (ncell * NQ * (int)sizeof(float) + 127) / 128; i += NT)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char *>(A.k_add32 + cell0 * NQ) +
                                                        128 * i));
    }
  cell_neighbours(A, cell0, ncell, s_nbr, s_face, tid, NT);
  if (UPW && tid == 0)
    *s_nboth = 0;
  __syncthreads();
  if (!UNI && !(GS::GEO_GLOBAL && FG))
    geometry_async<N, T>(A, cell0, ncell, s_face, Gb, Fb, tid, NT, !FG, !GS::GEO_GLOBAL);
  // cell geometry [vt0 | vt1 | vt2 | idet] of local cell cl: staged or global
  auto geo = [&](int cl) -> const T * {
    if (GS::GEO_GLOBAL)
      return static_cast<const T *>(A.cell_geo) + (cell0 + cl) * 4 * NQ;
    return Gb + cl * 4 * NQ;
  };

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

  // ---- phase 1: own values (one contiguous range of the CTA's cells) and
  //      the neighbours' values at the face points
  {
    if (INC && sizeof(T) == sizeof(float))
      {
        const float *src = A.r_in32 + cell0 * NQ;
        for (int i = tid; i < ncell * NQ; i += NT)
          Ub[i] = T(__ldg(src + i));
      }
    else
      {
        // 16-byte loads of pairs of values (a first value alone when the
        // range starts off a 16-byte boundary, a last one when one is left)
        const double *src  = A.r_in + cell0 * NQ;
        const int     tot  = ncell * NQ;
        const int     head = (reinterpret_cast<uintptr_t>(src) & 15) ? 1 : 0;
        const int     np   = (tot - head) / 2;
        if (tid == 0 && head)
          Ub[0] = from_double<T>(__ldg(src));
        if (tid == 1 && head + 2 * np < tot)
          Ub[tot - 1] = from_double<T>(__ldg(src + tot - 1));
        const double2 *src2 = reinterpret_cast<const double2 *>(src + head);
        for (int i = tid; i < np; i += NT)
          {
            const double2 v      = __ldg(src2 + i);
            Ub[head + 2 * i]     = from_double<T>(v.x);
            Ub[head + 2 * i + 1] = from_double<T>(v.y);
          }
      }
    if (TR && !TG)
      {
        const T *tr = static_cast<const T *>(A.tr_in) + cell0 * 6 * TRW * NF;
        for (int i = tid; i < ncell * 6 * TRW * NF; i += NT)
          Tb[i] = __ldg(tr + i);
      }
  }
  // the neighbours' values at the face points: one thread per face point
  // position (cell, fq), the six faces unrolled (face, direction, stride and
  // basis known at compile time)
  auto neighbour_value = [&](int cl, int j, int fq) {
    const int cf = cl * 6 + j, d = j >> 1;
    const int nb = s_nbr[cf];
    if (nb >= 0)
      {
        if (TR)
          {
            // the neighbour's own trace on the shared face (its face j ^ 1)
            const T *tn      = static_cast<const T *>(A.tr_in) + ((long long)nb * 6 + (j ^ 1)) * TRW * NF + fq;
            Nb[cf * NF + fq] = __ldg(tn);
            if (VISC)
              Nd[cf * NF + fq] = __ldg(tn + NF);
            return;
          }
        // pencil of the neighbour along d through face point fq, contracted
        // with its basis at the shared face: xi_d = 1 for the neighbour
        // below (low face, j even), xi_d = 0 for the one above
        const T        *l   = (j & 1) ? tb.l0 : tb.l1;
        const int       sd  = d == 0 ? 1 : d == 1 ? N : NF;
        const long long off = (long long)nb * NQ + idx3<N>(d, 0, fq % N, fq / N);
        T               v[N];
        if (INC && sizeof(T) == sizeof(float))
          {
#pragma unroll
            for (int a = 0; a < N; ++a)
              v[a] = T(__ldg(A.r_in32 + off + a * sd));
          }
        else
          {
#pragma unroll
            for (int a = 0; a < N; ++a)
              v[a] = from_double<T>(__ldg(A.r_in + off + a * sd));
          }
        T s = l[0] * v[0];
#pragma unroll
        for (int a = 1; a < N; ++a)
          s = fma(l[a], v[a], s);
        Nb[cf * NF + fq] = s;
        if (VISC)
          {
            const T *ld = (j & 1) ? tb.ld0 : tb.ld1;
            T        ds = ld[0] * v[0];
#pragma unroll
            for (int a = 1; a < N; ++a)
              ds = fma(ld[a], v[a], ds);
            Nd[cf * NF + fq] = ds;
          }
      }
    else
      {
        double g = 0.0;
        if (A.bc_exact)
          {
            const double *fx = d == 0 ? A.face_x[0] : d == 1 ? A.face_x[1] : A.face_x[2];
            const double *x  = fx + ((size_t)s_face[cf] * NF + fq) * 3;
            g                = exact_value(A.ex, x[0], x[1], x[2], A.t);
          }
        Nb[cf * NF + fq] = from_double<T>(g);
      }
  };
  for (int w = tid; w < (TG ? 0 : ncell * NF); w += NT)
    {
      const int cl = w / NF, fq = w % NF;
#pragma unroll 1
      for (int d = 0; d < 3; ++d)
        {
          neighbour_value(cl, 2 * d, fq);
          neighbour_value(cl, 2 * d + 1, fq);
        }
    }
  if (!UNI)
    __pipeline_wait_prior(0);
  __syncthreads();

  // neighbour value and normal derivative at face point r of face j of local
  // cell cl: staged, or with traces the neighbour's own trace on the shared
  // face (its face j ^ 1), or the Dirichlet data on a boundary face
  const T *tr_in = static_cast<const T *>(A.tr_in);
  auto     nbv   = [&](int cl, int j, int r) -> T {
    if constexpr (!TG)
      return Nb[(cl * 6 + j) * NF + r];
    else
      {
        const int nb = s_nbr[cl * 6 + j];
        if (nb >= 0)
          return __ldg(tr_in + ((long long)nb * 6 + (j ^ 1)) * TRW * NF + r);
        double g = 0.0;
        if (A.bc_exact)
          {
            const int     d  = j >> 1;
            const double *fx = d == 0 ? A.face_x[0] : d == 1 ? A.face_x[1] : A.face_x[2];
            const double *x  = fx + ((size_t)s_face[cl * 6 + j] * NF + r) * 3;
            g                = exact_value(A.ex, x[0], x[1], x[2], A.t);
          }
        return from_double<T>(g);
      }
  };
  auto nbd = [&](int cl, int j, int r) -> T {
    if constexpr (!VISC)
      return T(0);
    else
      return Nd[(cl * 6 + j) * NF + r];
  };
  auto trv = [&](const T *p, int o) -> T {
    if constexpr (TG)
      return __ldg(p + o);
    else
      return p[o];
  };
  // own traces of face j (value, and with SIPG the normal derivative)
  auto own_tr = [&](int cl, int j) -> const T * {
    if constexpr (TG)
      return tr_in + ((cell0 + cl) * 6 + j) * TRW * NF;
    else
      return Tb + (cl * 6 + j) * TRW * NF;
  };
  // Upwind traces (UPW, a compile-time variant: a runtime switch between
  // the two forms costs registers): at a face point with P = 0 or M = 0 the
  // flux reads one side's trace, that of the upwind cell.  On a low face
  // (flux M u_own + P u_nbr) the cell reads its own trace where M != 0 and
  // its neighbour's where P != 0; on a high face (-(P u_own + M u_nbr)) its
  // own where P != 0 and the neighbour's where M != 0.  Both cells of a face
  // see the same pair, so a cell writes for the next stage exactly the
  // traces of its own that it or its neighbour reads, and the flux is the
  // nonzero coefficient times the value read: the same value as the general
  // form, one product instead of a product and an FMA.
  constexpr bool upw = UPW;
  static_assert(!UPW || (TG && !VISC), "upwind traces are read in the passes");
  // upwind traces at face point r of the low face j and high face j + 1 of
  // local cell cl: the nonzero coefficient of each face and the trace on
  // its upwind side, in the form direction_pass_pm<..., UPW> takes; returns
  // in own_lo / own_hi whether this cell's own trace is read there (M != 0 on
  // the low face, P != 0 on the high face), which is what the stage writes
  using T2           = typename std::conditional<sizeof(T) == sizeof(double), double2, float2>::type;
  auto upwind_values = [&](int cl, int j, int r, FacePM<T> &pm, T &vlo, T &vhi, bool &own_lo, bool &own_hi) {
    const T2 pl = *reinterpret_cast<const T2 *>(faces(cl, j) + 2 * r);
    const T2 ph = *reinterpret_cast<const T2 *>(faces(cl, j + 1) + 2 * r);
    const T *Tr = own_tr(cl, j) + r;
    own_lo      = nonzero(pl.y);
    own_hi      = nonzero(ph.x);
    // the nonzero one of P, M as the bitwise or of the two (the other is
    // +0: 0.5 (c -+ |c|) rounds to +0), so that the compiler does not split
    // the flux product into two predicated ones, one per side
    pm.Plo = or_bits(pl.x, pl.y);
    pm.Phi = or_bits(ph.x, ph.y);
    pm.Mlo = pm.Mhi = T(0);
    vlo             = nonzero(pl.x) ? nbv(cl, j, r) : own_lo ? trv(Tr, 0) : T(0);
    vhi             = own_hi ? trv(Tr, TRW * NF) : nonzero(ph.y) ? nbv(cl, j + 1, r) : T(0);
  };

  // ---- phase 2: x-direction terms
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const T  *p  = Ub + cl * NQ + N * r;
      T         U[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        U[k] = p[k];
      const T *Tr = TR ? own_tr(cl, 0) + r : nullptr;
      if constexpr (UPW)
        {
          FacePM<T> pm;
          T         vlo, vhi;
          bool      own_lo, own_hi;
          upwind_values(cl, 0, r, pm, vlo, vhi, own_lo, own_hi);
          s_need[(cl * 6 + 0) * NF + r] = own_lo;
          s_need[(cl * 6 + 1) * NF + r] = own_hi;
          direction_pass_pm<N, T, UNI, VISC, 0, true, true>(A, tb, U, vlo, vhi, T(0), T(0), false, false, pm,
                                                            geo(cl) + N * r, 1, out);
        }
      else
        direction_pass<N, T, UNI, VISC, 0, TR>(A, tb, U, nbv(cl, 0, r), nbv(cl, 1, r), nbd(cl, 0, r),
                                               nbd(cl, 1, r), s_nbr[cl * 6 + 0] < 0, s_nbr[cl * 6 + 1] < 0, r,
                                               faces(cl, 0), faces(cl, 1), geo(cl) + N * r, 1, out,
                                               TR ? trv(Tr, 0) : T(0), TR ? trv(Tr, TRW * NF) : T(0),
                                               TR && VISC ? trv(Tr, NF) : T(0),
                                               TR && VISC ? trv(Tr, TRW * NF + NF) : T(0));
      T *z = Qb + cl * NQ + N * r;
#pragma unroll
      for (int k = 0; k < N; ++k)
        z[k] = out[k];
    }
  __syncthreads();

  // ---- phase 3: y-direction terms
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const int off = (r % N) + NF * (r / N);
      const T  *p   = Ub + cl * NQ + off;
      T         U[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        U[k] = p[k * N];
      const T *Tr = TR ? own_tr(cl, 2) + r : nullptr;
      if constexpr (UPW)
        {
          FacePM<T> pm;
          T         vlo, vhi;
          bool      own_lo, own_hi;
          upwind_values(cl, 2, r, pm, vlo, vhi, own_lo, own_hi);
          s_need[(cl * 6 + 2) * NF + r] = own_lo;
          s_need[(cl * 6 + 3) * NF + r] = own_hi;
          direction_pass_pm<N, T, UNI, VISC, 1, true, true>(A, tb, U, vlo, vhi, T(0), T(0), false, false, pm,
                                                            geo(cl) + NQ + off, N, out);
        }
      else
        direction_pass<N, T, UNI, VISC, 1, TR>(A, tb, U, nbv(cl, 2, r), nbv(cl, 3, r), nbd(cl, 2, r),
                                               nbd(cl, 3, r), s_nbr[cl * 6 + 2] < 0, s_nbr[cl * 6 + 3] < 0, r,
                                               faces(cl, 2), faces(cl, 3), geo(cl) + NQ + off, N, out,
                                               TR ? trv(Tr, 0) : T(0), TR ? trv(Tr, TRW * NF) : T(0),
                                               TR && VISC ? trv(Tr, NF) : T(0),
                                               TR && VISC ? trv(Tr, TRW * NF + NF) : T(0));
      T *z = Qb + cl * NQ + off;
#pragma unroll
      for (int k = 0; k < N; ++k)
        z[k * N] += out[k];
    }
  __syncthreads();

  // ---- phase 4: z-direction terms, 1/det J, and the Runge-Kutta update of
  //      the pencil straight from registers
  for (int w = tid; w < ncell * NF; w += NT)
    {
      const int cl = w / NF, r = w % NF;
      const T  *p  = Ub + cl * NQ + r;
      T         U[N], out[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        U[k] = p[k * NF];
      const T *G  = geo(cl);
      const T *Tr  = TR ? own_tr(cl, 4) + r : nullptr;
      bool     zlo = false, zhi = false; // the z traces this pencil writes (upwind traces)
      if constexpr (UPW)
        {
          FacePM<T> pm;
          T         vlo, vhi;
          upwind_values(cl, 4, r, pm, vlo, vhi, zlo, zhi);
          direction_pass_pm<N, T, UNI, VISC, 2, true, true>(A, tb, U, vlo, vhi, T(0), T(0), false, false, pm,
                                                            G + 2 * NQ + r, NF, out);
        }
      else
        direction_pass<N, T, UNI, VISC, 2, TR>(A, tb, U, nbv(cl, 4, r), nbv(cl, 5, r), nbd(cl, 4, r),
                                               nbd(cl, 5, r), s_nbr[cl * 6 + 4] < 0, s_nbr[cl * 6 + 5] < 0, r,
                                               faces(cl, 4), faces(cl, 5), G + 2 * NQ + r, NF, out,
                                               TR ? trv(Tr, 0) : T(0), TR ? trv(Tr, TRW * NF) : T(0),
                                               TR && VISC ? trv(Tr, NF) : T(0),
                                               TR && VISC ? trv(Tr, TRW * NF + NF) : T(0));
      T              *z  = Qb + cl * NQ + r;
      const long long gb = (cell0 + cl) * NQ + r;
      double          next[N]; // the next stage's input along the pencil (traces)
#pragma unroll
      for (int k = 0; k < N; ++k)
        {
          T zz = z[k * NF] + out[k];
          const long long gi = gb + k * NF;
          // (the implicit solver runs the FP64 operator without traces; the
          // other variants do not carry this branch and its registers)
          if (!TR && !INC && sizeof(T) == sizeof(double) && A.mode == kModeVmult)
            {
              // implicit operator in weak form on the Gauss-point basis (dual
              // coefficients, the rows of the Lagrange functions on the Gauss
              // points): JxW (c U - L-bracket), the bracket taken before the
              // inverse Jacobian determinant; JxW = w / idet (field) or w V
              // (uniform)
              const T wq = tb.gw[r % N] * tb.gw[r / N] * tb.gw[k];
              const T br = Consts<T>::out(A) * zz;
              const T cm = Consts<T>::mass(A);
              const T v  = UNI ? wq * Consts<T>::vol(A) * (cm * U[k] - br)
                               : wq * (cm * U[k] / G[3 * NQ + r + k * NF] - br);
              A.r_out[gi] = to_double<T>(v);
              next[k]     = 0.0;
              continue;
            }
          if (!UNI)
            zz *= G[3 * NQ + r + k * NF];
          double          kd = to_double<T>(zz);
          if (INC)
            {
              // FP32 increments with the anchor's K0 folded out
              next[k] = 0.0;
              if constexpr (sizeof(T) == sizeof(double))
                {
                  // the block's FP64 anchor on u_a: K0 and the first G
                  A.k_out[gi]   = kd;
                  A.k_out32[gi] = d2f_int(kd);
                  A.r_out32[gi] = d2f_int(A.a * kd);
                }
              else if (A.mode == kModeStage)
                {
                  const double e = A.u_in ? __ldcs(A.u_in + gi) : 0.0;
                  A.u_out[gi]    = fma(A.b, kd, e);
                  A.r_out32[gi]  = fmaf(A.inc_alphaf, __ldcs(A.k_add32 + gi), fmaf(A.inc_af, float(zz), d2f_int(e)));
                }
              else
                {
                  double un   = fma(A.b, kd, A.u_in ? __ldcs(A.u_in + gi) : 0.0);
                  un          = fma(A.inc_alpha, __ldcs(A.k_add + gi), un);
                  A.u_out[gi] = un + __ldcs(A.u_base + gi);
                }
              continue;
            }
          if (!TR && A.k_add)
            kd += __ldcs(A.k_add + gi);
          if (A.mode == kModeStage)
            {
              const double u  = (TR || A.u_in) ? __ldcs(A.u_in + gi) : 0.0;
              const double rn = fma(A.a, kd, u);
              A.u_out[gi]     = fma(A.b, kd, u);
              A.r_out[gi]     = rn;
              next[k]         = rn;
              if (!TR && A.k_out)
                A.k_out[gi] = kd;
            }
          else if (A.mode == kModeLastStage)
            {
              double un = fma(A.b, kd, __ldcs(A.u_in + gi));
              if (!TR && A.u_base)
                un += A.u_base[gi];
              A.u_out[gi] = un;
              next[k]     = un;
            }
          else
            {
              A.r_out[gi] = A.out_scale * kd;
              next[k]     = 0.0;
            }
        }
      if (TR && A.tr_out)
        {
          // the next input in the operator's precision (what the next stage
          // would load); z traces from registers, and the pencil goes to this
          // thread's own column of Qb (read above by this thread only) for
          // the x and y traces
          T nt[N], lo, hi;
#pragma unroll
          for (int k = 0; k < N; ++k)
            nt[k] = from_double<T>(next[k]);
          T *to = static_cast<T *>(A.tr_out) + ((cell0 + cl) * 6 + 4) * TRW * NF + r;
          if (upw)
            {
              if (upwind_pencil_traces<N, T>(tb, nt, zlo, zhi, to, to + TRW * NF))
                s_both[atomicAdd(s_nboth, 1)] = (2 * C + cl) * NF + r;
            }
          else
            {
              pencil_traces<N, T>(tb, nt, lo, hi);
              to[0]        = lo;
              to[TRW * NF] = hi;
            }
          if (VISC)
            {
              pencil_dtraces<N, T>(tb, nt, lo, hi);
              to[NF]           = lo;
              to[TRW * NF + NF] = hi;
            }
#pragma unroll
          for (int k = 0; k < N; ++k)
            z[k * NF] = nt[k];
        }
    }
  if (TR && A.tr_out)
    {
      __syncthreads();
      for (int w = tid; w < 2 * ncell * NF; w += NT)
        {
          const int dd = w / (ncell * NF), v = w % (ncell * NF);
          const int cl = v / NF, r = v % NF;
          const int off = dd == 0 ? N * r : (r % N) + NF * (r / N);
          const int st  = dd == 0 ? 1 : N;
          const T  *p   = Qb + cl * NQ + off;
          T         x[N], lo, hi;
#pragma unroll
          for (int k = 0; k < N; ++k)
            x[k] = p[k * st];
          T *to = static_cast<T *>(A.tr_out) + ((cell0 + cl) * 6 + 2 * dd) * TRW * NF + r;
          if (upw)
            {
              const unsigned char *nd = s_need + (cl * 6 + 2 * dd) * NF + r;
              if (upwind_pencil_traces<N, T>(tb, x, nd[0] != 0, nd[NF] != 0, to, to + TRW * NF))
                s_both[atomicAdd(s_nboth, 1)] = (dd * C + cl) * NF + r;
            }
          else
            {
              pencil_traces<N, T>(tb, x, lo, hi);
              to[0]        = lo;
              to[TRW * NF] = hi;
            }
          if (VISC)
            {
              pencil_dtraces<N, T>(tb, x, lo, hi);
              to[NF]            = lo;
              to[TRW * NF + NF] = hi;
            }
        }
      if (upw)
        {
          // the deferred high traces (usually none: no thread enters the loop)
          __syncthreads();
          const int nb = *s_nboth;
          for (int i = tid; i < nb; i += NT)
            {
              const int code = s_both[i];
              const int dd = code / (C * NF), cl = (code / NF) % C, r = code % NF;
              const int off = dd == 0 ? N * r : dd == 1 ? (r % N) + NF * (r / N) : r;
              const int st  = dd == 0 ? 1 : dd == 1 ? N : NF;
              const T  *p   = Qb + cl * NQ + off;
              T         h   = tb.l1[0] * p[0];
#pragma unroll
              for (int q = 1; q < N; ++q)
                h = fma(tb.l1[q], p[q * st], h);
              static_cast<T *>(A.tr_out)[((cell0 + cl) * 6 + 2 * dd + 1) * TRW * NF + r] = h;
            }
        }
    }
}

// resident CTAs per SM the compiler has to allow for: with traces at degree 4
// on field geometry the FP64 kernel is bounded to 72 registers (no spills),
// 7 CTAs per SM; measured on GB300 on 64^3 curved cells: faster than the
// unbounded 94 registers (5 CTAs, 2.2 %) and than 8 or 9 CTAs (64 and 56
// registers with spills)
template <int N, typename T, bool UNI, bool VISC, bool TR>
constexpr int gauss_min_blocks()
{
  return TR && !UNI && !VISC && N == 5 && sizeof(T) == sizeof(double) ? 7 : 1;
}

template <int N, typename T, bool UNI, bool VISC, bool TR, bool INC, bool UPW>
__global__ void __launch_bounds__(StageShape<N, T, UNI, VISC>::THREADS) stage_gauss_kernel(const StageArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_gauss_cta<N, T, UNI, VISC, TR, INC, UPW>(
    A, A.cell_begin + (long long)blockIdx.x * StageShape<N, T, UNI, VISC>::C, smem_raw);
}

// the same with the resident-CTA bound (only where gauss_min_blocks > 1: an
// explicit bound of 1 changes the register allocation of the others)
template <int N, typename T, bool UNI, bool VISC, bool TR, bool INC, bool UPW>
__global__ void __launch_bounds__(StageShape<N, T, UNI, VISC>::THREADS, (gauss_min_blocks<N, T, UNI, VISC, TR>()))
  stage_gauss_kernel_bounded(const StageArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_gauss_cta<N, T, UNI, VISC, TR, INC, UPW>(
    A, A.cell_begin + (long long)blockIdx.x * StageShape<N, T, UNI, VISC>::C, smem_raw);
}

template <int N, typename T, bool UNI, bool VISC, bool TR, bool INC, bool UPW>
constexpr auto gauss_kernel()
{
  if constexpr (gauss_min_blocks<N, T, UNI, VISC, TR>() > 1)
    return stage_gauss_kernel_bounded<N, T, UNI, VISC, TR, INC, UPW>;
  else
    return stage_gauss_kernel<N, T, UNI, VISC, TR, INC, UPW>;
}

template <int N, typename T, bool UNI, bool VISC, bool TR, bool INC = false, bool UPW = false>
cudaError_t launch_stage_gauss_t(const StageArgs &args, cudaStream_t stream)
{
  using GS = GaussShape<N, T, UNI, VISC, TR>;
  constexpr auto kernel = gauss_kernel<N, T, UNI, VISC, TR, INC, UPW>();
  static std::atomic<unsigned long long> configured{0};
  cudaError_t                            e = opt_in_smem(kernel, GS::SMEM, configured);
  if (e != cudaSuccess)
    return e;
  const long long blocks = (args.n_cells - args.cell_begin + GS::C - 1) / GS::C;
  kernel<<<(unsigned)blocks, GS::THREADS, GS::SMEM, stream>>>(args);
  return cudaGetLastError();
}

template <int N, typename T>
cudaError_t launch_stage_gauss_n(const StageArgs &args, cudaStream_t stream)
{
  // face traces: FP64 only (the library's choice; the kernel code is generic)
  if constexpr (sizeof(T) == sizeof(double))
    if (args.tr_in)
      {
        // the FP32-increment anchor reads traces on field geometry without
        // SIPG (and writes none)
        if (args.inc32 && !args.visc && !args.uniform)
          return args.upwind_tr ? launch_stage_gauss_t<N, T, false, false, true, true, true>(args, stream)
                                : launch_stage_gauss_t<N, T, false, false, true, true>(args, stream);
        if (args.upwind_tr && !args.visc && !args.uniform)
          return launch_stage_gauss_t<N, T, false, false, true, false, true>(args, stream);
        return args.visc ? launch_stage_gauss_t<N, T, false, true, true>(args, stream)
             : args.uniform ? launch_stage_gauss_t<N, T, true, false, true>(args, stream)
                            : launch_stage_gauss_t<N, T, false, false, true>(args, stream);
      }
  if (args.inc32)
    return args.visc ? launch_stage_gauss_t<N, T, false, true, false, true>(args, stream)
         : args.uniform ? launch_stage_gauss_t<N, T, true, false, false, true>(args, stream)
                        : launch_stage_gauss_t<N, T, false, false, false, true>(args, stream);
  if (args.visc)
    return launch_stage_gauss_t<N, T, false, true, false>(args, stream);
  return args.uniform ? launch_stage_gauss_t<N, T, true, false, false>(args, stream)
                      : launch_stage_gauss_t<N, T, false, false, false>(args, stream);
}

template <typename T>
cudaError_t launch_stage_gauss_any(int n, const StageArgs &args, cudaStream_t stream)
{
  switch (n)
    {
      case 2: return launch_stage_gauss_n<2, T>(args, stream);
      case 3: return launch_stage_gauss_n<3, T>(args, stream);
      case 4: return launch_stage_gauss_n<4, T>(args, stream);
      case 5: return launch_stage_gauss_n<5, T>(args, stream);
      case 6: return launch_stage_gauss_n<6, T>(args, stream);
      case 7: return launch_stage_gauss_n<7, T>(args, stream);
      default: return cudaErrorInvalidValue;
    }
}
} // namespace adv
