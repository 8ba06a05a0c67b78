// Instantiations of the collocation-form stage kernel with a binary64
// operator, and the change of basis of the fused LSRK loop.
#include "stage_gauss.cuh"

namespace adv
{
namespace
{
// u <- (M x M x M) u per cell, M = S (to the Gauss points) or S^-1, through
// shared memory: one thread per pencil, C cells per CTA.  MODE 1: to the
// Gauss points (optionally with the face traces of the result), 0: back to
// the Gauss-Lobatto nodes, 2: only the face traces of u (no change of basis),
// 3: M = S^T (dual coefficients from the Gauss-point to the nodal basis).
// UPW: upwind traces (StageArgs::upwind_tr; F carries the mesh and the FP64
// face coefficients): only the traces the first stage reads, as the stage
// kernel writes them.
template <int N, int MODE, bool UPW>
__global__ void __launch_bounds__(StageShape<N, double, true, false>::THREADS)
  basis_kernel(double *u, long long cell_begin, long long cell_end, double *traces, int width, const StageArgs F)
{
  using SH         = StageShape<N, double, true, false>;
  constexpr int C  = SH::C;
  constexpr int NQ = SH::NQ;
  constexpr int NF = SH::NF;
  constexpr int NT = SH::THREADS;
  __shared__ double    buf[C * NQ];
  // upwind traces: face ids, and the pencils whose high trace is deferred
  __shared__ int           s_face[UPW ? 6 * C : 1], s_nbr[UPW ? 6 * C : 1], s_nboth, s_both[UPW ? 3 * C * NF : 1];
  const DevTables<double> &tb    = tab<double>(N);
  const long long          cell0 = cell_begin + (long long)blockIdx.x * C;
  const int                ncell = (int)min((long long)C, cell_end - cell0);
  const int                tid   = threadIdx.x;
  double                  *g     = u + cell0 * NQ;
  constexpr bool TO_GAUSS = MODE == 1;
  if (UPW)
    {
      cell_neighbours(F, cell0, ncell, s_nbr, s_face, tid, NT);
      if (tid == 0)
        s_nboth = 0;
    }
  for (int i = tid; i < ncell * NQ; i += NT)
    buf[i] = g[i];
  __syncthreads();
#pragma unroll
  for (int d = 0; d < (MODE == 2 ? 0 : 3); ++d)
    {
      for (int w = tid; w < ncell * NF; w += NT)
        {
          const int cl = w / NF, r = w % NF;
          const int off = d == 0 ? N * r : d == 1 ? (r % N) + NF * (r / N) : r;
          const int st  = d == 0 ? 1 : d == 1 ? N : NF;
          double   *p   = buf + cl * NQ + off;
          double    in[N], out[N];
#pragma unroll
          for (int k = 0; k < N; ++k)
            in[k] = p[k * st];
          if (TO_GAUSS)
            sweep2<N, double, false>(tb.S, tb.S_eo, in, out);
          else if (MODE == 3)
            sweep2<N, double, false>(tb.St, tb.St_eo, in, out);
          else
            sweep2<N, double, false>(tb.Si, tb.Si_eo, in, out);
#pragma unroll
          for (int k = 0; k < N; ++k)
            p[k * st] = out[k];
        }
      __syncthreads();
    }
  if (MODE != 2)
    for (int i = tid; i < ncell * NQ; i += NT)
      g[i] = buf[i];
  if (MODE != 0 && traces)
    {
      // face traces of the result, [6][width][NF] per cell (StageArgs::tr_in):
      // values, and with width 2 also reference normal derivatives
      for (int w = tid; w < 3 * ncell * NF; w += NT)
        {
          const int d = w / (ncell * NF), v = w % (ncell * NF);
          const int cl = v / NF, r = v % NF;
          const int off = d == 0 ? N * r : d == 1 ? (r % N) + NF * (r / N) : r;
          const int st  = d == 0 ? 1 : d == 1 ? N : NF;
          double    x[N], lo, hi;
#pragma unroll
          for (int k = 0; k < N; ++k)
            x[k] = buf[cl * NQ + off + k * st];
          double *to = traces + ((cell0 + cl) * 6 + 2 * d) * width * NF + r;
          if (UPW)
            {
              // own trace read on the low face where M != 0, on the high face where P != 0
              const double *fg = d == 0 ? static_cast<const double *>(F.face_geo[0])
                               : d == 1 ? static_cast<const double *>(F.face_geo[1])
                                        : static_cast<const double *>(F.face_geo[2]);
              const double2 pl = *reinterpret_cast<const double2 *>(fg + (size_t)s_face[cl * 6 + 2 * d] * 2 * NF + 2 * r);
              const double2 ph =
                *reinterpret_cast<const double2 *>(fg + (size_t)s_face[cl * 6 + 2 * d + 1] * 2 * NF + 2 * r);
              if (upwind_pencil_traces<N, double>(tb, x, nonzero(pl.y), nonzero(ph.x), to, to + NF))
                s_both[atomicAdd(&s_nboth, 1)] = (d * C + cl) * NF + r;
              continue;
            }
          pencil_traces<N, double>(tb, x, lo, hi);
          to[0]          = lo;
          to[width * NF] = hi;
          if (width == 2)
            {
              pencil_dtraces<N, double>(tb, x, lo, hi);
              to[NF]     = lo;
              to[3 * NF] = hi;
            }
        }
      if (UPW)
        {
          // the deferred high traces (usually none)
          __syncthreads();
          for (int i = tid; i < s_nboth; i += NT)
            {
              const int code = s_both[i];
              const int d = code / (C * NF), cl = (code / NF) % C, r = code % NF;
              const int off = d == 0 ? N * r : d == 1 ? (r % N) + NF * (r / N) : r;
              const int st  = d == 0 ? 1 : d == 1 ? N : NF;
              double    h   = tb.l1[0] * buf[cl * NQ + off];
#pragma unroll
              for (int q = 1; q < N; ++q)
                h = fma(tb.l1[q], buf[cl * NQ + off + q * st], h);
              traces[((cell0 + cl) * 6 + 2 * d + 1) * NF + r] = h;
            }
        }
    }
}

template <int N>
cudaError_t launch_basis_n(double *u, long long cell_begin, long long cell_end, int mode, cudaStream_t s,
                           double *traces, int width, const StageArgs *upwind)
{
  using SH               = StageShape<N, double, true, false>;
  const long long blocks = (cell_end - cell_begin + SH::C - 1) / SH::C;
  if (blocks <= 0)
    return cudaSuccess;
  StageArgs F;
  if (upwind)
    F = *upwind;
  else
    memset(&F, 0, sizeof(F));
  const bool upw = upwind && traces && width == 1;
  if (mode == 1 && upw)
    basis_kernel<N, 1, true><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, traces, width, F);
  else if (mode == 1)
    basis_kernel<N, 1, false><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, traces, width, F);
  else if (mode == 2 && upw)
    basis_kernel<N, 2, true><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, traces, width, F);
  else if (mode == 2)
    basis_kernel<N, 2, false><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, traces, width, F);
  else if (mode == 3)
    basis_kernel<N, 3, false><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, nullptr, 1, F);
  else
    basis_kernel<N, 0, false><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, nullptr, 1, F);
  return cudaGetLastError();
}
} // namespace

cudaError_t upload_tables_gauss64(const DevTables<double> *d, const DevTables<float> *f)
{
  return upload_tables_local(d, f);
}

cudaError_t launch_stage_gauss_fp64(int n, const StageArgs &args, cudaStream_t stream)
{
  return launch_stage_gauss_any<double>(n, args, stream);
}

namespace
{
cudaError_t launch_basis_mode(int n, double *u, long long cell_begin, long long cell_end, int mode,
                              cudaStream_t stream, double *traces, int width, const StageArgs *upwind = nullptr)
{
  switch (n)
    {
      case 2: return launch_basis_n<2>(u, cell_begin, cell_end, mode, stream, traces, width, upwind);
      case 3: return launch_basis_n<3>(u, cell_begin, cell_end, mode, stream, traces, width, upwind);
      case 4: return launch_basis_n<4>(u, cell_begin, cell_end, mode, stream, traces, width, upwind);
      case 5: return launch_basis_n<5>(u, cell_begin, cell_end, mode, stream, traces, width, upwind);
      case 6: return launch_basis_n<6>(u, cell_begin, cell_end, mode, stream, traces, width, upwind);
      case 7: return launch_basis_n<7>(u, cell_begin, cell_end, mode, stream, traces, width, upwind);
      default: return cudaErrorInvalidValue;
    }
}
} // namespace

cudaError_t launch_basis_change(int n, double *u, long long cell_begin, long long cell_end, bool to_gauss,
                                cudaStream_t stream, double *traces, int width, const StageArgs *upwind)
{
  return launch_basis_mode(n, u, cell_begin, cell_end, to_gauss ? 1 : 0, stream, traces, width, upwind);
}

cudaError_t launch_basis_dual_to_nodal(int n, double *u, long long cell_begin, long long cell_end,
                                       cudaStream_t stream)
{
  return launch_basis_mode(n, u, cell_begin, cell_end, 3, stream, nullptr, 1);
}

cudaError_t launch_face_traces(int n, const double *u, long long cell_begin, long long cell_end,
                               cudaStream_t stream, double *traces, int width, const StageArgs *upwind)
{
  return launch_basis_mode(n, const_cast<double *>(u), cell_begin, cell_end, 2, stream, traces, width, upwind);
}
} // namespace adv
