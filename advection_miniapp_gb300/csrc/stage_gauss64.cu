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
template <int N, int MODE>
__global__ void __launch_bounds__(StageShape<N, double, true, false>::THREADS)
  basis_kernel(double *u, long long cell_begin, long long cell_end, double *traces, int width)
{
  using SH         = StageShape<N, double, true, false>;
  constexpr int C  = SH::C;
  constexpr int NQ = SH::NQ;
  constexpr int NF = SH::NF;
  constexpr int NT = SH::THREADS;
  __shared__ double    buf[C * NQ];
  const DevTables<double> &tb    = tab<double>(N);
  const long long          cell0 = cell_begin + (long long)blockIdx.x * C;
  const int                ncell = (int)min((long long)C, cell_end - cell0);
  const int                tid   = threadIdx.x;
  double                  *g     = u + cell0 * NQ;
  constexpr bool TO_GAUSS = MODE == 1;
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
          pencil_traces<N, double>(tb, x, lo, hi);
          double *to     = traces + ((cell0 + cl) * 6 + 2 * d) * width * NF + r;
          to[0]          = lo;
          to[width * NF] = hi;
          if (width == 2)
            {
              pencil_dtraces<N, double>(tb, x, lo, hi);
              to[NF]     = lo;
              to[3 * NF] = hi;
            }
        }
    }
}

template <int N>
cudaError_t launch_basis_n(double *u, long long cell_begin, long long cell_end, int mode, cudaStream_t s,
                           double *traces, int width)
{
  using SH               = StageShape<N, double, true, false>;
  const long long blocks = (cell_end - cell_begin + SH::C - 1) / SH::C;
  if (blocks <= 0)
    return cudaSuccess;
  if (mode == 1)
    basis_kernel<N, 1><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, traces, width);
  else if (mode == 2)
    basis_kernel<N, 2><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, traces, width);
  else if (mode == 3)
    basis_kernel<N, 3><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, nullptr, 1);
  else
    basis_kernel<N, 0><<<(unsigned)blocks, SH::THREADS, 0, s>>>(u, cell_begin, cell_end, nullptr, 1);
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
                              cudaStream_t stream, double *traces, int width)
{
  switch (n)
    {
      case 2: return launch_basis_n<2>(u, cell_begin, cell_end, mode, stream, traces, width);
      case 3: return launch_basis_n<3>(u, cell_begin, cell_end, mode, stream, traces, width);
      case 4: return launch_basis_n<4>(u, cell_begin, cell_end, mode, stream, traces, width);
      case 5: return launch_basis_n<5>(u, cell_begin, cell_end, mode, stream, traces, width);
      case 6: return launch_basis_n<6>(u, cell_begin, cell_end, mode, stream, traces, width);
      case 7: return launch_basis_n<7>(u, cell_begin, cell_end, mode, stream, traces, width);
      default: return cudaErrorInvalidValue;
    }
}
} // namespace

cudaError_t launch_basis_change(int n, double *u, long long cell_begin, long long cell_end, bool to_gauss,
                                cudaStream_t stream, double *traces, int width)
{
  return launch_basis_mode(n, u, cell_begin, cell_end, to_gauss ? 1 : 0, stream, traces, width);
}

cudaError_t launch_basis_dual_to_nodal(int n, double *u, long long cell_begin, long long cell_end,
                                       cudaStream_t stream)
{
  return launch_basis_mode(n, u, cell_begin, cell_end, 3, stream, nullptr, 1);
}

cudaError_t launch_face_traces(int n, const double *u, long long cell_begin, long long cell_end,
                               cudaStream_t stream, double *traces, int width)
{
  return launch_basis_mode(n, const_cast<double *>(u), cell_begin, cell_end, 2, stream, traces, width);
}
} // namespace adv
