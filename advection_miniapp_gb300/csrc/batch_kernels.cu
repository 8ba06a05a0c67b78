// Batched multi-solve stage kernels of the serving loop.
//
// One launch performs one Runge-Kutta stage for every active solve of a group
// (same degree and operator precision; affine periodic meshes with constant
// velocity, the serving mix).  The CTAs are mapped to (solve, first cell)
// pairs by two device tables; each CTA builds its solve's stage arguments in
// shared memory and runs the same per-CTA code as the single-mesh fused step
// loop in the form that loop picks by default (collocation for the FP64
// operator, nodal for the FP32 one), so a solve computes bit-for-bit the same
// values alone, inside a batch, and through adv_lsrk_steps.
// Slot tables live in device memory so that a captured CUDA graph of a tick
// (steps x stages launches + one step-advance launch per step) stays valid
// while solves join and leave the batch.
#include "batch_kernels.h"
#include "stage_gauss.cuh"

namespace adv
{
namespace
{
template <typename T>
constexpr bool kBatchCollocation = sizeof(T) == sizeof(double);

// dynamic shared memory of the per-CTA code the group runs
template <int N, typename T>
constexpr int kBatchSmem = kBatchCollocation<T> ? GaussShape<N, T, true, false, true>::SMEM
                                                : StageShape<N, T, true, false>::SMEM;

template <int N, typename T>
__global__ void __launch_bounds__(StageShape<N, T, true, false>::THREADS) batch_stage_kernel(const BatchLaunch L)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StageArgs sA;
  __shared__ int       skip;
  __shared__ long long cell0;
  if ((int)blockIdx.x >= *L.n_ctas)
    return;
  if (threadIdx.x == 0)
    {
      const int        si = L.cta_slot[blockIdx.x];
      const BatchSlot &S  = L.slots[si];
      skip                = !S.active || S.steps_done >= S.steps_total;
      cell0               = L.cta_cell0[blockIdx.x];
      if (!skip)
        {
          StageArgs a;
          memset(&a, 0, sizeof(a));
          for (int d = 0; d < 3; ++d)
            {
              a.nc[d] = a.npos[d] = S.n;
              a.cv[d]  = S.cv[d], a.P[d] = S.P[d], a.M[d] = S.M[d];
              a.cvf[d] = S.cvf[d], a.Pf[d] = S.Pf[d], a.Mf[d] = S.Mf[d];
            }
          a.n_cells   = (long long)S.n * S.n * S.n;
          a.periodic  = 7;
          a.uniform   = 1;
          a.out_scale = 1.0;
          // stage rotation of the three registers (as adv_lsrk_steps)
          const int  st   = L.stage;
          const bool last = st == L.n_stages - 1;
          if (st == 0)
            a.r_in = S.u, a.u_in = S.u, a.u_out = S.k, a.r_out = S.r;
          else if (st == 1)
            a.r_in = S.r, a.u_in = S.k, a.u_out = S.u, a.r_out = S.k;
          else
            {
              a.r_in  = (st % 2 == 0) ? S.k : S.r;
              a.u_in  = S.u;
              a.u_out = S.u;
              a.r_out = last ? nullptr : ((st % 2 == 0) ? S.r : S.k);
            }
          a.b    = L.bi[st] * S.dt;
          a.a    = last ? 0.0 : L.ai[st] * S.dt;
          a.mode = last ? kModeLastStage : kModeStage;
          if (kBatchCollocation<T>)
            {
              // stage count of the solve so far: even reads t0, odd reads t1
              // (the single-mesh loop alternates the same way from t0)
              const bool odd = ((S.steps_done * L.n_stages + st) & 1) != 0;
              a.tr_in        = odd ? S.t1 : S.t0;
              a.tr_out       = odd ? S.t0 : S.t1;
            }
          sA     = a;
        }
    }
  __syncthreads();
  if (skip)
    return;
  if constexpr (kBatchCollocation<T>)
    stage_gauss_cta<N, T, true, false, true>(sA, cell0, smem_raw);
  else
    stage_cta<N, T, true, false>(sA, cell0, smem_raw);
}

__global__ void batch_advance_kernel(BatchSlot *slots, const int *n_slots)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < *n_slots && slots[i].active && slots[i].steps_done < slots[i].steps_total)
    slots[i].steps_done += 1;
}

template <int N, typename T>
cudaError_t prepare_batch_t()
{
  return cudaFuncSetAttribute(batch_stage_kernel<N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kBatchSmem<N, T>);
}

template <int N, typename T>
cudaError_t launch_batch_t(const BatchLaunch &L, int cta_capacity, cudaStream_t s)
{
  using SH = StageShape<N, T, true, false>;
  batch_stage_kernel<N, T><<<cta_capacity, SH::THREADS, kBatchSmem<N, T>, s>>>(L);
  return cudaGetLastError();
}
} // namespace

cudaError_t upload_tables_batch(const DevTables<double> *d, const DevTables<float> *f)
{
  return upload_tables_local(d, f);
}

bool batch_collocation(int precision)
{
  return precision == 0;
}

int batch_cells_per_cta(int n)
{
  return n == 2 ? StageShape<2, double, true, false>::C
       : n == 3 ? StageShape<3, double, true, false>::C
       : n == 4 ? StageShape<4, double, true, false>::C
       : n == 5 ? StageShape<5, double, true, false>::C
       : n == 6 ? StageShape<6, double, true, false>::C
       : n == 7 ? StageShape<7, double, true, false>::C
                : 0;
}

cudaError_t launch_batch_stage(int n, int precision, const BatchLaunch &L, int cta_capacity, cudaStream_t s)
{
  switch (n * 2 + precision)
    {
      case 2 * 2 + 0: return launch_batch_t<2, double>(L, cta_capacity, s);
      case 2 * 2 + 1: return launch_batch_t<2, float>(L, cta_capacity, s);
      case 3 * 2 + 0: return launch_batch_t<3, double>(L, cta_capacity, s);
      case 3 * 2 + 1: return launch_batch_t<3, float>(L, cta_capacity, s);
      case 4 * 2 + 0: return launch_batch_t<4, double>(L, cta_capacity, s);
      case 4 * 2 + 1: return launch_batch_t<4, float>(L, cta_capacity, s);
      case 5 * 2 + 0: return launch_batch_t<5, double>(L, cta_capacity, s);
      case 5 * 2 + 1: return launch_batch_t<5, float>(L, cta_capacity, s);
      case 6 * 2 + 0: return launch_batch_t<6, double>(L, cta_capacity, s);
      case 6 * 2 + 1: return launch_batch_t<6, float>(L, cta_capacity, s);
      case 7 * 2 + 0: return launch_batch_t<7, double>(L, cta_capacity, s);
      case 7 * 2 + 1: return launch_batch_t<7, float>(L, cta_capacity, s);
      default: return cudaErrorInvalidValue;
    }
}

cudaError_t prepare_batch_stage(int n, int precision)
{
  switch (n * 2 + precision)
    {
      case 2 * 2 + 0: return prepare_batch_t<2, double>();
      case 2 * 2 + 1: return prepare_batch_t<2, float>();
      case 3 * 2 + 0: return prepare_batch_t<3, double>();
      case 3 * 2 + 1: return prepare_batch_t<3, float>();
      case 4 * 2 + 0: return prepare_batch_t<4, double>();
      case 4 * 2 + 1: return prepare_batch_t<4, float>();
      case 5 * 2 + 0: return prepare_batch_t<5, double>();
      case 5 * 2 + 1: return prepare_batch_t<5, float>();
      case 6 * 2 + 0: return prepare_batch_t<6, double>();
      case 6 * 2 + 1: return prepare_batch_t<6, float>();
      case 7 * 2 + 0: return prepare_batch_t<7, double>();
      case 7 * 2 + 1: return prepare_batch_t<7, float>();
      default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch_advance(BatchSlot *slots, const int *n_slots, int slot_capacity, cudaStream_t s)
{
  batch_advance_kernel<<<(slot_capacity + 127) / 128, 128, 0, s>>>(slots, n_slots);
  return cudaGetLastError();
}
} // namespace adv
