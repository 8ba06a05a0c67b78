// Launch interface of the batched multi-solve kernels (batch_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "device_common.cuh"

namespace adv
{
// One active solve of a serving group (device memory, read by every stage launch).
struct BatchSlot
{
  double   *u, *r, *k;      // solution and the two Runge-Kutta registers
  double   *t0, *t1;        // collocation form: face traces of the stage inputs (even / odd stage count)
  int       n;              // cells per direction of the periodic unit cube
  int       steps_total;    // time steps of the solve
  int       steps_done;     // advanced by the step-advance kernel
  int       active;
  double    dt;
  double    cv[3], P[3], M[3];    // uniform operator constants (a_d / h and the upwind split)
  float     cvf[3], Pf[3], Mf[3];
  int       pad;
};

struct BatchLaunch
{
  const BatchSlot *slots;
  const int       *cta_slot;  // solve of each CTA
  const long long *cta_cell0; // first cell (within its solve) of each CTA
  const int       *n_ctas;    // CTAs in use (device memory: graphs stay valid as the batch changes)
  int              stage, n_stages;
  double           bi[16], ai[16];
};

cudaError_t upload_tables_batch(const DevTables<double> *d, const DevTables<float> *f);
int         batch_cells_per_cta(int n);
// whether the group's vectors hold Gauss-point values (collocation form)
bool        batch_collocation(int precision);
// sets the kernel's shared-memory limit on the current device (call before capturing a graph)
cudaError_t prepare_batch_stage(int n, int precision);
cudaError_t launch_batch_stage(int n, int precision, const BatchLaunch &L, int cta_capacity, cudaStream_t s);
cudaError_t launch_batch_advance(BatchSlot *slots, const int *n_slots, int slot_capacity, cudaStream_t s);
} // namespace adv
