// Private definition of adv_handle and the helpers shared by the C ABI
// translation units (api.cu, implicit_api.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/advection_gb300.h"
#include "geometry.h"
#include "kernels.h"
#include "tables.h"

struct adv_handle
{
  adv_config       cfg;
  adv::Mesh        mesh;
  adv::Tables1D    tb;
  int              device = 0;
  double           h_min  = 0.0;
  // uniform-case constants
  double cv[3] = {}, P[3] = {}, M[3] = {};
  // device buffers
  void    *d_cell_geo    = nullptr;     // field geometry in the operator's precision
  void    *d_face_geo[3] = {};
  double  *d_cell_geo64    = nullptr;   // FP32 increments: the FP64 copy for the anchor stage
  double  *d_face_geo64[3] = {};
  double  *d_face_x[3]   = {};
  double  *d_partials    = nullptr;
  double  *d_scratch[2]  = {};
  void    *d_traces[2]   = {}; // face traces of the collocation step loop (lazily allocated)
  float   *d_inc32       = nullptr; // FP32 increments: two G registers and K0 in binary32 (lazily)
  // device address of the library's static stage scratch (adv_perform_stage_noalloc),
  // looked up when the handle is created, with its device current
  double  *noalloc_scratch = nullptr;
  int64_t  device_bytes  = 0;
  int64_t  launches      = 0;
  adv::DiagArgs diag;
  // per cell (v0, v1, v2, 1/|K|): cell average of J^{-1} a and inverse volume, for the FDM preconditioner
  double *d_fdm_cell_d = nullptr;
  float  *d_fdm_cell_f = nullptr;
  // call timing (adv_set_timing): event pairs around the device work of each
  // timed call, folded into the totals when queried
  bool                                            timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timed_events;
  double                                          timed_seconds = 0.0;
  int64_t                                         timed_calls   = 0;
  int                                             trace_depth   = 0; // entry points nested in a traced call
  // adv_lsrk_steps_host: copy streams (host -> device, device -> host) and
  // the events that order the chunked copies against the stage launches
  cudaStream_t             copy_stream[2] = {};
  std::vector<cudaEvent_t> pipe_events;
};


namespace adv
{
namespace detail
{
int            fail(int code, const std::string &msg);
int            cuda_fail(cudaError_t e, const char *where);
// stage arguments at time t for the operator precision op_precision
// (0 = FP64, 1 = FP32; -1 = the handle's own)
adv::StageArgs base_args(const adv_handle &h, double t, int op_precision = -1);
int            launch(adv_handle *h, const adv::StageArgs &A, cudaStream_t s);
int            check_device(const adv_handle *h);
// uploads the 1D tables to every translation unit on this device (once)
int            ensure_tables(int device);
// arguments of the projection / mass-energy / L2-error kernels for a mesh
void           make_diag(const adv_config &cfg, const adv::Mesh &m, const adv::Tables1D &tb, adv::DiagArgs &g);
// An NVTX range named after the entry point for the duration of the call
// and, when the handle times its calls, a pair of events around the device
// work the call enqueues on its stream.
class CallTrace
{
public:
  CallTrace(adv_handle *h, const char *name, cudaStream_t s);
  ~CallTrace();
  CallTrace(const CallTrace &)            = delete;
  CallTrace &operator=(const CallTrace &) = delete;

private:
  adv_handle  *h_  = nullptr;
  cudaStream_t s_  = nullptr;
  cudaEvent_t  e0_ = nullptr;
};
} // namespace detail
} // namespace adv

#define ADV_CUDA(call)                                   \
  do                                                     \
    {                                                    \
      cudaError_t e_ = (call);                           \
      if (e_ != cudaSuccess)                             \
        return adv::detail::cuda_fail(e_, #call);        \
    }                                                    \
  while (0)
