// Serving loop: continuous batching of independent advection solves on one GPU.
//
// Requests (a periodic affine mesh of n^3 cells, degree k, constant velocity,
// end time, operator precision) are admitted in FIFO order while their state
// (three FP64 vectors) fits a device-memory budget.  Admitted solves join the
// group of their (degree, precision); every group has its own stream and a
// captured CUDA graph of one tick (steps_per_tick steps of the batched
// multi-solve stage kernel plus a step-advance kernel), replayed while solves
// join and leave: the slot tables the kernels read live in device memory.
// Groups run concurrently on their streams, so solves of different degrees
// and precisions overlap on the device.  Device memory of a solve is taken and
// returned stream-ordered (cudaMallocAsync / cudaFreeAsync), so admissions and
// retirements do not synchronise the device.  The host polls tick completion
// with events, retires finished solves (L2 error against the exact solution)
// and admits waiting ones.  There is no counterpart in the reference, which
// runs one solve per program.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "batch_kernels.h"
#include "geometry.h"
#include "handle.h"
#include "kernels.h"
#include "tables.h"

using adv::detail::fail;

namespace
{
double now_s()
{
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct SReq
{
  adv_config          cfg;
  double              t_end = 0, courant = 0.5;
  int                 n = 0, npts = 0, precision = 0;
  int64_t             n_dofs = 0, bytes = 0;
  double              dt = 0;
  int                 steps = 0, steps_done = 0;
  double             *u = nullptr, *r = nullptr, *k = nullptr;
  double             *t0 = nullptr, *t1 = nullptr; // face traces (collocation groups)
  int                 state = 0; // 0 queued, 1 active, 2 done, 3 failed (device memory or launch at admission), 4 cancelled
  bool                cancel = false; // cancellation requested while active
  double              t_submit = 0, t_admit = 0, t_done = 0, rel_l2 = -1;
  std::vector<double> solution;
  adv::DiagArgs       diag;
  double              cv[3] = {}, P[3] = {}, M[3] = {};
};

struct SGroup
{
  int                  npts = 0, precision = 0;
  cudaStream_t         stream = nullptr;
  cudaEvent_t          event  = nullptr;
  bool                 in_flight = false, dirty = false;
  std::vector<int64_t> members;
  adv::BatchSlot      *d_slots = nullptr, *h_slots = nullptr;
  int                 *d_counts = nullptr; // [n_slots, n_ctas]
  int                 *d_cta_slot = nullptr;
  long long           *d_cta_cell0 = nullptr;
  double              *d_partials = nullptr;
  int                  slot_cap = 0, cta_cap = 0;
  size_t               launched = 0; // members covered by the tick in flight (admissions append after them)
  cudaGraphExec_t      exec = nullptr;
};
} // namespace

struct adv_server
{
  int64_t             budget = 0, used = 0;
  int                 steps_per_tick = 8, max_active = 256, keep_solutions = 0;
  std::vector<double> bi, ai;
  std::vector<SReq>   reqs;
  std::deque<int64_t> queue;
  int                 active = 0;
  int64_t             completed = 0, ticks = 0, launches = 0;
  std::map<int, SGroup> groups; // key: npts * 2 + precision
  int                 device = 0;
  int                 policy = ADV_SERVE_FIFO;
};

namespace
{
int ensure_group(adv_server *S, int npts, int precision, SGroup **out)
{
  const int key = npts * 2 + precision;
  auto      it  = S->groups.find(key);
  if (it == S->groups.end())
    {
      SGroup g;
      g.npts      = npts;
      g.precision = precision;
      ADV_CUDA(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
      ADV_CUDA(cudaEventCreateWithFlags(&g.event, cudaEventDisableTiming));
      ADV_CUDA(adv::prepare_batch_stage(npts, precision));
      ADV_CUDA(cudaMalloc(&g.d_partials, 3 * 4096 * sizeof(double)));
      ADV_CUDA(cudaMalloc(&g.d_counts, 2 * sizeof(int)));
      it = S->groups.emplace(key, g).first;
    }
  *out = &it->second;
  return ADV_OK;
}

// grow the device tables and capture the tick graph for the new capacities
int grow_and_capture(adv_server *S, SGroup &g, int need_slots, int need_ctas)
{
  bool recapture = g.exec == nullptr;
  if (need_slots > g.slot_cap)
    {
      const int cap = std::max(need_slots, std::max(16, 2 * g.slot_cap));
      cudaFree(g.d_slots);
      cudaFreeHost(g.h_slots);
      ADV_CUDA(cudaMalloc(&g.d_slots, cap * sizeof(adv::BatchSlot)));
      ADV_CUDA(cudaMallocHost(&g.h_slots, cap * sizeof(adv::BatchSlot)));
      g.slot_cap = cap;
      recapture  = true;
    }
  if (need_ctas > g.cta_cap)
    {
      const int cap = std::max(need_ctas, std::max(1024, 2 * g.cta_cap));
      cudaFree(g.d_cta_slot);
      cudaFree(g.d_cta_cell0);
      ADV_CUDA(cudaMalloc(&g.d_cta_slot, cap * sizeof(int)));
      ADV_CUDA(cudaMalloc(&g.d_cta_cell0, cap * sizeof(long long)));
      g.cta_cap = cap;
      recapture = true;
    }
  if (!recapture)
    return ADV_OK;
  if (g.exec)
    cudaGraphExecDestroy(g.exec);
  g.exec = nullptr;
  adv::BatchLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.slots     = g.d_slots;
  L.cta_slot  = g.d_cta_slot;
  L.cta_cell0 = g.d_cta_cell0;
  L.n_ctas    = g.d_counts + 1;
  L.n_stages  = (int)S->bi.size();
  for (size_t i = 0; i < S->bi.size(); ++i)
    L.bi[i] = S->bi[i];
  for (size_t i = 0; i < S->ai.size(); ++i)
    L.ai[i] = S->ai[i];
  cudaGraph_t graph = nullptr;
  ADV_CUDA(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
  for (int step = 0; step < S->steps_per_tick; ++step)
    {
      for (int st = 0; st < L.n_stages; ++st)
        {
          L.stage = st;
          cudaError_t e = adv::launch_batch_stage(g.npts, g.precision, L, g.cta_cap, g.stream);
          if (e != cudaSuccess)
            {
              cudaStreamEndCapture(g.stream, &graph);
              if (graph)
                cudaGraphDestroy(graph);
              return adv::detail::cuda_fail(e, "capture of the batched stage kernel");
            }
        }
      cudaError_t e = adv::launch_batch_advance(g.d_slots, g.d_counts, g.slot_cap, g.stream);
      if (e != cudaSuccess)
        {
          cudaStreamEndCapture(g.stream, &graph);
          if (graph)
            cudaGraphDestroy(graph);
          return adv::detail::cuda_fail(e, "capture of the step-advance kernel");
        }
    }
  ADV_CUDA(cudaStreamEndCapture(g.stream, &graph));
  cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess)
    return adv::detail::cuda_fail(e, "cudaGraphInstantiate");
  return ADV_OK;
}

// rebuild the slot and CTA tables of an idle group from its members
int rebuild(adv_server *S, SGroup &g)
{
  const int            C = adv::batch_cells_per_cta(g.npts);
  std::vector<int>       cta_slot;
  std::vector<long long> cta_cell0;
  std::vector<adv::BatchSlot> slots(g.members.size());
  for (size_t i = 0; i < g.members.size(); ++i)
    {
      SReq          &q = S->reqs[g.members[i]];
      adv::BatchSlot &b = slots[i];
      std::memset(&b, 0, sizeof(b));
      b.u = q.u, b.r = q.r, b.k = q.k;
      b.t0 = q.t0, b.t1 = q.t1;
      b.n           = q.n;
      b.steps_total = q.steps;
      b.steps_done  = q.steps_done;
      b.active      = 1;
      b.dt          = q.dt;
      for (int d = 0; d < 3; ++d)
        {
          b.cv[d] = q.cv[d], b.P[d] = q.P[d], b.M[d] = q.M[d];
          b.cvf[d] = (float)q.cv[d], b.Pf[d] = (float)q.P[d], b.Mf[d] = (float)q.M[d];
        }
      const long long cells = (long long)q.n * q.n * q.n;
      for (long long c = 0; c < cells; c += C)
        {
          cta_slot.push_back((int)i);
          cta_cell0.push_back(c);
        }
    }
  if (int e = grow_and_capture(S, g, (int)slots.size(), (int)cta_slot.size()))
    return e;
  const int counts[2] = {(int)slots.size(), (int)cta_slot.size()};
  ADV_CUDA(cudaMemcpyAsync(g.d_slots, slots.data(), slots.size() * sizeof(adv::BatchSlot), cudaMemcpyHostToDevice,
                           g.stream));
  ADV_CUDA(cudaMemcpyAsync(g.d_cta_slot, cta_slot.data(), cta_slot.size() * sizeof(int), cudaMemcpyHostToDevice,
                           g.stream));
  ADV_CUDA(cudaMemcpyAsync(g.d_cta_cell0, cta_cell0.data(), cta_cell0.size() * sizeof(long long),
                           cudaMemcpyHostToDevice, g.stream));
  ADV_CUDA(cudaMemcpyAsync(g.d_counts, counts, sizeof(counts), cudaMemcpyHostToDevice, g.stream));
  // pageable sources: the copies above are staged before they return
  g.dirty = false;
  return ADV_OK;
}

// an active solve leaves without a result (cancelled): its memory goes back
int drop(adv_server *S, SGroup &g, int64_t id)
{
  SReq &q = S->reqs[id];
  for (double *p : {q.u, q.r, q.k, q.t0, q.t1})
    if (p)
      ADV_CUDA(cudaFreeAsync(p, g.stream));
  q.u = q.r = q.k = q.t0 = q.t1 = nullptr;
  q.state  = 4;
  q.t_done = now_s();
  S->used -= q.bytes;
  --S->active;
  ++S->completed;
  g.dirty = true;
  return ADV_OK;
}

int retire(adv_server *S, SGroup &g, int64_t id)
{
  SReq &q = S->reqs[id];
  int   nb = 0;
  if (adv::batch_collocation(g.precision))
    {
      const long long cells = (long long)q.n * q.n * q.n;
      ADV_CUDA(adv::launch_basis_change(q.npts, q.u, 0, cells, false, g.stream));
      ++S->launches;
    }
  ADV_CUDA(adv::launch_l2_error(q.diag, q.u, q.t_end, g.d_partials, &nb, g.stream));
  ++S->launches;
  std::vector<double> part(3 * nb);
  ADV_CUDA(cudaMemcpyAsync(part.data(), g.d_partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, g.stream));
  if (S->keep_solutions)
    {
      q.solution.resize(q.n_dofs);
      ADV_CUDA(cudaMemcpyAsync(q.solution.data(), q.u, q.n_dofs * sizeof(double), cudaMemcpyDeviceToHost, g.stream));
    }
  ADV_CUDA(cudaStreamSynchronize(g.stream));
  double e2 = 0, n2 = 0;
  for (int b = 0; b < nb; ++b)
    e2 += part[3 * b], n2 += part[3 * b + 1];
  q.rel_l2 = n2 > 0 ? std::sqrt(e2 / n2) : std::sqrt(e2);
  ADV_CUDA(cudaFreeAsync(q.u, g.stream));
  ADV_CUDA(cudaFreeAsync(q.r, g.stream));
  ADV_CUDA(cudaFreeAsync(q.k, g.stream));
  if (q.t0)
    {
      ADV_CUDA(cudaFreeAsync(q.t0, g.stream));
      ADV_CUDA(cudaFreeAsync(q.t1, g.stream));
    }
  q.u = q.r = q.k = q.t0 = q.t1 = nullptr;
  q.state  = 2;
  q.t_done = now_s();
  S->used -= q.bytes;
  --S->active;
  ++S->completed;
  g.dirty = true;
  return ADV_OK;
}

int admit(adv_server *S, int64_t id)
{
  SReq   &q = S->reqs[id];
  SGroup *g = nullptr;
  if (int e = ensure_group(S, q.npts, q.precision, &g))
    return e;
  const size_t    nb    = q.n_dofs * sizeof(double);
  const bool      col   = adv::batch_collocation(q.precision);
  const long long cells = (long long)q.n * q.n * q.n;
  const size_t    tb    = (size_t)cells * 6 * q.npts * q.npts * sizeof(double);
  cudaError_t     e     = cudaMallocAsync((void **)&q.u, nb, g->stream);
  if (e == cudaSuccess)
    e = cudaMallocAsync((void **)&q.r, nb, g->stream);
  if (e == cudaSuccess)
    e = cudaMallocAsync((void **)&q.k, nb, g->stream);
  if (e == cudaSuccess && col)
    e = cudaMallocAsync((void **)&q.t0, tb, g->stream);
  if (e == cudaSuccess && col)
    e = cudaMallocAsync((void **)&q.t1, tb, g->stream);
  if (e == cudaSuccess)
    e = adv::launch_project(q.diag, 0.0, q.u, g->stream);
  if (e == cudaSuccess && col)
    e = adv::launch_basis_change(q.npts, q.u, 0, cells, true, g->stream, q.t0);
  if (e != cudaSuccess)
    {
      // the request fails alone: give back what it holds, keep serving
      cudaGetLastError();
      for (double *p : {q.u, q.r, q.k, q.t0, q.t1})
        if (p)
          cudaFreeAsync(p, g->stream);
      q.u = q.r = q.k = q.t0 = q.t1 = nullptr;
      q.state  = 3;
      q.t_done = now_s();
      ++S->completed;
      return ADV_OK;
    }
  S->launches += col ? 2 : 1;
  q.state   = 1;
  q.t_admit = now_s();
  g->members.push_back(id);
  g->dirty = true;
  S->used += q.bytes;
  ++S->active;
  return ADV_OK;
}
} // namespace

extern "C" {

int adv_server_create(int64_t memory_budget_bytes, int steps_per_tick, int max_active, int keep_solutions,
                      adv_server **out)
{
  if (!out || memory_budget_bytes <= 0 || steps_per_tick < 1 || steps_per_tick > 1000 || max_active < 1)
    return fail(ADV_ERR_INVALID, "bad server parameters");
  *out   = nullptr;
  auto S = std::make_unique<adv_server>();
  S->budget         = memory_budget_bytes;
  S->steps_per_tick = steps_per_tick;
  S->max_active     = max_active;
  S->keep_solutions = keep_solutions;
  adv::lsrk_coefficients(ADV_LSRK_5_4, S->ai, S->bi);
  ADV_CUDA(cudaGetDevice(&S->device));
  if (int e = adv::detail::ensure_tables(S->device))
    return e;
  *out = S.release();
  return ADV_OK;
}

int adv_server_set_policy(adv_server *S, int policy)
{
  if (!S || (policy != ADV_SERVE_FIFO && policy != ADV_SERVE_SHORTEST_FIRST))
    return fail(ADV_ERR_INVALID, "unknown admission policy");
  S->policy = policy;
  return ADV_OK;
}

int adv_server_destroy(adv_server *S)
{
  if (!S)
    return ADV_OK;
  for (auto &kv : S->groups)
    cudaStreamSynchronize(kv.second.stream);
  for (auto &q : S->reqs)
    {
      cudaFree(q.u);
      cudaFree(q.r);
      cudaFree(q.k);
      cudaFree(q.t0);
      cudaFree(q.t1);
    }
  for (auto &kv : S->groups)
    {
      SGroup &g = kv.second;
      if (g.exec)
        cudaGraphExecDestroy(g.exec);
      cudaFree(g.d_slots);
      cudaFreeHost(g.h_slots);
      cudaFree(g.d_counts);
      cudaFree(g.d_cta_slot);
      cudaFree(g.d_cta_cell0);
      cudaFree(g.d_partials);
      cudaEventDestroy(g.event);
      cudaStreamDestroy(g.stream);
    }
  delete S;
  return ADV_OK;
}

int adv_server_submit(adv_server *S, const adv_config *cfg, double t_end, double courant, int64_t *request_id)
{
  if (!S || !cfg || !request_id)
    return fail(ADV_ERR_INVALID, "null argument");
  const adv_config &c = *cfg;
  if (c.mesh_type != ADV_MESH_CARTESIAN || !c.periodic || c.velocity_type != ADV_VELOCITY_CONSTANT ||
      c.diffusion != 0.0 || c.factor_skew != 0.0)
    return fail(ADV_ERR_INVALID, "the serving loop takes affine periodic meshes with constant velocity, "
                                 "conservative form, no diffusion");
  if (c.n_cells[0] != c.n_cells[1] || c.n_cells[1] != c.n_cells[2] || c.n_cells[0] < 1)
    return fail(ADV_ERR_INVALID, "the serving loop takes n^3 meshes");
  if (c.degree < 1 || c.degree > 6)
    return fail(ADV_ERR_INVALID, "degree must be in 1..6");
  if (c.precision != ADV_PRECISION_FP64 && c.precision != ADV_PRECISION_FP32_OPERATOR)
    return fail(ADV_ERR_INVALID, "unknown precision");
  if (!(t_end > 0.0) || !(courant > 0.0))
    return fail(ADV_ERR_INVALID, "t_end and courant must be positive");
  const double anorm = std::sqrt(c.velocity[0] * c.velocity[0] + c.velocity[1] * c.velocity[1] +
                                 c.velocity[2] * c.velocity[2]);
  if (!(anorm > 0.0))
    return fail(ADV_ERR_INVALID, "zero velocity");
  SReq q;
  q.cfg       = c;
  q.t_end     = t_end;
  q.courant   = courant;
  q.n         = c.n_cells[0];
  q.npts      = c.degree + 1;
  q.precision = c.precision;
  q.n_dofs    = (int64_t)q.n * q.n * q.n * q.npts * q.npts * q.npts;
  q.bytes     = 3 * q.n_dofs * (int64_t)sizeof(double);
  if (adv::batch_collocation(q.precision)) // two face-trace buffers of 6 n^2 values per cell
    q.bytes += 2 * 6 * (q.n_dofs / q.npts) * (int64_t)sizeof(double);
  adv::Mesh m;
  adv::setup_mesh(c, m);
  adv::Tables1D tb;
  tb.init(c.degree);
  adv::detail::make_diag(c, m, tb, q.diag);
  double hmin = m.h[0];
  for (int d = 0; d < 3; ++d)
    {
      hmin   = std::min(hmin, m.h[d]);
      q.cv[d] = c.velocity[d] / m.h[d];
      q.P[d]  = 0.5 * (q.cv[d] + c.flux_alpha * std::fabs(q.cv[d]));
      q.M[d]  = 0.5 * (q.cv[d] - c.flux_alpha * std::fabs(q.cv[d]));
    }
  // time step rule and rounding of setup_dofs (advection_solver.cc:1155-1167)
  const double dt0 = courant * hmin / anorm / std::pow(std::max(1, c.degree), 1.5);
  q.steps          = std::max(1, (int)std::ceil(t_end / dt0 - 1e-12));
  q.dt             = t_end / q.steps;
  q.t_submit       = now_s();
  if (q.bytes > S->budget)
    return fail(ADV_ERR_OUT_OF_MEMORY, "the request alone exceeds the memory budget");
  *request_id = (int64_t)S->reqs.size();
  S->reqs.push_back(std::move(q));
  S->queue.push_back(*request_id);
  return ADV_OK;
}

// One scheduling round: retire solves of finished ticks, admit waiting
// requests within the budget, start the next tick of every idle group.
int adv_server_poll(adv_server *S, int *n_completed)
{
  if (!S)
    return fail(ADV_ERR_INVALID, "null argument");
  int cur = -1;
  ADV_CUDA(cudaGetDevice(&cur));
  if (cur != S->device)
    return fail(ADV_ERR_INVALID, "server created on another device than the current one");
  int done = 0;
  for (auto &kv : S->groups)
    {
      SGroup &g = kv.second;
      if (!g.in_flight)
        continue;
      const cudaError_t q = cudaEventQuery(g.event);
      if (q == cudaErrorNotReady)
        continue;
      if (q != cudaSuccess)
        return adv::detail::cuda_fail(q, "tick of a serving group");
      g.in_flight = false;
      std::vector<int64_t> keep;
      for (size_t i = 0; i < g.members.size(); ++i)
        {
          if (i >= g.launched)
            {
              keep.push_back(g.members[i]); // admitted during the tick
              continue;
            }
          SReq &r      = S->reqs[g.members[i]];
          r.steps_done = g.h_slots[i].steps_done;
          if (r.cancel)
            {
              if (int e = drop(S, g, g.members[i]))
                return e;
              ++done;
            }
          else if (r.steps_done >= r.steps)
            {
              if (int e = retire(S, g, g.members[i]))
                return e;
              ++done;
            }
          else
            keep.push_back(g.members[i]);
        }
      g.members.swap(keep);
    }
  while (!S->queue.empty() && S->active < S->max_active)
    {
      auto pick = S->queue.begin();
      if (S->policy == ADV_SERVE_SHORTEST_FIRST)
        {
          // the queued request with the least work (DoFs x steps)
          for (auto it = S->queue.begin(); it != S->queue.end(); ++it)
            {
              const SReq &a = S->reqs[*it], &b = S->reqs[*pick];
              if ((double)a.n_dofs * a.steps < (double)b.n_dofs * b.steps)
                pick = it;
            }
        }
      const int64_t id = *pick;
      if (S->used + S->reqs[id].bytes > S->budget)
        break;
      S->queue.erase(pick);
      if (int e = admit(S, id))
        return e;
    }
  for (auto &kv : S->groups)
    {
      SGroup &g = kv.second;
      if (g.in_flight || g.members.empty())
        continue;
      if (g.dirty)
        if (int e = rebuild(S, g))
          return e;
      ADV_CUDA(cudaGraphLaunch(g.exec, g.stream));
      ADV_CUDA(cudaMemcpyAsync(g.h_slots, g.d_slots, g.members.size() * sizeof(adv::BatchSlot),
                               cudaMemcpyDeviceToHost, g.stream));
      ADV_CUDA(cudaEventRecord(g.event, g.stream));
      g.in_flight = true;
      g.launched  = g.members.size();
      ++S->ticks;
      S->launches += (int64_t)S->steps_per_tick * ((int64_t)S->bi.size() + 1);
    }
  if (n_completed)
    *n_completed = done;
  return ADV_OK;
}

int adv_server_cancel(adv_server *S, int64_t id)
{
  if (!S || id < 0 || id >= (int64_t)S->reqs.size())
    return fail(ADV_ERR_INVALID, "unknown request");
  SReq &q = S->reqs[id];
  if (q.state == 0)
    {
      for (auto it = S->queue.begin(); it != S->queue.end(); ++it)
        if (*it == id)
          {
            S->queue.erase(it);
            break;
          }
      q.state  = 4;
      q.t_done = now_s();
      ++S->completed;
      return ADV_OK;
    }
  if (q.state == 1)
    {
      q.cancel = true; // leaves at the end of its group's current tick
      return ADV_OK;
    }
  return fail(ADV_ERR_INVALID, "request already finished");
}

int adv_server_drain(adv_server *S)
{
  if (!S)
    return fail(ADV_ERR_INVALID, "null argument");
  while (S->completed < (int64_t)S->reqs.size())
    if (int e = adv_server_poll(S, nullptr))
      return e;
  return ADV_OK;
}

int adv_server_result(adv_server *S, int64_t id, int *state, double *rel_l2_error, double *latency_s, int *steps,
                      double *dt)
{
  if (!S || id < 0 || id >= (int64_t)S->reqs.size())
    return fail(ADV_ERR_INVALID, "unknown request");
  const SReq &q = S->reqs[id];
  if (state)
    *state = q.state;
  if (rel_l2_error)
    *rel_l2_error = q.rel_l2;
  if (latency_s)
    *latency_s = q.state == 2 ? q.t_done - q.t_submit : -1.0;
  if (steps)
    *steps = q.steps;
  if (dt)
    *dt = q.dt;
  return ADV_OK;
}

int adv_server_solution(adv_server *S, int64_t id, double *host_out, int64_t n)
{
  if (!S || !host_out || id < 0 || id >= (int64_t)S->reqs.size())
    return fail(ADV_ERR_INVALID, "unknown request");
  const SReq &q = S->reqs[id];
  if (q.state != 2 || (int64_t)q.solution.size() != n)
    return fail(ADV_ERR_INVALID, "no stored solution of that size (keep_solutions off or request not done)");
  std::memcpy(host_out, q.solution.data(), n * sizeof(double));
  return ADV_OK;
}

int adv_server_stats(const adv_server *S, int64_t *out)
{
  if (!S || !out)
    return fail(ADV_ERR_INVALID, "null argument");
  out[0] = (int64_t)S->reqs.size();
  out[1] = (int64_t)S->queue.size();
  out[2] = S->active;
  out[3] = S->completed;
  out[4] = S->used;
  out[5] = S->budget;
  out[6] = S->ticks;
  out[7] = S->launches;
  return ADV_OK;
}

} // extern "C"
