// C++ call surface of the reference miniapp over the advection_gb300 C ABI.
//
// AdvectionOperation and LowStorageRungeKuttaIntegrator keep the member
// functions, argument order and meaning of the reference classes
// (kronbichler/advection_miniapp, advection_solver.cc:329-431 and 822-944),
// so code written against them compiles against this header with
// DeviceVector in place of LinearAlgebra::distributed::Vector<double>.
// Errors are reported by exceptions like the reference's AssertThrow
// (advection_solver.cc:1344-1369); the C ABI below never throws.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "advection_gb300.h"

namespace advection_gb300
{
inline void check(int code, const char *where)
{
  if (code != ADV_OK)
    throw std::runtime_error(std::string(where) + " failed: " + adv_last_error());
}

// Owning FP64 device vector in the operator's DoF layout.
class DeviceVector
{
public:
  DeviceVector() = default;
  DeviceVector(const DeviceVector &) = delete;
  DeviceVector &operator=(const DeviceVector &) = delete;
  DeviceVector(DeviceVector &&o) noexcept { *this = std::move(o); }
  DeviceVector &operator=(DeviceVector &&o) noexcept
  {
    std::swap(ptr_, o.ptr_);
    std::swap(size_, o.size_);
    return *this;
  }
  ~DeviceVector()
  {
    if (ptr_)
      cudaFree(ptr_);
  }
  void reinit(int64_t n)
  {
    if (ptr_)
      cudaFree(ptr_);
    ptr_  = nullptr;
    size_ = n;
    if (cudaMalloc(&ptr_, n * sizeof(double)) != cudaSuccess)
      throw std::runtime_error("cudaMalloc of a DoF vector failed");
    cudaMemset(ptr_, 0, n * sizeof(double));
  }
  double       *data() { return ptr_; }
  const double *data() const { return ptr_; }
  int64_t       size() const { return size_; }
  // swap of the storage, like LinearAlgebra::distributed::Vector::swap
  void swap(DeviceVector &o) noexcept
  {
    std::swap(ptr_, o.ptr_);
    std::swap(size_, o.size_);
  }
  std::vector<double> to_host() const
  {
    std::vector<double> h(size_);
    if (cudaMemcpy(h.data(), ptr_, size_ * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      throw std::runtime_error("cudaMemcpy to host failed");
    return h;
  }

private:
  double *ptr_  = nullptr;
  int64_t size_ = 0;
};

// AdvectionOperation (advection_solver.cc:329-431) on the GPU.
class AdvectionOperation
{
public:
  AdvectionOperation() = default;
  explicit AdvectionOperation(const adv_config &cfg) { reinit(cfg); }
  AdvectionOperation(const AdvectionOperation &) = delete;
  AdvectionOperation &operator=(const AdvectionOperation &) = delete;
  ~AdvectionOperation()
  {
    if (h_)
      adv_destroy(h_);
  }

  // reinit(dof_handler) in the reference: mesh and geometry come from cfg here
  void reinit(const adv_config &cfg)
  {
    if (h_)
      adv_destroy(h_);
    h_ = nullptr;
    check(adv_create(&cfg, &h_), "adv_create");
    check(adv_n_dofs(h_, &n_dofs_), "adv_n_dofs");
  }

  void    set_stream(cudaStream_t s) { stream_ = s; }
  int64_t n_dofs() const { return n_dofs_; }

  void initialize_dof_vector(DeviceVector &vec) const { vec.reinit(n_dofs_); }

  void apply(const DeviceVector &src, DeviceVector &dst, const double current_time) const
  {
    check(adv_apply(h_, src.data(), dst.data(), current_time, stream_), "apply");
  }

  void perform_stage(const double current_time, const double factor_solution, const double factor_ai,
                     const DeviceVector &current_ri, DeviceVector &vec_ki, DeviceVector &solution,
                     DeviceVector &next_ri) const
  {
    check(adv_perform_stage(h_, current_time, factor_solution, factor_ai, current_ri.data(),
                            vec_ki.data(), solution.data(), next_ri.data(), stream_),
          "perform_stage");
  }

  void project_initial(DeviceVector &dst) const
  {
    check(adv_project(h_, 0.0, dst.data(), stream_), "project_initial");
  }

  std::array<double, 3> compute_mass_and_energy(const DeviceVector &vec) const
  {
    std::array<double, 3> out{};
    check(adv_mass_energy(h_, vec.data(), out.data(), stream_), "compute_mass_and_energy");
    return out;
  }

  // (||u_h - u(t)||, ||u(t)||) as in output_results (advection_solver.cc:1183-1208)
  std::pair<double, double> l2_error(const DeviceVector &vec, const double t) const
  {
    double out[2];
    check(adv_l2_error(h_, vec.data(), t, out, stream_), "l2_error");
    return {out[0], out[1]};
  }

  double time_step(const double courant) const
  {
    double dt = 0;
    check(adv_time_step(h_, courant, &dt), "time_step");
    return dt;
  }

  // output_results (advection_solver.cc:1220-1241)
  void write_vtu(const DeviceVector &vec, const double t, const std::string &path) const
  {
    check(adv_write_vtu(h_, vec.data(), t, path.c_str(), stream_), "write_vtu");
  }
  void save_state(const DeviceVector &vec, const double t, const std::string &path) const
  {
    check(adv_save_state(h_, vec.data(), t, path.c_str(), stream_), "save_state");
  }
  double load_state(DeviceVector &vec, const std::string &path) const
  {
    double t = 0;
    check(adv_load_state(h_, vec.data(), &t, path.c_str(), stream_), "load_state");
    return t;
  }

  adv_handle  *handle() const { return h_; }
  cudaStream_t stream() const { return stream_; }

private:
  adv_handle  *h_      = nullptr;
  int64_t      n_dofs_ = 0;
  cudaStream_t stream_ = nullptr;
};

// LowStorageRungeKuttaIntegrator (advection_solver.cc:822-944).
class LowStorageRungeKuttaIntegrator
{
public:
  explicit LowStorageRungeKuttaIntegrator(const int scheme)
    : scheme_(scheme)
  {
    int n = 0;
    check(adv_lsrk_coefficients(scheme, nullptr, nullptr, &n), "adv_lsrk_coefficients");
    bi_.resize(n);
    ai_.resize(n - 1);
    check(adv_lsrk_coefficients(scheme, ai_.data(), bi_.data(), &n), "adv_lsrk_coefficients");
  }

  unsigned int n_stages() const { return bi_.size(); }

  // The GPU operator runs the whole step in the library (fused stages with
  // buffer rotation, no copies).
  void perform_time_step(const AdvectionOperation &op, const double current_time, const double time_step,
                         DeviceVector &solution, DeviceVector &vec_ri, DeviceVector &vec_ki) const
  {
    check(adv_lsrk_step(op.handle(), scheme_, current_time, time_step, solution.data(), vec_ri.data(),
                        vec_ki.data(), op.stream()),
          "perform_time_step");
  }

  // n_steps steps on a solution in host memory (page-locked for the copies
  // to overlap): copied in, advanced and copied back (adv_lsrk_steps_host);
  // host_solution holds the result once the operator's stream has passed it.
  void perform_time_steps_host(const AdvectionOperation &op, const double current_time, const double time_step,
                               const int n_steps, double *host_solution, DeviceVector &solution,
                               DeviceVector &vec_ri, DeviceVector &vec_ki) const
  {
    check(adv_lsrk_steps_host(op.handle(), scheme_, current_time, time_step, n_steps, host_solution,
                              solution.data(), vec_ri.data(), vec_ki.data(), op.stream()),
          "perform_time_steps_host");
  }

  // Any other operator with the reference's perform_stage gets the
  // reference's stage loop (advection_solver.cc:906-939).
  template <typename VectorType, typename Operator>
  void perform_time_step(const Operator &pde_operator, const double current_time, const double time_step,
                         VectorType &solution, VectorType &vec_ri, VectorType &vec_ki) const
  {
    pde_operator.perform_stage(current_time, bi_[0] * time_step, ai_[0] * time_step, solution, vec_ri,
                               solution, vec_ri);
    double sum_previous_bi = 0;
    for (unsigned int stage = 1; stage < bi_.size(); ++stage)
      {
        const double c_i = sum_previous_bi + ai_[stage - 1];
        pde_operator.perform_stage(current_time + c_i * time_step, bi_[stage] * time_step,
                                   (stage == bi_.size() - 1 ? 0 : ai_[stage] * time_step), vec_ri, vec_ki,
                                   solution, vec_ri);
        sum_previous_bi += bi_[stage - 1];
      }
  }

private:
  int                 scheme_;
  std::vector<double> bi_, ai_;
};
} // namespace advection_gb300
