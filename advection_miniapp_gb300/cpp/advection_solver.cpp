// GPU counterpart of the reference program advection_solver.cc: the same
// problem driver (AdvectionProblem::run, advection_solver.cc:1246-1318) and
// main() (advection_solver.cc:1323-1372), written against the reference's
// call surface in advection_gb300.hpp.
//
//   advection_solver [refinements=3] [degree=3] [steps=200] [deformed=0] [fp32=0]
//
// refinements r gives 2^r cells per direction of the unit cube (the
// reference's refine_global); the run is periodic with velocity
// (1, 0.15, -0.05), upwind flux, LSRK(5,4) and Courant 0.5 / k^1.5.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <exception>

#include "advection_gb300.hpp"

using namespace advection_gb300;

int main(int argc, char **argv)
{
  try
    {
      const int refinements = argc > 1 ? std::atoi(argv[1]) : 3;
      const int degree      = argc > 2 ? std::atoi(argv[2]) : 3;
      const int steps       = argc > 3 ? std::atoi(argv[3]) : 200;
      const int deformed    = argc > 4 ? std::atoi(argv[4]) : 0;
      const int fp32        = argc > 5 ? std::atoi(argv[5]) : 0;

      adv_config cfg;
      adv_config_default(&cfg);
      cfg.degree = degree;
      for (int d = 0; d < 3; ++d)
        cfg.n_cells[d] = 1 << refinements;
      if (deformed)
        {
          cfg.mesh_type   = ADV_MESH_DEFORMED;
          cfg.deformation = 0.08;
        }
      cfg.precision = fp32 ? ADV_PRECISION_FP32_OPERATOR : ADV_PRECISION_FP64;

      AdvectionOperation advection_operator(cfg);
      const double       time_step = advection_operator.time_step(0.5);
      std::printf("   Number of elements:            %d\n", cfg.n_cells[0] * cfg.n_cells[1] * cfg.n_cells[2]);
      std::printf("   Polynomial degree:             %d\n", degree);
      std::printf("   Number of degrees of freedom:  %lld\n", (long long)advection_operator.n_dofs());
      std::printf("   Time step size: %.10g\n\n", time_step);

      DeviceVector solution, rk_register_1, rk_register_2;
      advection_operator.initialize_dof_vector(solution);
      advection_operator.initialize_dof_vector(rk_register_1);
      advection_operator.initialize_dof_vector(rk_register_2);
      advection_operator.project_initial(solution);

      auto output = [&](double time) {
        const auto err = advection_operator.l2_error(solution, time);
        const auto me  = advection_operator.compute_mass_and_energy(solution);
        std::printf("   Time %8.3g  error %.10e  mass %16.10g  energy %16.10g  H1-semi %9.4g\n", time,
                    err.first / err.second, me[0], me[1], me[2]);
      };
      output(0.0);

      const LowStorageRungeKuttaIntegrator time_integrator(ADV_LSRK_5_4);
      double                               time = 0.0, wtime = 0.0;
      for (int step = 0; step < steps; ++step)
        {
          const auto t0 = std::chrono::steady_clock::now();
          time_integrator.perform_time_step(advection_operator, time, time_step, solution, rk_register_1,
                                            rk_register_2);
          cudaStreamSynchronize(advection_operator.stream());
          wtime += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
          time += time_step;
        }
      output(time);
      std::printf("\n   Performed %d time steps.\n", steps);
      std::printf("   Average wall clock time per time step: %gs, time per element: %gs\n", wtime / steps,
                  wtime / steps / (double(cfg.n_cells[0]) * cfg.n_cells[1] * cfg.n_cells[2]));
    }
  catch (std::exception &exc)
    {
      std::fprintf(stderr, "Exception on processing: \n%s\nAborting!\n", exc.what());
      return 1;
    }
  return 0;
}
