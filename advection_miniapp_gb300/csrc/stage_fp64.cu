// Instantiations of the fused stage kernel with a binary64 operator.
#include "stage_kernel.cuh"

namespace adv
{
cudaError_t upload_tables_stage64(const DevTables<double> *d, const DevTables<float> *f)
{
  return upload_tables_local(d, f);
}

cudaError_t launch_stage_fp64(int n, const StageArgs &args, cudaStream_t stream)
{
  switch (n)
    {
      case 2: return launch_stage_n<2, double>(args, stream);
      case 3: return launch_stage_n<3, double>(args, stream);
      case 4: return launch_stage_n<4, double>(args, stream);
      case 5: return launch_stage_n<5, double>(args, stream);
      case 6: return launch_stage_n<6, double>(args, stream);
      case 7: return launch_stage_n<7, double>(args, stream);
      default: return cudaErrorInvalidValue;
    }
}

int stage_cells_per_block_fp64(int n)
{
  switch (n)
    {
      case 2: return stage_cells<2, double>();
      case 3: return stage_cells<3, double>();
      case 4: return stage_cells<4, double>();
      case 5: return stage_cells<5, double>();
      case 6: return stage_cells<6, double>();
      case 7: return stage_cells<7, double>();
      default: return 0;
    }
}
} // namespace adv
