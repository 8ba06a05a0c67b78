// Instantiations of the fused stage kernel with a binary32 operator.
#include "stage_kernel.cuh"

namespace adv
{
cudaError_t upload_tables_stage32(const DevTables<double> *d, const DevTables<float> *f)
{
  return upload_tables_local(d, f);
}

cudaError_t launch_stage_fp32(int n, const StageArgs &args, cudaStream_t stream)
{
  switch (n)
    {
      case 2: return launch_stage_n<2, float>(args, stream);
      case 3: return launch_stage_n<3, float>(args, stream);
      case 4: return launch_stage_n<4, float>(args, stream);
      case 5: return launch_stage_n<5, float>(args, stream);
      case 6: return launch_stage_n<6, float>(args, stream);
      case 7: return launch_stage_n<7, float>(args, stream);
      default: return cudaErrorInvalidValue;
    }
}

int stage_cells_per_block_fp32(int n)
{
  switch (n)
    {
      case 2: return stage_cells<2, float>();
      case 3: return stage_cells<3, float>();
      case 4: return stage_cells<4, float>();
      case 5: return stage_cells<5, float>();
      case 6: return stage_cells<6, float>();
      case 7: return stage_cells<7, float>();
      default: return 0;
    }
}
} // namespace adv
