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
      case 2: return launch_stage_t<2, float>(args, stream);
      case 3: return launch_stage_t<3, float>(args, stream);
      case 4: return launch_stage_t<4, float>(args, stream);
      case 5: return launch_stage_t<5, float>(args, stream);
      case 6: return launch_stage_t<6, float>(args, stream);
      case 7: return launch_stage_t<7, float>(args, stream);
      default: return cudaErrorInvalidValue;
    }
}

int stage_cells_per_block_fp32(int n)
{
  switch (n)
    {
      case 2: return StageShape<2, float>::C;
      case 3: return StageShape<3, float>::C;
      case 4: return StageShape<4, float>::C;
      case 5: return StageShape<5, float>::C;
      case 6: return StageShape<6, float>::C;
      case 7: return StageShape<7, float>::C;
      default: return 0;
    }
}
} // namespace adv
