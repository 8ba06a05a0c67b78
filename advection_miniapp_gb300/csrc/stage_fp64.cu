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
      case 2: return launch_stage_t<2, double>(args, stream);
      case 3: return launch_stage_t<3, double>(args, stream);
      case 4: return launch_stage_t<4, double>(args, stream);
      case 5: return launch_stage_t<5, double>(args, stream);
      case 6: return launch_stage_t<6, double>(args, stream);
      case 7: return launch_stage_t<7, double>(args, stream);
      default: return cudaErrorInvalidValue;
    }
}

int stage_cells_per_block_fp64(int n)
{
  switch (n)
    {
      case 2: return StageShape<2, double>::C;
      case 3: return StageShape<3, double>::C;
      case 4: return StageShape<4, double>::C;
      case 5: return StageShape<5, double>::C;
      case 6: return StageShape<6, double>::C;
      case 7: return StageShape<7, double>::C;
      default: return 0;
    }
}
} // namespace adv
