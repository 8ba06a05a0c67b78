// Instantiations of the collocation-form stage kernel with a binary32
// operator (binary64 vectors).
#include "stage_gauss.cuh"

namespace adv
{
cudaError_t upload_tables_gauss32(const DevTables<double> *d, const DevTables<float> *f)
{
  return upload_tables_local(d, f);
}

cudaError_t launch_stage_gauss_fp32(int n, const StageArgs &args, cudaStream_t stream)
{
  return launch_stage_gauss_any<float>(n, args, stream);
}
} // namespace adv
