// hcc_stage_f32_r2.cu — stage kernels, float arithmetic, reconstruction degree 2.
#include "hcc_stage_impl.cuh"
namespace hcc {
const StageOps *stage_ops_f32_r2(int D, int M, int pde) { return lookup_rdeg<float, 2>(D, M, pde); }
}  // namespace hcc
