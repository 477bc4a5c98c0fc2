// hcc_stage_f32_r1.cu — stage kernels, float arithmetic, reconstruction degree 1.
#include "hcc_stage_impl.cuh"
namespace hcc {
const StageOps *stage_ops_f32_r1(int D, int M, int pde) { return lookup_rdeg<float, 1>(D, M, pde); }
}  // namespace hcc
