// hcc_stage_f64_r1.cu — stage kernels, double arithmetic, reconstruction degree 1.
#include "hcc_stage_impl.cuh"
namespace hcc {
const StageOps *stage_ops_f64_r1(int D, int M, int pde) { return lookup_rdeg<double, 1>(D, M, pde); }
}  // namespace hcc
