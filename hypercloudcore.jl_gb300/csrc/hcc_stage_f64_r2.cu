// hcc_stage_f64_r2.cu — stage kernels, double arithmetic, reconstruction degree 2.
#include "hcc_stage_impl.cuh"
namespace hcc {
const StageOps *stage_ops_f64_r2(int D, int M, int pde) { return lookup_rdeg<double, 2>(D, M, pde); }
}  // namespace hcc
