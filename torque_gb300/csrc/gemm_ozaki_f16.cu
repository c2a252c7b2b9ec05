// Instantiations of the tensor-core GEMM kernel for binary16 operands
// (kind::f16 with fp16 A and B, fp32 accumulation).
#include "oz_gemm.cuh"

namespace tq {
tq_status oz_gemm_set_attr_f16() { return oz_gemm_set_attr<OZ_F16>(); }
tq_status oz_gemm_run_f16(const OzLaunch &L, unsigned grid, cudaStream_t st) {
  return oz_gemm_run<OZ_F16>(L, grid, st);
}
}  // namespace tq
