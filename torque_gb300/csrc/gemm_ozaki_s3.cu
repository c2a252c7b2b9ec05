// Instantiations of the sliced GEMM kernel for slice specialisation S = 3 (three-way bf16 split).
#include "oz_gemm.cuh"

namespace tq {
tq_status oz_gemm_set_attr_s3() { return oz_gemm_set_attr<3>(); }
tq_status oz_gemm_run_s3(const OzLaunch &L, unsigned grid, cudaStream_t st) {
  return oz_gemm_run<3>(L, grid, st);
}
}  // namespace tq
