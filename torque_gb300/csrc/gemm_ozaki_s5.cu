// Instantiations of the sliced GEMM kernel for slice specialisation S = 5 (the FP64-level default).
#include "oz_gemm.cuh"

namespace tq {
tq_status oz_gemm_set_attr_s5() { return oz_gemm_set_attr<5>(); }
tq_status oz_gemm_run_s5(const OzLaunch &L, unsigned grid, cudaStream_t st) {
  return oz_gemm_run<5>(L, grid, st);
}
}  // namespace tq
