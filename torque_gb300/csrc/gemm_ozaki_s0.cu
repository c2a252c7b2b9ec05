// Instantiations of the sliced GEMM kernel for slice specialisation S = 0 (any slice count, chosen per job).
#include "oz_gemm.cuh"

namespace tq {
tq_status oz_gemm_set_attr_s0() { return oz_gemm_set_attr<0>(); }
tq_status oz_gemm_run_s0(const OzLaunch &L, unsigned grid, cudaStream_t st) {
  return oz_gemm_run<0>(L, grid, st);
}
}  // namespace tq
