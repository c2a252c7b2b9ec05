// Per-pair geometry shared by the GEMM kernels: the matrix views of the two
// operand sub-boxes of a matched block pair.
//
// The reference builds, for A block i and B block j, the matrices
//   A_rep (m x k): rows over A's free legs (column-major, ascending legs),
//                  columns over the contracted legs in pair order;
//   B_rep (n x k): the same for B;
// and stores C = A_rep * B_rep^T column-major as the output block
// (src/tensor/block_sparse.h:17-80, :527-551; src/gpu/block_sparse.cuh:700-930).
// Here the views are read in place from the block data through their strides;
// legs whose strides are contiguous are merged so that the common layouts
// become a plain 2-D strided matrix.
#pragma once
#include "tq_internal.h"

namespace tq {

struct Operand {
  int64_t base;  // element offset of the sub-box origin in the tensor data
  int64_t rows, cols;
  int32_t nr, nc;  // legs left after merging
  int64_t rdim[TQ_MAXR], rst[TQ_MAXR];
  int64_t cdim[TQ_MAXR], cst[TQ_MAXR];
};

// Intersection of the contracted intervals of A block i and B block j, pair order.
__device__ __forceinline__ void contraction_range(const DevBS &A, const DevBS &B,
                                                  const LegSpec &L, int64_t i, int64_t j,
                                                  int64_t *cb, int64_t *ce) {
  for (int k = 0; k < L.nc; k++) {
    const int64_t ab = A.begin[i * A.rank + L.al[k]], bb = B.begin[j * B.rank + L.bl[k]];
    const int64_t ae = A.end[i * A.rank + L.al[k]], be = B.end[j * B.rank + L.bl[k]];
    cb[k] = ab > bb ? ab : bb;
    ce[k] = ae < be ? ae : be;
  }
}

__device__ __forceinline__ void merge_legs(int32_t &n, int64_t *dim, int64_t *st) {
  int32_t w = 0;
  for (int32_t q = 0; q < n; q++) {
    if (dim[q] == 1) continue;
    if (w > 0 && st[q] == st[w - 1] * dim[w - 1]) {
      dim[w - 1] *= dim[q];
    } else {
      dim[w] = dim[q];
      st[w] = st[q];
      w++;
    }
  }
  n = w;
}

// Operand view of block `blk` of T: rows over its free legs (full block range),
// columns over the contracted legs con[0..ncon) restricted to [cb, ce].
__device__ __forceinline__ void build_operand(const DevBS &T, int64_t blk, int32_t nfree,
                                              const int32_t *free_legs, int32_t ncon,
                                              const int32_t *con, const int64_t *cb,
                                              const int64_t *ce, Operand &op) {
  const int64_t *b = T.begin + blk * T.rank;
  const int64_t *e = T.end + blk * T.rank;
  const int64_t *s = T.strides + blk * T.rank;
  op.base = T.offsets[blk];
  op.rows = 1;
  op.cols = 1;
  op.nr = nfree;
  for (int32_t q = 0; q < nfree; q++) {
    op.rdim[q] = e[free_legs[q]] - b[free_legs[q]] + 1;
    op.rst[q] = s[free_legs[q]];
    op.rows *= op.rdim[q];
  }
  op.nc = ncon;
  for (int32_t k = 0; k < ncon; k++) {
    op.cdim[k] = ce[k] - cb[k] + 1;
    op.cst[k] = s[con[k]];
    op.base += (cb[k] - b[con[k]]) * s[con[k]];
    op.cols *= op.cdim[k];
  }
  merge_legs(op.nr, op.rdim, op.rst);
  merge_legs(op.nc, op.cdim, op.cst);
}

__device__ __forceinline__ int64_t mixed_addr(int64_t x, int32_t n, const int64_t *dim,
                                              const int64_t *st) {
  if (n == 0) return 0;
  if (n == 1) return x * st[0];
  int64_t a = 0;
  for (int32_t q = 0; q < n; q++) {
    const int64_t d = dim[q];
    a += (x % d) * st[q];
    x /= d;
  }
  return a;
}

// Single row / column stride when the merged view is 2-D (else -1).
__device__ __forceinline__ int64_t row_stride(const Operand &op) {
  return op.nr == 0 ? 0 : (op.nr == 1 ? op.rst[0] : -1);
}
__device__ __forceinline__ int64_t col_stride(const Operand &op) {
  return op.nc == 0 ? 0 : (op.nc == 1 ? op.cst[0] : -1);
}

}  // namespace tq
