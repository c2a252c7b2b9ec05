// Work description of the grouped block GEMM: one launch covers every output
// block of a contraction (or of a batch of contractions).
#pragma once
#include "geometry.cuh"

namespace tq {

// One contraction instance of a (possibly batched) launch.
struct GemmJob {
  DevBS A, B;
  LegSpec L;
  const int32_t *pa, *pb;      // matched pairs, reference order
  const int64_t *seg;          // [n_out+1] pairs of output o: perm[seg[o]..seg[o+1])
  const int64_t *perm;         // NULL: identity (reference layout)
  const int64_t *tile_start;   // [n_out+1] first tile of output o
  const int64_t *c_off;        // output block offsets
  void *C;
  int64_t n_out;
};

constexpr int NT_TM = 64, NT_TN = 64, NT_TK = 16, NT_THREADS = 256;

// Native-precision grouped GEMM: C_o = sum over the pairs of o of A_rep B_rep^T.
tq_status launch_gemm_native(const GemmJob &job, int64_t n_tiles, tq_dtype dt, cudaStream_t s);

// Rank-0 results: the sum over all pairs of dot(A_sub, B_sub) (the reference's
// cublas?dot + add<<<1,1>>> path, src/gpu/block_sparse.cuh:979-1010), as
// fixed-order partial sums followed by one fixed-order reduction.
tq_status launch_dot_native(const GemmJob &job, int64_t n_pairs, const int64_t *chunk_start,
                            int64_t n_chunks, void *partials, tq_dtype dt, cudaStream_t s);

constexpr int64_t DOT_CHUNK = 4096;

}  // namespace tq
