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
  const int64_t *tile_start;   // [n_out] first work item of output o (tiles x K chunks)
  const int64_t *c_off;        // output block offsets
  void *C;
  int64_t n_out;
  // split-K of the native kernel (all NULL: one chunk per tile)
  const int32_t *chunks;       // per output: K chunks per tile
  const int64_t *kfused;       // per output: fused K (sum of k over its pairs)
  const int64_t *split_off;    // per output: first partial tile (64x64) in scratch
  void *scratch;
};

// Work list of one native launch: which outputs, how many K chunks each.
struct NativeWork {
  int64_t n_work = 0;          // CTAs of the GEMM launch
  int64_t n_split = 0;         // output tiles reduced from partials
  const int64_t *work_start = nullptr, *split_start = nullptr, *split_off = nullptr;
  const int32_t *chunks = nullptr;
  const int64_t *kfused = nullptr;
  void *scratch = nullptr;
};

constexpr int NT_TM = 64, NT_TN = 64, NT_TK = 16, NT_THREADS = 256;

// Native-precision grouped GEMM: C_o = sum over the pairs of o of A_rep B_rep^T.
// With split-K (job.chunks set) chunked tiles write partials that a second
// kernel sums in chunk order (w.split_start: [n_out] first reduced tile).
tq_status launch_gemm_native(const GemmJob &job, int64_t n_tiles, tq_dtype dt, cudaStream_t s,
                             const NativeWork *w = nullptr);

// Rank-0 results: the sum over all pairs of dot(A_sub, B_sub) (the reference's
// cublas?dot + add<<<1,1>>> path, src/gpu/block_sparse.cuh:979-1010), as
// fixed-order partial sums followed by one fixed-order reduction.
tq_status launch_dot_native(const GemmJob &job, int64_t n_pairs, const int64_t *chunk_start,
                            int64_t n_chunks, void *partials, tq_dtype dt, cudaStream_t s);

constexpr int64_t DOT_CHUNK = 4096;

}  // namespace tq
