// Work description of the tensor-core (sliced) forms of the grouped GEMM.  A
// launch covers a batch of contractions ("jobs"): one contraction is a batch of
// one; many independent contractions share one persistent launch.
#pragma once
#include "gemm.cuh"

namespace tq {

constexpr int OZ_M = 128;        // output rows per tile (A side, TMEM lanes)
constexpr int OZ_N = 96;         // widest tile: output columns per tile (B side)
// tile widths the GEMM is instantiated for (the schedule's choice per launch)
constexpr int OZ_TILE_NS[3] = {32, 64, 96};
constexpr int OZ_BAND = 8;       // row tiles per band of the tile order
constexpr int OZ_CHUNK = 21;     // most k-steps of 16 an accumulator holds (K = 336)
constexpr int OZ_MAXS = 7;       // most slices supported
constexpr int OZ_MAX_STAGES = 8;
constexpr int OZ_EXP_ZERO = -(1 << 20);  // exponent of an all-zero row
// Binary16 operands take one product per 16-column k-step; OZ_F16_PACK
// consecutive k-steps are packed as the "slices" of one wider step (the same
// bytes in memory), so that one pipeline stage (two bulk copies and two
// barrier waits) carries that many MMAs: the producer's per-stage cost, not
// the tensor core, bounded the one-MMA stages.
constexpr int OZ_F16_PACK = 8;
// Five- and three-slice jobs (the FP64- and FP32-level forms) carry two
// 16-column k-steps per pipeline stage (30 or 12 MMAs per stage instead of 15
// or 6: a stage's fixed cost, a barrier round and two bulk copies, is then
// paid half as often); each accumulator holds at most OZ_CHUNK / 2 packed
// steps (320 columns, inside the 336-column bound of exact accumulation).
constexpr int OZ_PACK5 = 2;
__host__ __device__ constexpr int32_t oz_pack_for(int32_t s) {
  return s == 5 || s == 3 ? OZ_PACK5 : 1;
}
__host__ __device__ inline int32_t oz_pack_of(int32_t s, bool f16) {
  return f16 ? 1 : oz_pack_for(s);
}
// columns of K per (packed) step of a job
__host__ __device__ inline int64_t oz_kstep_cols(bool f16, int32_t pack) {
  return f16 ? 16 * OZ_F16_PACK : 16 * (int64_t)pack;
}

// Charge-class layout (when the contraction allows it).  Free boxes whose blocks
// carry the same set of matched contracted boxes form a class; when every pair of
// free boxes that match at all match on their whole sets, the contraction is a
// sum over classes of dense products R_c S_c^T, where R_c stacks the rows of all
// A free boxes of class c and its columns run over the class's contracted boxes
// (U(1) symmetry gives one class per charge sector).  The sliced operands are
// then stored per class, and an output tile spans several output blocks, so rows
// and columns are padded only at the end of a class, not of every block.
struct OzRowMap {   // one row of a class on one side (a virtual row)
  int64_t xoff;     // A side: index of the row's free box in the class's output-offset table
  int32_t xi;       // the row's free box, as its position in the class
  int32_t xr;       // row within that free box
  int32_t m;        // rows of that free box
  int32_t pad;
};

struct OzClassItem {  // one work item of the class-layout slicing pass
  int64_t unit;       // slice storage of the row tile, 256-byte units
  int64_t vrow0;      // first virtual row of the row tile
  int64_t blk_base;   // the class's entries in blk: [free box * nbox + box]
  int32_t koff, nk;   // k-step offset of the box within the class, its k-steps
  int32_t rows;       // rows of the row tile
  int32_t box, nbox;  // the contracted box, boxes of the class
  int32_t pad;
};

struct OzClassOut {  // one class as an output of the GEMM
  int64_t m, n;      // virtual rows (A side) and columns (B side)
  int64_t erow, ecol;  // first virtual row / column (also the exponent tables' index)
};

// One operand side (A or B) of one job, for the slicing passes: every block of
// the tensor is one operand unit viewed as a rows x k matrix (rows over the
// free legs, columns over the contracted legs in pair order, each block's full
// range).
struct OzSide {
  DevBS T;
  int32_t nfree, ncon;
  int32_t free_legs[TQ_MAXR], con[TQ_MAXR];
  const int64_t *key;         // free-box class key per block
  const int64_t *row_off;     // per key: first row in the exponent table
  const int64_t *row_start;   // per block: exclusive scan of rows
  const int64_t *tile_start;  // per block: exclusive scan of row tiles
  const int64_t *unit_off;    // per block: slice storage offset, 256-byte units
  int32_t *exps;              // exponent table
  uint8_t *slices;            // slice storage
  int64_t n_rows, n_tiles, n_exps;
  int32_t s, rt_rows;
  int32_t f16;                // binary16 data: copied as they are (one slice, no exponents)
  int32_t pack;               // 16-column k-steps per stored step (oz_pack_of)
  // class layout (items != NULL): n_tiles counts the items
  const OzClassItem *items;
  const OzRowMap *rmap;       // per virtual row
  const int32_t *blk;         // block of (free box, contracted box) per class
};

// One block pair of a job, in the order the GEMM walks them (pairs of each
// output block consecutive): byte offsets of the two blocks' slices and the
// pair's k-steps of 16.
struct __align__(8) OzPairRec {
  int64_t a_off, b_off;
  int32_t nk, pad;
};

struct OzJob {
  GemmJob g;
  const OzPairRec *prs;       // [n_pairs] by position in the pair order (seg)
  const int64_t *tile_start;  // [n_out+1] first 128x96 tile of output o
  int64_t n_tiles;
  const int64_t *ksum;        // per output: k-steps of 16 over its pairs
  const int32_t *nk_pair;     // per pair: k-steps of 16
  const uint8_t *sliceA, *sliceB;
  const int64_t *unitA, *unitB;
  const int64_t *keyA, *keyB;
  const int64_t *rowA, *rowB;
  const int32_t *expA, *expB;
  int32_t s;
  int32_t tile_n;             // output columns per tile (every job of a launch alike)
  int32_t f16;                // binary16 operands and result, fp32 accumulation (s = 1)
  int32_t pack;               // 16-column k-steps per pipeline stage (oz_pack_of)
  // class layout (cls != NULL): the GEMM's outputs are the classes, each with one
  // pseudo-pair (its whole contracted range); tile_start and ksum are per class
  const OzClassOut *cls;
  int64_t n_cls;
  const OzRowMap *rmapA, *rmapB;
  const int64_t *offs;        // per class and (A free box, B free box): output block offset
};

// One output tile of a launch, decoded once when the launch is built: the GEMM's
// three roles read it with one load instead of a chain of dependent lookups.
struct __align__(16) OzTileRec {
  int64_t seg0, seg1;   // pairs of the tile's output block (positions in the pair order)
  int64_t ksum;         // k-steps of 16 over those pairs
  int64_t c_off;        // offset of the output block in C
  int64_t m, n;         // rows and columns of the output block
  int64_t erow, ecol;   // first row / column of the block in the exponent tables
  int32_t job, mt, nt;  // job index, row tile, column tile
  int32_t packed;       // ga | gb << 8 | nmma << 16 (row groups of A and B, MMA width)
};

// Kernel parameter of a batched launch (arrays in device memory).
struct OzLaunch {
  const OzJob *jobs;
  const int64_t *job_tile_start;   // [n_jobs+1]
  int32_t n_jobs;
  int64_t n_tiles;
  const OzSide *sides;
  const int64_t *side_row_start;   // [n_sides+1]
  const int64_t *side_tile_start;  // [n_sides+1]
  const int64_t *side_exp_start;   // [n_sides+1]
  int32_t n_sides;
  int64_t n_rows, n_slice_tiles, n_exps;
  int32_t s_max, nstages, tile_n;
  int32_t s_all;           // the slice count of every job, or 0 when they differ
  int32_t f16;             // every job has binary16 operands (jobs of one launch agree)
  int32_t *err;
  const OzTileRec *tiles;  // [n_tiles]
  uint64_t wait_ns;        // limit of every pipeline wait (nanoseconds of wall time)
  uint64_t delay_ns;       // producer start delay (failure-path tests only; else 0)
};

// Device copies of the job and side lists plus their prefix sums.
struct OzBatchDev {
  DevArray<OzJob> jobs;
  DevArray<OzSide> sides;
  DevArray<int64_t> prefixes;  // job tiles | side rows | side tiles | side exps
  DevArray<int32_t> err;
  DevArray<OzTileRec> tiles;
  OzLaunch L{};
  int sms = 0;  // multiprocessors of the device: the persistent grid
};

int oz_stages(int s, int tile_n);
// The pair table of job J (J's pair arrays, unit offsets and k-steps made).
tq_status oz_pair_table(const OzJob &J, int64_t n_pairs, OzPairRec *out, cudaStream_t st);
tq_status oz_batch_build(const std::vector<OzJob> &jobs, const std::vector<OzSide> &sides,
                         cudaStream_t s, OzBatchDev &out);
// Row exponents and slices of every side of the batch.
tq_status oz_batch_prepare(const OzBatchDev &b, cudaStream_t s);
// The persistent tensor-core GEMM over every output tile of every job.
tq_status oz_batch_gemm(const OzBatchDev &b, cudaStream_t s);
// Reads (and clears) the bounded-wait error flag; synchronises the stream.
tq_status oz_batch_check(const OzBatchDev &b, cudaStream_t s);

}  // namespace tq
