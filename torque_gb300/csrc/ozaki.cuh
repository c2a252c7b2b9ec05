// Work description of the tensor-core (sliced) forms of the grouped GEMM.
#pragma once
#include "gemm.cuh"

namespace tq {

constexpr int OZ_M = 128;        // output rows per tile (A side, TMEM lanes)
constexpr int OZ_N = 96;         // output columns per tile (B side)
constexpr int OZ_CHUNK = 15;     // k-steps of 16 per exact flush (K = 240)
constexpr int OZ_MAXS = 7;       // most slices supported
constexpr int OZ_MAX_STAGES = 8;
constexpr int OZ_EXP_ZERO = -(1 << 20);  // exponent of an all-zero row

// One operand side (A or B) of the slicing passes: every block of the tensor
// is one operand unit viewed as a rows x k matrix (rows over the free legs,
// columns over the contracted legs in pair order, each block's full range).
struct OzSide {
  DevBS T;
  int32_t nfree, ncon;
  int32_t free_legs[TQ_MAXR], con[TQ_MAXR];
  const int64_t *key;         // free-box class key per block
  const int64_t *row_off;     // per key: first row in the exponent table
  const int64_t *row_start;   // per block: exclusive scan of rows
  const int64_t *tile_start;  // per block: exclusive scan of row tiles
  const int64_t *unit_off;    // per block: slice storage offset, 256-byte units
};

struct OzJob {
  GemmJob g;
  const int64_t *tile_start;  // [n_out+1] first 128x96 tile of output o
  int64_t n_tiles;
  const int64_t *ksum;        // per output: k-steps of 16 over its pairs
  const int32_t *nk_pair;     // per pair: k-steps of 16
  const uint8_t *sliceA, *sliceB;
  const int64_t *unitA, *unitB;
  const int64_t *keyA, *keyB;
  const int64_t *rowA, *rowB;
  const int32_t *expA, *expB;
  int32_t s, nstages;
  int32_t *err;
};

int oz_stages(int s);
// Row exponents and slices of both operands.
tq_status launch_ozaki_prepare(const OzJob &job, const OzSide &SA, const OzSide &SB,
                               int64_t rowsA, int64_t rowsB, int64_t tilesA, int64_t tilesB,
                               int32_t *expA, int32_t *expB, int64_t nexpA, int64_t nexpB,
                               cudaStream_t st);
// The persistent tensor-core GEMM over all output tiles.
tq_status launch_ozaki_gemm(const OzJob &job, cudaStream_t st);

}  // namespace tq
