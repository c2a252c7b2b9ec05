/*
 * torque_oracle.h -- CPU restatement of Torque's block-sparse contraction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA path is checked
 * against.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * --impl reference legs may load it.  The product library never links it.
 *
 * Every function restates the reference algorithm (Walter-Feng/Torque) and cites
 * the file:line it follows.  Conventions of the reference, kept here:
 *   - column-major everywhere: leg 0 is fastest (src/util/space.h:11-24);
 *   - a block-sparse tensor is a list of boxes with inclusive begin/end points per
 *     leg; metadata matrices are rank x n_blocks, column = block
 *     (src/tensor/block_sparse.h:114-145);
 *   - block data lives back to back; block_offsets = exclusive scan of the block
 *     element counts (src/util/space.h:77-88);
 *   - boxes may overlap; query sums every block containing the index
 *     (src/tensor/block_sparse.h:373-409).
 */
#ifndef TORQUE_ORACLE_H
#define TORQUE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A block-sparse tensor as plain arrays (host memory). */
typedef struct {
  int32_t rank;
  const int64_t *dimension;  /* [rank] */
  int64_t n_blocks;
  const int64_t *begin;      /* [n_blocks*rank], block b leg l at b*rank+l */
  const int64_t *end;        /* inclusive end points, same layout */
  const int64_t *strides;    /* per-block index tables, same layout */
  const int64_t *offsets;    /* [n_blocks] element offset of each block */
  const double *data;
} orc_bs;

/* Status codes (mirror the product library's). */
#define ORC_OK 0
#define ORC_ERR_INVALID 1
#define ORC_ERR_RANGE 4
/* mode 2 only: the as-written strides would read outside the tensor's values,
 * where the reference's result is undefined. */
#define ORC_ERR_READ 6

/*
 * Block-pair matching: for every A block (ascending) the B blocks (ascending)
 * whose contracted-leg intervals overlap on every contracted leg.
 * Restates torque::block_sparse::block_in_range (src/tensor/block_sparse.cpp:6-60)
 * driven by the A-block loop of contract (src/gpu/block_sparse.cuh:626-652).
 * If pa/pb are NULL only counts.  Returns the number of pairs, or -1 if cap is
 * exceeded.
 */
int64_t orc_match(const orc_bs *A, const orc_bs *B, int32_t nc,
                  const int64_t *a_legs, const int64_t *b_legs,
                  int64_t *pa, int64_t *pb, int64_t cap);

/*
 * Per-pair boxes for pair (i, j):
 *   out_begin/out_end [rankA-nc + rankB-nc]: A free legs then B free legs
 *     (src/tensor/block_sparse.cpp:66-79, :110-119);
 *   con_begin/con_end [nc]: intersection on contracted legs, pair order
 *     (block_sparse.cpp:42-60, :94-101);
 *   a_sub_begin/a_sub_end [rankA], b_sub_begin/b_sub_end [rankB]: the sub-boxes
 *     of the two blocks that take part (block_sparse.cpp:83-106, :130-148).
 * Any output pointer may be NULL.
 */
void orc_pair_boxes(const orc_bs *A, const orc_bs *B, int32_t nc,
                    const int64_t *a_legs, const int64_t *b_legs,
                    int64_t i, int64_t j,
                    int64_t *out_begin, int64_t *out_end,
                    int64_t *con_begin, int64_t *con_end,
                    int64_t *a_sub_begin, int64_t *a_sub_end,
                    int64_t *b_sub_begin, int64_t *b_sub_end);

/*
 * Values of the output block of one pair, in the reference's layout: an m x n
 * column-major matrix C = A_rep * B_rep^T where A_rep rows run over A's free legs
 * (column-major, ascending legs) and columns over the contracted legs in pair
 * order; likewise B_rep (src/tensor/block_sparse.h:17-80, :527-542).
 * mode 0: the reference's intended arithmetic (each block's own strides),
 *         Neumaier-compensated double sums (accurate oracle);
 * mode 1: plain double sums in the same order as a naive gemm loop (the CPU
 *         baseline arithmetic);
 * mode 2: the reference CPU path as written: the element strides come from
 *         column j_block of each tensor's index tables, not the pair's own
 *         blocks (src/tensor/block_sparse.h:531,538).  Returns ORC_ERR_RANGE
 *         when j_block is past a tensor's block count (Armadillo would throw)
 *         and ORC_ERR_READ when those strides would address an element past
 *         the end of a tensor's values (the reference reads there; its
 *         result is undefined, and the oracle reads nothing).
 * j_block is the position of B block j in A block i's match list.
 */
int32_t orc_pair_values(const orc_bs *A, const orc_bs *B, int32_t nc,
                        const int64_t *a_legs, const int64_t *b_legs,
                        int64_t i, int64_t j, int64_t j_block, int32_t mode,
                        double *out);

/*
 * Full reference-layout contraction (src/tensor/block_sparse.h:416-584):
 * pairs in reference order, output block b = pair b, offsets = exclusive scan.
 * out_data must hold orc_contract_size() elements.  For a rank-0 result
 * (every leg contracted) out_data[0] receives the sum over all pairs
 * (block_sparse.h:553-579).
 */
int64_t orc_contract_size(const orc_bs *A, const orc_bs *B, int32_t nc,
                          const int64_t *a_legs, const int64_t *b_legs);
int32_t orc_contract(const orc_bs *A, const orc_bs *B, int32_t nc,
                     const int64_t *a_legs, const int64_t *b_legs, int32_t mode,
                     int64_t *out_begin, int64_t *out_end, int64_t *out_offsets,
                     double *out_data);

/*
 * The CPU baseline: the reference CPU path's per-pair work for a list of pairs,
 * in parallel over pairs (OpenMP).  For each pair the two sub-blocks are first
 * gathered into contiguous matrices A_rep (m x k) and B_rep (n x k), as
 * sort_into_matrix does (src/tensor/block_sparse.h:17-80, :527-539), then
 * C = A_rep B_rep^T is formed in double (block_sparse.h:541-542).  out_offsets[q]
 * is where pair q's m x n column-major block goes.  Returns the thread count.
 */
int32_t orc_pairs_baseline(const orc_bs *A, const orc_bs *B, int32_t nc, const int64_t *a_legs,
                           const int64_t *b_legs, int64_t n, const int64_t *pa,
                           const int64_t *pb, const int64_t *out_offsets, double *out);

/* query: sum over every block containing idx (src/tensor/block_sparse.h:373-409). */
double orc_query(const orc_bs *T, const int64_t *idx);

/* Zero-fill then add every block (the densified tensor, column-major over
 * dimension).  Overlaps add, as query does. */
void orc_densify(const orc_bs *T, double *dense);

/* hard_transpose of every block (src/tensor/block_sparse.h:608-651): output
 * blocks keep their order; new strides are column-major of the permuted dims. */
void orc_hard_transpose(const orc_bs *T, const int64_t *perm, double *out_data);

/* Exclusive prefix sum (src/util/space.h:77-88). */
void orc_nest_sum(const int64_t *x, int64_t n, int64_t *out);

#ifdef __cplusplus
}
#endif
#endif
