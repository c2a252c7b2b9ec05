/*
 * torque_gb300.h -- C ABI of the GB300-native block-sparse contraction library.
 *
 * The drop-in boundary for Torque's block-sparse GPU path
 * (torque::gpu::BlockSparseTensor<T>, src/gpu/block_sparse.cuh).  The C++
 * header include/torque_gb300/block_sparse.hpp rebuilds the reference class on
 * top of these entry points; other languages bind them directly (ctypes, cgo,
 * JNI) through the plain pointers, sizes and status codes below.
 *
 * Conventions kept from the reference:
 *   - column-major: leg 0 is fastest (src/util/space.h:11-24);
 *   - metadata matrices are rank x n_blocks with one column per block, passed
 *     as flat arrays where block b, leg l is element [b*rank + l] (the memory
 *     layout of an arma::umat);
 *   - boxes are inclusive [begin, end] per leg; they may overlap, and query sums
 *     every block containing the index (block_sparse.cuh:506-552);
 *   - block data are back to back; block_offsets = exclusive scan of the block
 *     element counts (src/util/space.h:77-88).
 * Changes from the reference:
 *   - every call returns a tq_status instead of exit()ing the process
 *     (src/gpu/util/lib_helper.cuh:39-77); tq_last_error_string() explains it;
 *   - work is ordered on the caller's stream; only calls that must hand a
 *     number to the host (query, to_number, metadata reads, output sizing in
 *     contract) synchronise that stream;
 *   - no cuBLAS/cuTT handle: contract takes none.
 */
#ifndef TORQUE_GB300_H
#define TORQUE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *tq_stream; /* a cudaStream_t; NULL = legacy default */

typedef enum {
  TQ_OK = 0,
  TQ_ERR_INVALID = 1,     /* API misuse: the reference throws Error here */
  TQ_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  TQ_ERR_OOM = 3,         /* device allocation failed (or was refused by the hook) */
  TQ_ERR_RANGE = 4,       /* index outside the tensor */
  TQ_ERR_UNSUPPORTED = 5, /* valid input outside what the library implements */
  TQ_ERR_TIMEOUT = 6      /* a bounded device wait gave up */
} tq_status;

/* Element types: the reference instantiates float, double and half
 * (src/gpu/block_sparse.cu:66-148).  TQ_F16 is IEEE binary16; its native
 * contraction accumulates every output element in FP32 and rounds it to
 * binary16 once (the reference's cublasHgemm path, block_sparse.cuh:894-930,
 * accumulates in half).  The tensor-core forms take TQ_F64 only. */
typedef enum { TQ_F32 = 0, TQ_F64 = 1, TQ_F16 = 2 } tq_dtype;

typedef enum { TQ_MEM_HOST = 0, TQ_MEM_DEVICE = 1 } tq_memkind;

/* Arithmetic of the block GEMMs. */
typedef enum {
  TQ_PREC_NATIVE = 0, /* plain arithmetic in the tensor's type (the drop-in) */
  TQ_PREC_OZAKI = 1,  /* FP64-level: exact integer slices on the bf16 tensor cores */
  TQ_PREC_BF16X3 = 2, /* FP32-level: three-way bf16 split products */
  TQ_PREC_TENSOR = 3  /* half tensors only: fp16 x fp16 products on the tensor cores
                         (tcgen05 kind::f16), fp32 accumulation, fp32 sums of the
                         accumulators, one rounding of each result element */
} tq_precision;

/* Block list of a contraction result. */
typedef enum {
  TQ_LAYOUT_REFERENCE = 0, /* one output block per matched block pair, in the
                              reference's order (block_sparse.cuh:626-674) */
  TQ_LAYOUT_REDUCED = 1    /* one block per distinct output box, partials of the
                              pairs that land in it summed in FP64 */
} tq_layout;

typedef struct {
  int32_t precision; /* tq_precision */
  int32_t layout;    /* tq_layout */
  int32_t slices;    /* Ozaki slice count (0 = default); ignored otherwise */
  int32_t tile_n;    /* tensor-core forms: output columns per tile, 32, 64 or 96
                        (0 = 96); ignored otherwise */
  int32_t native_fill; /* tensor-core forms, block grouping: output blocks whose
                          tensor-core tiles are filled to less than
                          native_fill / 1000 run in plain FP64 instead (0 = none) */
  int32_t reserved;
} tq_contract_opts;

typedef struct tq_bs tq_bs; /* opaque block-sparse tensor */

/* ---- construction ---------------------------------------------------- */

/* BlockSparseTensor(const arma::uvec & dimension)
 * (src/gpu/block_sparse.cuh:180-187): no blocks; a rank-0 tensor holds one
 * zero. */
tq_status tq_bs_create_empty(tq_dtype dtype, int32_t rank, const int64_t *dimension,
                             tq_bs **out);

/* BlockSparseTensor(const T*, const umat& begin, const umat& end,
 *                   const uvec& dim, cudaMemcpyKind) (block_sparse.cuh:189-236),
 * and with explicit index tables (block_sparse.cuh:238-281).  index_tables may
 * be NULL (column-major strides of each block, the reference's default). */
tq_status tq_bs_create(tq_dtype dtype, int32_t rank, const int64_t *dimension,
                       int64_t n_blocks, const int64_t *begin_points,
                       const int64_t *end_points, const int64_t *index_tables,
                       const void *data, tq_memkind kind, tq_stream stream,
                       tq_bs **out);

/* Adopts a device buffer the caller allocated with cudaMalloc: the reference's
 * raw move-in constructor BlockSparseTensor(T* data, rank, dimension,
 * blocks_dimension, begin_points, end_points, block_n_elem, block_offsets,
 * index_tables) (block_sparse.cuh:283-304).  The tensor owns device_data from
 * then on and frees it with cudaFree (as the reference's destructor does,
 * :361-364); no copy is made.  block_offsets may be NULL; if given it must be
 * the exclusive scan of the block sizes (TQ_ERR_UNSUPPORTED otherwise).  On
 * any error the buffer stays the caller's. */
tq_status tq_bs_adopt(tq_dtype dtype, int32_t rank, const int64_t *dimension, int64_t n_blocks,
                      const int64_t *begin_points, const int64_t *end_points,
                      const int64_t *index_tables, const int64_t *block_offsets,
                      void *device_data, tq_bs **out);

/* The same block list with every element zero (the reference's
 * DenseTensor(dimension) and SparseTensor(dimension) constructors,
 * src/gpu/dense.cuh:68-84, src/gpu/sparse.cuh:95-103, start from zeros). */
tq_status tq_bs_create_zeros(tq_dtype dtype, int32_t rank, const int64_t *dimension,
                             int64_t n_blocks, const int64_t *begin_points,
                             const int64_t *end_points, const int64_t *index_tables,
                             tq_stream stream, tq_bs **out);

/* Overwrite all block data (n_elem elements; one for a rank-0 tensor) from
 * host or device memory: DenseTensor::initialize (src/gpu/dense.cuh:172-184). */
tq_status tq_bs_set_data(tq_bs *t, const void *data, tq_memkind kind, tq_stream stream);
/* The same copy, only enqueued on `stream` (no synchronisation): the caller
 * keeps `data` alive and unchanged until the stream has passed the copy.  From
 * page-locked host memory the copy runs on a copy engine while other streams
 * compute (a serving loop copies step i+1's inputs during step i's GEMM).  No
 * reference counterpart. */
tq_status tq_bs_set_data_async(tq_bs *t, const void *data, tq_memkind kind, tq_stream stream);

/* Copy constructor (block_sparse.cuh:306-327): deep device copy. */
tq_status tq_bs_clone(const tq_bs *t, tq_stream stream, tq_bs **out);

/* Destructor (block_sparse.cuh:361-364). */
tq_status tq_bs_destroy(tq_bs *t);

/* append_block / append_blocks (block_sparse.cuh:376-446).  The buffer grows
 * geometrically instead of being reallocated per call. */
tq_status tq_bs_append_blocks(tq_bs *t, int64_t n_blocks, const int64_t *begin_points,
                              const int64_t *end_points, const int64_t *index_tables,
                              const void *data, tq_memkind kind, tq_stream stream);

/* ---- element access ---------------------------------------------------- */

/* query (block_sparse.cuh:506-552): sum over every block holding the index. */
tq_status tq_bs_query(const tq_bs *t, const int64_t *indices, void *value);

/* modify (block_sparse.cuh:451-502): set in the first block holding the index,
 * zero it in the others, or append a one-element block if none holds it and
 * the value is nonzero. */
tq_status tq_bs_modify(tq_bs *t, const int64_t *indices, const void *value);

/* to_number (block_sparse.cuh:367-374): the value of a rank-0 tensor. */
tq_status tq_bs_to_number(const tq_bs *t, void *value);

/* ---- metadata ---------------------------------------------------------- */

tq_status tq_bs_shape(const tq_bs *t, tq_dtype *dtype, int32_t *rank, int64_t *n_blocks,
                      int64_t *n_elem);
/* The public members dimension, begin_points, end_points, index_tables,
 * block_offsets (block_sparse.cuh:147-178).  Any pointer may be NULL. */
tq_status tq_bs_metadata(const tq_bs *t, int64_t *dimension, int64_t *begin_points,
                         int64_t *end_points, int64_t *index_tables,
                         int64_t *block_offsets);
/* The device buffer (the reference's protected T* data). */
tq_status tq_bs_device_data(const tq_bs *t, void **ptr);
/* Copy all block data to dst (host or device), ordered on stream. */
tq_status tq_bs_copy_data(const tq_bs *t, void *dst, tq_memkind kind, tq_stream stream);

/* ---- operations -------------------------------------------------------- */

/* contract (block_sparse.cuh:558-1026): contract legs a_legs[k] of A with
 * b_legs[k] of B (the two columns of the reference's n x 2 contracting_indices).
 * The result's legs are A's free legs then B's free legs, each in order.
 * opts may be NULL (native precision, reference layout). */
tq_status tq_bs_contract(const tq_bs *A, const tq_bs *B, int32_t n_legs,
                         const int64_t *a_legs, const int64_t *b_legs,
                         const tq_contract_opts *opts, tq_stream stream, tq_bs **out);

/* The block list contract would produce, from its symbolic stage alone: the
 * pair matching of block_in_range (src/tensor/block_sparse.cpp:6-175) and the
 * group assembly of contract (block_sparse.cuh:620-674), with no block
 * GEMM run and no result data allocated, so the structure of a result too large
 * to hold can still be read.  layout is a tq_layout.  *n_blocks and *n_elem
 * receive the result's block and element counts; when cap >= *n_blocks the
 * non-NULL host arrays are filled: begin_points and end_points (rank x
 * n_blocks, as tq_bs_metadata), block_offsets (n_blocks) and, in the reference
 * layout only, pair_a / pair_b (n_blocks: the A and B block of each output
 * block).  Call once with cap = 0 to size the arrays. */
tq_status tq_contract_blocks(const tq_bs *A, const tq_bs *B, int32_t n_legs,
                             const int64_t *a_legs, const int64_t *b_legs, int32_t layout,
                             int64_t cap, int64_t *n_blocks, int64_t *n_elem,
                             int64_t *begin_points, int64_t *end_points,
                             int64_t *block_offsets, int64_t *pair_a, int64_t *pair_b,
                             tq_stream stream);

/* The element-sparse contract of the reference's SparseTensor
 * (src/gpu/sparse.cuh:270-375) for tensors whose blocks each hold one element:
 * C[free A legs, free B legs] = sum over matching contracted indices of A B.
 * Matches are found by sorting both operands by their contracted index and
 * joining equal runs (O(nnz log nnz + products)), where the reference forms
 * all nnz_A x nnz_B products.  The result has one one-element block per
 * distinct output element, in column-major order of its coordinates (A's free
 * legs, then B's), every product summed; unlike the reference, the first
 * output element is kept (sparse.cuh:370-371 drops it).  Products are formed
 * in FP64 and each sum is rounded to the element type once.  At least one leg
 * must stay free (a full contraction to a scalar is tq_bs_contract's). */
tq_status tq_bs_contract_elements(const tq_bs *A, const tq_bs *B, int32_t n_legs,
                                  const int64_t *a_legs, const int64_t *b_legs,
                                  tq_stream stream, tq_bs **out);

/* hard_transpose (block_sparse.cuh:1031-1122): permute the legs of every block;
 * new leg l is old leg perm[l]. */
tq_status tq_bs_hard_transpose(const tq_bs *t, const int64_t *perm, tq_stream stream,
                               tq_bs **out);

/* Leg fusion (no reference counterpart; a PEPS double layer needs it): legs
 * `leg` and `leg`+1 become one leg of dimension dim_a * dim_b.  Leg a is cut
 * into n_sec_a sectors at bounds_a[0..n_sec_a] (bounds_a[0] = 0, last = dim),
 * leg b likewise; sector pair (a, b) occupies the fused range starting at
 * pair_offset[a + n_sec_a * b], of length size_a * size_b (the ranges must
 * tile the fused leg).  Every block must cover whole sectors on both legs with
 * contiguous strides across them; its data are then already in the fused
 * layout and are copied unchanged. */
tq_status tq_bs_fuse_legs(const tq_bs *t, int32_t leg, int64_t n_sec_a, const int64_t *bounds_a,
                          int64_t n_sec_b, const int64_t *bounds_b, const int64_t *pair_offset,
                          tq_stream stream, tq_bs **out);

/* Inverse of tq_bs_fuse_legs (no reference counterpart; a sweep needs it to go
 * back from D^2 to D x D without leaving the device): leg `leg` becomes legs
 * `leg` (dim bounds_a[n_sec_a]) and `leg`+1 (dim bounds_b[n_sec_b]), with the
 * same sector bounds and pair offsets that fused them.  Every block must cover
 * exactly one sector pair's range of the leg; its data are already in the split
 * layout and are copied unchanged. */
tq_status tq_bs_split_leg(const tq_bs *t, int32_t leg, int64_t n_sec_a, const int64_t *bounds_a,
                          int64_t n_sec_b, const int64_t *bounds_b, const int64_t *pair_offset,
                          tq_stream stream, tq_bs **out);

/* Block lists of charge-conserving (U(1) or Z_n) tensors (no reference
 * counterpart: Torque leaves the mapping of symmetry sectors to boxes to its
 * caller, src/tensor/block_sparse.h:109-145).  Leg l has n_sectors[l] sectors
 * whose charges and sizes are concatenated over the legs (leg 0 first), laid out
 * as contiguous coordinate ranges in the given order, and a direction
 * directions[l] = +1 (incoming) or -1 (outgoing).  A block exists for every
 * sector tuple with sum(direction * charge) == total (mod modulus for Z_n;
 * modulus 0 = U(1)); blocks are listed in column-major order of the sector
 * indices (leg 0 fastest).  *n_blocks receives the count; when cap >= it,
 * begin_points / end_points (rank x n_blocks, as tq_bs_create takes them) are
 * filled.  Call once with cap = 0 to size them. */
tq_status tq_charge_blocks(int32_t rank, const int64_t *n_sectors, const int64_t *charges,
                           const int64_t *sizes, const int32_t *directions, int64_t total,
                           int64_t modulus, int64_t cap, int64_t *n_blocks,
                           int64_t *begin_points, int64_t *end_points);
/* A tensor over that block list, its data in block order (each block
 * column-major) from host or device memory, or all zeros when data is NULL. */
tq_status tq_bs_create_charges(tq_dtype dtype, int32_t rank, const int64_t *n_sectors,
                               const int64_t *charges, const int64_t *sizes,
                               const int32_t *directions, int64_t total, int64_t modulus,
                               const void *data, tq_memkind kind, tq_stream stream,
                               tq_bs **out);

/* Block-level truncated SVD for PEPS / MPS sweeps (no reference counterpart:
 * the reference has only a cuSOLVER QR example that nothing calls,
 * test/cusolver_playground.cpp:7).  Legs row_legs (in that order) against the
 * others (ascending): the tensor is block diagonal over classes of row and
 * column boxes linked by blocks (one per charge sector for a symmetric
 * tensor); each class matrix is decomposed in FP64 by one-sided Jacobi
 * rotations on the device; the singular values of all classes are ranked
 * together and at most max_keep of them (all when max_keep <= 0) above
 * cutoff * the largest are kept (zeros never).  Returns U[row legs..., bond],
 * S[bond] and V[bond, column legs...] over a new bond leg with one sector per
 * class that keeps values (values descending within a sector), so that T is
 * approximated by sum_k U[..., k] S[k] V[k, ...].  float64 tensors whose
 * blocks are sector boxes (intervals of a leg equal or disjoint). */
tq_status tq_bs_svd(const tq_bs *t, int32_t n_row_legs, const int64_t *row_legs,
                    int64_t max_keep, double cutoff, tq_stream stream, tq_bs **U, tq_bs **S,
                    tq_bs **V);
/* Block-level QR (an extension, same class structure as tq_bs_svd): each
 * class matrix A (M x N) is factored by Householder reflections in FP64 on the
 * device as A = Q R with Q (M x k, orthonormal columns), R (k x N, upper
 * trapezoidal, non-negative diagonal), k = min(M, N).  Returns Q[row legs...,
 * bond] and R[bond, column legs...] over a new bond leg with one sector of k
 * per class (classes in the order of their first row box), so that T =
 * sum_k Q[..., k] R[k, ...].  float64 tensors of sector boxes. */
tq_status tq_bs_qr(const tq_bs *t, int32_t n_row_legs, const int64_t *row_legs, tq_stream stream,
                   tq_bs **Q, tq_bs **R);

/* slice (block_sparse.cuh:1124-1176): split every block into prod(divisor)
 * boxes without moving data, as the reference does. */
tq_status tq_bs_slice(const tq_bs *t, const int64_t *divisor, tq_stream stream,
                      tq_bs **out);

/* torque::util::nest_sum (src/util/space.h:77-88) on the device: offsets[i] =
 * counts[0] + ... + counts[i-1], *total = the sum of all n counts.  The block
 * offsets of a block list are the nest_sum of its block element counts.  All
 * three pointers are device memory; ordered on stream. */
tq_status tq_nest_sum(const int64_t *counts, int64_t n, int64_t *offsets, int64_t *total,
                      tq_stream stream);

/* tq_nest_sum for callers that cannot allocate device memory (no counterpart in
 * the reference).  It calls no cudaMalloc/cudaFree and no allocating library
 * routine: its scratch is a 32 KB array of static device memory that the library
 * keeps on every GPU that loads it.  At most 4,194,304 counts (larger n returns
 * TQ_ERR_INVALID).  The first call on a device looks up that array's device
 * address, so make that first call before any stream capture.  All calls share
 * the array: calls that overlap on the GPU race; sequential calls are
 * independent. */
tq_status tq_nest_sum_noalloc(const int64_t *counts, int64_t n, int64_t *offsets,
                              int64_t *total, tq_stream stream);

/* ---- plans: the symbolic and numeric stages of contract, separately ------- */

typedef struct tq_plan tq_plan;

/* Runs the index kernels (pair matching, output boxes and offsets), allocates
 * the result and returns it with its metadata filled and its data not yet
 * computed.  Synchronises the stream once to size the result. */
tq_status tq_plan_create(const tq_bs *A, const tq_bs *B, int32_t n_legs,
                         const int64_t *a_legs, const int64_t *b_legs,
                         const tq_contract_opts *opts, tq_stream stream,
                         tq_plan **plan, tq_bs **out);
/* Numeric stage: computes the result's data.  No host synchronisation, no
 * allocation: safe to capture in a CUDA graph.  A and B must be alive. */
tq_status tq_plan_execute(tq_plan *plan, tq_stream stream);
/* The numeric stage of tq_plan_execute with the result written to dst
 * instead of the result tensor's own buffer (which is then not written).
 * dst holds the result's n_elem elements in the result's layout and is
 * device memory (TQ_MEM_DEVICE) or host memory (TQ_MEM_HOST).  Page-locked
 * host memory (cudaHostAlloc, cudaHostRegister) is written by the kernels
 * themselves over the host link while they run, so no device-to-host copy
 * follows the GEMM; pageable host memory gets the computed result by one
 * copy.  TQ_MEM_HOST synchronises the stream before returning.  The
 * reference has no counterpart: its results are copied out of device memory
 * (src/gpu/block_sparse.cuh:558-1026 leaves the result on the device). */
tq_status tq_plan_execute_to(tq_plan *plan, void *dst, tq_memkind kind, tq_stream stream);
/* Useful flops of the plan: sum over matched block pairs of 2*m*n*k. */
tq_status tq_plan_flops(const tq_plan *plan, double *flops, int64_t *n_pairs);
/* Record CUDA events on the launching stream around the phases of each
 * tq_plan_execute (operand preparation, block GEMM). */
tq_status tq_plan_set_profiling(tq_plan *plan, int32_t enable);
/* Durations of the last profiled execute; synchronises on its last event. */
tq_status tq_plan_last_timings(tq_plan *plan, float *prepare_ms, float *gemm_ms);
/* Status of the tensor-core kernel's bounded waits in the last execute
 * (synchronises the stream): TQ_OK or TQ_ERR_TIMEOUT. */
tq_status tq_plan_check(tq_plan *plan, tq_stream stream);
tq_status tq_plan_destroy(tq_plan *plan);
/* A new schedule (precision, slices, tile_n, native_fill; the layout stays)
 * for a planned contraction, keeping its symbolic stage.  A plan created for
 * plain arithmetic in the reference layout cannot take a tensor-core schedule
 * (TQ_ERR_INVALID).  Synchronises the stream.  No reference counterpart. */
tq_status tq_plan_reschedule(tq_plan *plan, const tq_contract_opts *opts, tq_stream stream);

/* ---- schedule autotuning and the learned cost model ------------------- */
/* No reference counterpart: the reference runs one fixed cuBLAS path
 * (block_sparse.cuh:870-930). */

#define TQ_N_FEATURES 32

typedef struct {
  tq_contract_opts opts; /* the candidate schedule (layout: the plan's) */
  int32_t status;        /* TQ_OK, or why the candidate could not run */
  float ms;              /* numeric stage, fastest of the timed runs (CUDA events) */
  double rel_err;        /* max|C - C_fp64| / max|C_fp64| over the result */
} tq_tune_entry;

/* Exhaustive autotuner: runs every candidate schedule on the plan (one
 * warm-up, then `reps` timed runs), measures its error against the plain FP64
 * result of the same plan, and sets *best to the fastest candidate whose error
 * is at most target_rel_err (-1: none).  The plan is left with the winner's
 * schedule (its own if none).  A negative target times the candidates only
 * (no FP64 reference run; rel_err = -1; the fastest wins): for tuning the tile
 * width and grouping of a slice count already known to meet the target.
 * Synchronises; float64 tensors only. */
tq_status tq_autotune(tq_plan *plan, double target_rel_err, tq_tune_entry *cands,
                      int32_t n_cands, int32_t reps, int32_t *best, tq_stream stream);

/* The cost model's input: TQ_N_FEATURES floats describing the planned
 * contraction and the target accuracy (-log10(target)/16, ranks, contracted
 * legs and dimension, log flops, pairs and output blocks, and flop-weighted
 * histograms of the block GEMM sizes m, n, k).  Synchronises. */
tq_status tq_plan_features(const tq_plan *plan, double target_rel_err, float *features,
                           tq_stream stream);

/* A 3-layer FP32 perceptron (n_in -> width -> width -> n_out, ReLU), trained
 * and evaluated on the device by the library's own kernels.  Inputs, outputs
 * and targets are device arrays, row-major, one row per sample. */
typedef struct tq_mlp tq_mlp;
tq_status tq_mlp_create(int32_t n_in, int32_t width, int32_t n_out, uint64_t seed, tq_mlp **out);
tq_status tq_mlp_destroy(tq_mlp *mlp);
tq_status tq_mlp_num_params(const tq_mlp *mlp, int64_t *n_params);
/* Parameters as W1[width][n_in] b1 W2[width][width] b2 W3[n_out][width] b3. */
tq_status tq_mlp_get_params(tq_mlp *mlp, float *host);
tq_status tq_mlp_set_params(tq_mlp *mlp, const float *host);
/* Y (n x n_out, device) = network(X (n x n_in, device)). */
tq_status tq_mlp_forward(tq_mlp *mlp, const float *X, int64_t n, float *Y, tq_stream stream);
/* Loss (mean over samples and outputs of mask * (Y - T)^2, mask NULL = all
 * ones) and its gradient with respect to every parameter, copied to the host
 * (either pointer may be NULL).  Synchronises. */
tq_status tq_mlp_gradients(tq_mlp *mlp, const float *X, const float *T, const float *mask,
                           int64_t n, float *grads_host, float *loss_host, tq_stream stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on the masked mean squared error
 * of a batch; the batch loss goes to loss_dev (device, may be NULL).  No host
 * synchronisation; the activation buffers grow on the first call with a larger
 * batch. */
tq_status tq_mlp_train_step(tq_mlp *mlp, const float *X, const float *T, const float *mask,
                            int64_t n, float lr, float *loss_dev, tq_stream stream);

/* ---- batches: many contractions in one launch -------------------------- */

typedef struct tq_batch tq_batch;

/* Groups planned contractions into one numeric stage.  Plans in the same wave
 * are independent: the operand preparation of all their tensor-core plans runs
 * as one set of kernels and their block GEMMs as ONE persistent launch over the
 * output tiles of every plan.  wave[i] (non-decreasing; NULL = all in wave 0)
 * orders dependent contractions: a wave may read results of earlier waves
 * (e.g. the two contractions of a PEPS site update).  Native-precision and
 * rank-0 plans run after the tensor-core launch of their wave.  The plans must
 * outlive the batch.  Rescheduling a plan (tq_plan_reschedule, tq_autotune)
 * frees the arrays the batch's device tables point into: every batch built
 * from it before then refuses to run (TQ_ERR_INVALID) and must be built again. */
tq_status tq_batch_create(tq_plan *const *plans, int32_t n, const int32_t *wave,
                          tq_stream stream, tq_batch **out);
/* The numeric stage of every plan, ordered on stream; no host synchronisation,
 * no allocation (capturable). */
tq_status tq_batch_execute(tq_batch *batch, tq_stream stream);
/* The same as one CUDA graph: captured on the first call, replayed after. */
tq_status tq_batch_graph_launch(tq_batch *batch, tq_stream stream);
/* Bounded-wait status of the last execution (synchronises the stream). */
tq_status tq_batch_check(tq_batch *batch, tq_stream stream);
/* Kernels one execution of the batch launches. */
tq_status tq_batch_kernels(const tq_batch *batch, int64_t *kernels);
tq_status tq_batch_destroy(tq_batch *batch);

/* ---- errors and hooks -------------------------------------------------- */

/* Device memory comes from the library's own stream-ordered pool per device,
 * which keeps freed memory for reuse; this returns every unused byte of those
 * pools to the driver (synchronises the devices that have one). */
tq_status tq_release_cached_memory(void);

/* Message of the last failing call on this thread. */
const char *tq_last_error_string(void);

/* Test hook: the next `after` device allocations succeed, then every one is
 * refused with TQ_ERR_OOM until reset with after < 0. */
void tq_debug_fail_alloc_after(int64_t after);

/* Kernels the library has launched in this process so far. */
int64_t tq_debug_kernel_launches(void);
/* Failure-path test hook of the tensor-core forms: the launches built from now
 * on (plan creation, reschedule, batch creation) give up every pipeline wait
 * after wait_ns nanoseconds of wall time (0 = the default, 2 s) and hold their
 * producer back for producer_delay_ns before it issues anything (0 = none).
 * With a delay well above the limit, the waiting roles give up, the kernel
 * drains and frees its tensor memory, and the next check returns
 * TQ_ERR_TIMEOUT; nothing is left in flight.  Reset with (0, 0). */
void tq_debug_set_waits(uint64_t wait_ns, uint64_t producer_delay_ns);

#ifdef __cplusplus
}
#endif
#endif
