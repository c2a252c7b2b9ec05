// Integer index kernels of the contraction: block-pair matching, per-pair
// boxes, output offsets (device prefix scans) and the grouping of pairs by
// output box.  All bit-exact against the reference's host code
// (src/tensor/block_sparse.cpp:6-175, src/gpu/block_sparse.cuh:620-674).
#pragma once
#include "tq_internal.h"

namespace tq {

// Exclusive prefix sum of n int64 values; *total_dev (device) receives the sum.
tq_status scan_exclusive(const int64_t *in, int64_t *out, int64_t n, int64_t *total_dev,
                         cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs by key, keys < 2^key_bits.
// keys/vals are sorted in place (tmp buffers allocated inside).
tq_status radix_sort_pairs(int64_t *keys, int64_t *vals, int64_t n, int key_bits,
                           cudaStream_t s);

// Pair matching.  counts[i] = number of B blocks overlapping A block i on every
// contracted leg; emit writes the pairs in reference order (A ascending, then B
// ascending) given the exclusive scan of counts.
tq_status match_pairs(const DevBS &A, const DevBS &B, const LegSpec &legs, int64_t *counts,
                      cudaStream_t s);
tq_status emit_pairs(const DevBS &A, const DevBS &B, const LegSpec &legs,
                     const int64_t *row_off, int32_t *pa, int32_t *pb, cudaStream_t s);

}  // namespace tq
