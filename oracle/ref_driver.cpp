// C entry points over the reference's own CPU block-sparse tensor
// (torque::BlockSparseTensor<double>, src/tensor/block_sparse.h:110-656 of
// Walter-Feng/Torque, with block_in_range from src/tensor/block_sparse.cpp),
// compiled from the reference's sources against the Armadillo API subset in
// arma_api/.  TEST INFRASTRUCTURE ONLY: it lets the tests and fixture scripts
// run the reference's code on the same inputs as the oracle and the CUDA
// path.  Nothing in the library links it.
//
// build_ref.py compiles this file twice: once against the reference header as
// it is, and once with the header's two stride lookups of the CPU contract
// corrected (block_sparse.h:531,538).  In the second build the corrected
// header text arrives first in the same translation unit, so the include
// below is skipped.
//
// Metadata crosses the boundary in the reference's own layout: begin and end
// points are rank x n_blocks column-major (column = block), as arma::umat
// stores them.  Every call returns 0 on success, 1 when the reference threw
// its Error type, 2 for any other exception (Armadillo-style bounds errors);
// ref_last_error() gives the message.
#ifndef TORQUE_TENSOR_BLOCK_SPARSE_H
#include "tensor/block_sparse.h"
#endif

#include <cstdint>
#include <cstdlib>
#include <exception>
#include <string>

namespace {

typedef torque::BlockSparseTensor<double> Tensor;

// The tensor keeps its values in a protected member; a derived type names it.
struct DataAccess : Tensor {
  static double *get(const Tensor &t) { return (t.*(&DataAccess::data)).get(); }
  static double *release(Tensor &t) { return (t.*(&DataAccess::data)).release(); }
};

thread_local std::string last_error;

arma::umat to_umat(const uint64_t *p, arma::uword rows, arma::uword cols) {
  arma::umat m(rows, cols);
  for (arma::uword i = 0; i < rows * cols; i++) m[i] = p[i];
  return m;
}

arma::uvec to_uvec(const uint64_t *p, arma::uword n) {
  arma::uvec v(n);
  for (arma::uword i = 0; i < n; i++) v[i] = p[i];
  return v;
}

template <class F> int32_t guarded(F f) {
  try {
    f();
    return 0;
  } catch (const Error &e) {
    last_error = e.what();
    return 1;
  } catch (const std::exception &e) {
    last_error = e.what();
    return 2;
  }
}

}  // namespace

extern "C" {

typedef struct ref_tensor ref_tensor;

const char *ref_last_error(void) { return last_error.c_str(); }

// BlockSparseTensor(const T*, begin_points, end_points, total_dimension)
// (block_sparse.h:155-202).  The tensor copies the values.
int32_t ref_tensor_new(int32_t rank, const uint64_t *dimension, int64_t n_blocks,
                       const uint64_t *begin, const uint64_t *end, const double *data,
                       ref_tensor **out) {
  return guarded([&] {
    Tensor *t = new Tensor(data, to_umat(begin, rank, n_blocks), to_umat(end, rank, n_blocks),
                           to_uvec(dimension, rank));
    *out = reinterpret_cast<ref_tensor *>(t);
  });
}

// BlockSparseTensor(dimension) (block_sparse.h:147-153): no blocks, one
// zeroed element (a rank-0 tensor's value).
int32_t ref_tensor_new_empty(int32_t rank, const uint64_t *dimension, ref_tensor **out) {
  return guarded([&] {
    Tensor *t = new Tensor(to_uvec(dimension, rank));
    *out = reinterpret_cast<ref_tensor *>(t);
  });
}

// The reference's destructor releases the buffer without freeing it
// (block_sparse.h:259-262); the buffer is freed here.
void ref_tensor_free(ref_tensor *h) {
  if (!h) return;
  Tensor *t = reinterpret_cast<Tensor *>(h);
  std::free(DataAccess::release(*t));
  delete t;
}

// contract(tensor, contracting_indices) (block_sparse.h:414-584);
// legs is the n x 2 contracting-index matrix, column-major (column 0 = this
// tensor's legs).
int32_t ref_contract(const ref_tensor *a, const ref_tensor *b, int32_t n, const uint64_t *legs,
                     ref_tensor **out) {
  return guarded([&] {
    const Tensor &A = *reinterpret_cast<const Tensor *>(a);
    const Tensor &B = *reinterpret_cast<const Tensor *>(b);
    Tensor *c = new Tensor(A.contract(B, to_umat(legs, n, 2)));
    *out = reinterpret_cast<ref_tensor *>(c);
  });
}

// hard_transpose(permutation) (block_sparse.h:607-651)
int32_t ref_hard_transpose(const ref_tensor *a, const uint64_t *perm, ref_tensor **out) {
  return guarded([&] {
    const Tensor &A = *reinterpret_cast<const Tensor *>(a);
    Tensor *c = new Tensor(A.hard_transpose(to_uvec(perm, A.rank)));
    *out = reinterpret_cast<ref_tensor *>(c);
  });
}

// query(indices) (block_sparse.h:372-411)
int32_t ref_query(const ref_tensor *a, int32_t n, const uint64_t *indices, double *value) {
  return guarded([&] {
    const Tensor &A = *reinterpret_cast<const Tensor *>(a);
    *value = A.query(to_uvec(indices, n));
  });
}

// modify(indices, number) (block_sparse.h:322-369)
int32_t ref_modify(ref_tensor *a, int32_t n, const uint64_t *indices, double number) {
  return guarded([&] {
    Tensor &A = *reinterpret_cast<Tensor *>(a);
    A.modify(to_uvec(indices, n), number);
  });
}

// append_block(data, begin_point, end_point, index_table) (block_sparse.h:285-317)
int32_t ref_append_block(ref_tensor *a, int32_t rank, const double *data, const uint64_t *begin,
                         const uint64_t *end, const uint64_t *index_table) {
  return guarded([&] {
    Tensor &A = *reinterpret_cast<Tensor *>(a);
    A.append_block(data, to_uvec(begin, rank), to_uvec(end, rank), to_uvec(index_table, rank));
  });
}

// rank, block count and element count of a tensor
void ref_tensor_info(const ref_tensor *a, int32_t *rank, int64_t *n_blocks, int64_t *n_elem) {
  const Tensor &A = *reinterpret_cast<const Tensor *>(a);
  *rank = int32_t(A.rank);
  *n_blocks = int64_t(A.begin_points.n_cols);
  *n_elem = A.rank ? int64_t(arma::sum(A.block_n_elem)) : 1;
}

// The public metadata members and the values, as the tensor holds them:
// begin/end/index tables rank x n_blocks column-major, offsets per block.
// A null destination is skipped.
void ref_tensor_read(const ref_tensor *a, uint64_t *dimension, uint64_t *begin, uint64_t *end,
                     uint64_t *index_tables, uint64_t *offsets, double *data) {
  const Tensor &A = *reinterpret_cast<const Tensor *>(a);
  if (dimension)
    for (arma::uword i = 0; i < A.dimension.n_elem; i++) dimension[i] = A.dimension[i];
  if (begin)
    for (arma::uword i = 0; i < A.begin_points.n_elem; i++) begin[i] = A.begin_points[i];
  if (end)
    for (arma::uword i = 0; i < A.end_points.n_elem; i++) end[i] = A.end_points[i];
  if (index_tables)
    for (arma::uword i = 0; i < A.index_tables.n_elem; i++) index_tables[i] = A.index_tables[i];
  if (offsets)
    for (arma::uword i = 0; i < A.block_offsets.n_elem; i++) offsets[i] = A.block_offsets[i];
  if (data) {
    const arma::uword n = A.rank ? arma::sum(A.block_n_elem) : 1;
    const double *p = DataAccess::get(A);
    for (arma::uword i = 0; i < n; i++) data[i] = p[i];
  }
}

// block_in_range(contracting_indices, A begin, A end, B begins, B ends)
// (block_sparse.cpp:6-175): the B blocks whose contracted intervals meet the
// A block.  Writes up to cap indices; returns how many there are (or -1 with
// ref_last_error set).
int64_t ref_block_in_range(int32_t n, const uint64_t *legs, int32_t rank_a,
                           const uint64_t *a_begin, const uint64_t *a_end, int32_t rank_b,
                           int64_t n_b, const uint64_t *b_begin, const uint64_t *b_end,
                           uint64_t *found, int64_t cap) {
  int64_t count = -1;
  const int32_t st = guarded([&] {
    const auto info = torque::block_sparse::block_in_range(
        to_umat(legs, n, 2), to_uvec(a_begin, rank_a), to_uvec(a_end, rank_a),
        to_umat(b_begin, rank_b, n_b), to_umat(b_end, rank_b, n_b));
    count = int64_t(info.block_indices.n_elem);
    for (int64_t i = 0; i < count && i < cap; i++) found[i] = info.block_indices[i];
  });
  return st ? -1 : count;
}

// Register a Fortran-convention dgemm for the matrix product (the reference
// reaches BLAS through Armadillo); null restores the loop.
void ref_set_dgemm(void *fn) { arma::set_dgemm(reinterpret_cast<arma::dgemm_fn>(fn)); }

// Seconds spent in matrix products since the last reset.
double ref_product_seconds(void) { return arma::product_seconds(); }
void ref_reset_product_seconds(void) { arma::product_seconds() = 0.0; }

}  // extern "C"
