// C entry points over the reference's own CPU block-sparse tensor
// (torque::BlockSparseTensor<T>, T = double or float,
// src/tensor/block_sparse.h:110-656 of Walter-Feng/Torque, with block_in_range
// from src/tensor/block_sparse.cpp), compiled from the reference's sources
// against the Armadillo API subset in arma_api/.  TEST INFRASTRUCTURE ONLY: it
// lets the tests and fixture scripts run the reference's code on the same
// inputs as the oracle and the CUDA path.  Nothing in the library links it.
//
// build_ref.py compiles this file twice: once against the reference header as
// it is, and once with the header's two stride lookups of the CPU contract
// corrected (block_sparse.h:531,538).  In the second build the corrected
// header text arrives first in the same translation unit, so the include
// below is skipped.
//
// A handle carries its element type (REF_F64 or REF_F32); values cross the
// boundary in that type, scalars (query, modify) as double.  Metadata crosses
// in the reference's own layout: begin and end points are rank x n_blocks
// column-major (column = block), as arma::umat stores them.  Every call
// returns 0 on success, 1 when the reference threw its Error type, 2 for any
// other exception (Armadillo-style bounds errors, mixed element types);
// ref_last_error() gives the message.
#ifndef TORQUE_TENSOR_BLOCK_SPARSE_H
#include "tensor/block_sparse.h"
#endif

#include <cstdint>
#include <cstdlib>
#include <exception>
#include <stdexcept>
#include <string>
#include <type_traits>

#define REF_F64 0
#define REF_F32 1

struct ref_tensor {
  int32_t dtype;
  void *t;  // torque::BlockSparseTensor<double> or <float>
};

namespace {

template <class T> using Tensor = torque::BlockSparseTensor<T>;

// The tensor keeps its values in a protected member; a derived type names it.
template <class T> struct DataAccess : Tensor<T> {
  static T *get(const Tensor<T> &t) { return (t.*(&DataAccess::data)).get(); }
  static T *release(Tensor<T> &t) { return (t.*(&DataAccess::data)).release(); }
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

template <class T> constexpr int32_t code() {
  return std::is_same<T, double>::value ? REF_F64 : REF_F32;
}

template <class T> ref_tensor *wrap(Tensor<T> *t) { return new ref_tensor{code<T>(), t}; }

// The handle's tensor, which must hold T.
template <class T> Tensor<T> &as(const ref_tensor *h) {
  if (h->dtype != code<T>()) throw std::invalid_argument("tensors of different element types");
  return *static_cast<Tensor<T> *>(h->t);
}

// ---- per-type bodies of the entry points ----

template <class T> void free_t(ref_tensor *h) {
  Tensor<T> *t = &as<T>(h);
  std::free(DataAccess<T>::release(*t));
  delete t;
}

template <class T> void contract_t(const ref_tensor *a, const ref_tensor *b, int32_t n,
                                   const uint64_t *legs, ref_tensor **out) {
  *out = wrap(new Tensor<T>(as<T>(a).contract(as<T>(b), to_umat(legs, n, 2))));
}

template <class T> void transpose_t(const ref_tensor *a, const uint64_t *perm, ref_tensor **out) {
  const Tensor<T> &A = as<T>(a);
  *out = wrap(new Tensor<T>(A.hard_transpose(to_uvec(perm, A.rank))));
}

template <class T> void query_t(const ref_tensor *a, int32_t n, const uint64_t *idx, double *v) {
  *v = double(as<T>(a).query(to_uvec(idx, n)));
}

template <class T> void modify_t(ref_tensor *a, int32_t n, const uint64_t *idx, double number) {
  as<T>(a).modify(to_uvec(idx, n), T(number));
}

template <class T> void append_t(ref_tensor *a, int32_t rank, const void *data,
                                 const uint64_t *begin, const uint64_t *end,
                                 const uint64_t *table) {
  as<T>(a).append_block(static_cast<const T *>(data), to_uvec(begin, rank), to_uvec(end, rank),
                        to_uvec(table, rank));
}

template <class T> void info_t(const ref_tensor *a, int32_t *rank, int64_t *n_blocks,
                               int64_t *n_elem) {
  const Tensor<T> &A = as<T>(a);
  *rank = int32_t(A.rank);
  *n_blocks = int64_t(A.begin_points.n_cols);
  *n_elem = A.rank ? int64_t(arma::sum(A.block_n_elem)) : 1;
}

template <class T> void read_t(const ref_tensor *a, uint64_t *dimension, uint64_t *begin,
                               uint64_t *end, uint64_t *index_tables, uint64_t *offsets,
                               void *data) {
  const Tensor<T> &A = as<T>(a);
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
    const T *p = DataAccess<T>::get(A);
    T *o = static_cast<T *>(data);
    for (arma::uword i = 0; i < n; i++) o[i] = p[i];
  }
}

}  // namespace

// Runs BODY<double> or BODY<float> after the element type of handle H.
#define REF_DISPATCH(H, BODY, ...)     \
  do {                                 \
    if ((H)->dtype == REF_F64)         \
      BODY<double>(__VA_ARGS__);       \
    else                               \
      BODY<float>(__VA_ARGS__);        \
  } while (0)

extern "C" {

const char *ref_last_error(void) { return last_error.c_str(); }

// BlockSparseTensor(const T*, begin_points, end_points, total_dimension)
// (block_sparse.h:155-202).  The tensor copies the values.
int32_t ref_tensor_new(int32_t dtype, int32_t rank, const uint64_t *dimension, int64_t n_blocks,
                       const uint64_t *begin, const uint64_t *end, const void *data,
                       ref_tensor **out) {
  return guarded([&] {
    const arma::umat b = to_umat(begin, rank, n_blocks), e = to_umat(end, rank, n_blocks);
    const arma::uvec d = to_uvec(dimension, rank);
    if (dtype == REF_F64)
      *out = wrap(new Tensor<double>(static_cast<const double *>(data), b, e, d));
    else
      *out = wrap(new Tensor<float>(static_cast<const float *>(data), b, e, d));
  });
}

// BlockSparseTensor(dimension) (block_sparse.h:147-153): no blocks, one
// zeroed element (a rank-0 tensor's value).
int32_t ref_tensor_new_empty(int32_t dtype, int32_t rank, const uint64_t *dimension,
                             ref_tensor **out) {
  return guarded([&] {
    const arma::uvec d = to_uvec(dimension, rank);
    if (dtype == REF_F64)
      *out = wrap(new Tensor<double>(d));
    else
      *out = wrap(new Tensor<float>(d));
  });
}

// The reference's destructor releases the buffer without freeing it
// (block_sparse.h:259-262); the buffer is freed here.
void ref_tensor_free(ref_tensor *h) {
  if (!h) return;
  REF_DISPATCH(h, free_t, h);
  delete h;
}

// contract(tensor, contracting_indices) (block_sparse.h:414-584); legs is the
// n x 2 contracting-index matrix, column-major (column 0 = this tensor's
// legs).  Both tensors hold the same element type.
int32_t ref_contract(const ref_tensor *a, const ref_tensor *b, int32_t n, const uint64_t *legs,
                     ref_tensor **out) {
  return guarded([&] { REF_DISPATCH(a, contract_t, a, b, n, legs, out); });
}

// hard_transpose(permutation) (block_sparse.h:607-651)
int32_t ref_hard_transpose(const ref_tensor *a, const uint64_t *perm, ref_tensor **out) {
  return guarded([&] { REF_DISPATCH(a, transpose_t, a, perm, out); });
}

// query(indices) (block_sparse.h:372-411)
int32_t ref_query(const ref_tensor *a, int32_t n, const uint64_t *indices, double *value) {
  return guarded([&] { REF_DISPATCH(a, query_t, a, n, indices, value); });
}

// modify(indices, number) (block_sparse.h:322-369)
int32_t ref_modify(ref_tensor *a, int32_t n, const uint64_t *indices, double number) {
  return guarded([&] { REF_DISPATCH(a, modify_t, a, n, indices, number); });
}

// append_block(data, begin_point, end_point, index_table) (block_sparse.h:285-317)
int32_t ref_append_block(ref_tensor *a, int32_t rank, const void *data, const uint64_t *begin,
                         const uint64_t *end, const uint64_t *index_table) {
  return guarded([&] { REF_DISPATCH(a, append_t, a, rank, data, begin, end, index_table); });
}

// element type, rank, block count and element count of a tensor
void ref_tensor_info(const ref_tensor *a, int32_t *dtype, int32_t *rank, int64_t *n_blocks,
                     int64_t *n_elem) {
  *dtype = a->dtype;
  REF_DISPATCH(a, info_t, a, rank, n_blocks, n_elem);
}

// The public metadata members and the values, as the tensor holds them:
// begin/end/index tables rank x n_blocks column-major, offsets per block,
// values in the tensor's element type.  A null destination is skipped.
void ref_tensor_read(const ref_tensor *a, uint64_t *dimension, uint64_t *begin, uint64_t *end,
                     uint64_t *index_tables, uint64_t *offsets, void *data) {
  REF_DISPATCH(a, read_t, a, dimension, begin, end, index_tables, offsets, data);
}

// block_in_range(contracting_indices, A begin, A end, B begins, B ends)
// (block_sparse.cpp:6-175): the B blocks whose contracted intervals meet the
// A block, and each pair's output box (new_begin_points / new_end_points:
// A's free legs then B's, rank_out x count column-major).  Writes up to cap
// pairs (boxes skipped where the destinations are null); returns how many
// there are (or -1 with ref_last_error set).
int64_t ref_block_in_range(int32_t n, const uint64_t *legs, int32_t rank_a,
                           const uint64_t *a_begin, const uint64_t *a_end, int32_t rank_b,
                           int64_t n_b, const uint64_t *b_begin, const uint64_t *b_end,
                           uint64_t *found, uint64_t *new_begin, uint64_t *new_end,
                           int64_t cap) {
  int64_t count = -1;
  const int32_t st = guarded([&] {
    const auto info = torque::block_sparse::block_in_range(
        to_umat(legs, n, 2), to_uvec(a_begin, rank_a), to_uvec(a_end, rank_a),
        to_umat(b_begin, rank_b, n_b), to_umat(b_end, rank_b, n_b));
    count = int64_t(info.block_indices.n_elem);
    const int64_t m = count < cap ? count : cap;
    for (int64_t i = 0; i < m; i++) found[i] = info.block_indices[i];
    const arma::uword ro = info.new_begin_points.n_rows;
    if (new_begin && new_end && count)
      for (arma::uword i = 0; i < ro * arma::uword(m); i++) {
        new_begin[i] = info.new_begin_points[i];
        new_end[i] = info.new_end_points[i];
      }
  });
  return st ? -1 : count;
}

// Register a Fortran-convention dgemm for the double matrix product (the
// reference reaches BLAS through Armadillo); null restores the loop.
void ref_set_dgemm(void *fn) { arma::set_dgemm(reinterpret_cast<arma::dgemm_fn>(fn)); }

// Seconds spent in matrix products since the last reset.
double ref_product_seconds(void) { return arma::product_seconds(); }
void ref_reset_product_seconds(void) { arma::product_seconds() = 0.0; }

}  // extern "C"
