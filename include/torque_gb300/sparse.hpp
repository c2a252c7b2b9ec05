// torque::gpu::SparseTensor<T> (element-sparse, COO) over the C ABI of
// libtorque_gb300.
//
// The reference class (src/gpu/sparse.cuh:81-436) stores linear indices and
// values, contracts by testing every pair of nonzeros (handle_indices_kernel,
// sparse.cu:88-139), multiplying all value pairs with a k=1 GEMM and reducing
// by key.  Here every nonzero is a one-element block of a block-sparse
// tensor: the library's matcher pairs nonzeros with equal contracted
// coordinates, and the reduced layout sums the products landing on the same
// output coordinate, one output block per distinct coordinate in ascending
// linear order.  Differences from the reference, on purpose:
//   * `indices` is a host vector (the reference exposes a device vector);
//   * contract keeps every output element (the reference drops the first
//     reduced key, sparse.cuh:370-371, assuming it is the -1 of non-matching
//     pairs, which removes a real element when every pair matches);
//   * modify(index, 0) stores a zero instead of removing the element; query
//     answers the same.
#pragma once

#include <algorithm>
#include <numeric>

#include "dense.hpp"

namespace torque {
namespace gpu {

template <typename T>
class SparseTensor {
 public:
  arma::uword rank = 0;
  arma::uvec dimension;
  arma::uvec index_table;
  std::vector<int64_t> indices;  // linear index (through index_table) of each element

  // SparseTensor(dimension) (sparse.cuh:95-103): no elements (a scalar is 0).
  explicit SparseTensor(const arma::uvec &dim)
      : rank(dim.n_elem), dimension(dim), index_table(detail::index_table_of(dim)) {
    const auto d = detail::flat(dim);
    detail::check(tq_bs_create_empty(detail::dtype<T>(), (int32_t)rank, d.data(), &h_));
  }

  // SparseTensor(source, indices, index_table, dimension) (sparse.cuh:105-137).
  SparseTensor(const T *source_data, const arma::uvec &element_indices,
               const arma::uvec &table, const arma::uvec &dim)
      : rank(dim.n_elem), dimension(dim), index_table(table) {
    if (!source_data) throw Error("Source data not allocated!");
    build(source_data, element_indices);
  }

  SparseTensor(const SparseTensor &o)
      : rank(o.rank), dimension(o.dimension), index_table(o.index_table), indices(o.indices) {
    detail::check(tq_bs_clone(o.h_, nullptr, &h_));
  }
  SparseTensor(SparseTensor &&o) noexcept
      : rank(o.rank), dimension(std::move(o.dimension)), index_table(std::move(o.index_table)),
        indices(std::move(o.indices)) {
    std::swap(h_, o.h_);
  }
  SparseTensor &operator=(SparseTensor &&o) noexcept {
    rank = o.rank;
    dimension = std::move(o.dimension);
    index_table = std::move(o.index_table);
    indices = std::move(o.indices);
    std::swap(h_, o.h_);
    return *this;
  }
  SparseTensor &operator=(const SparseTensor &o) {
    if (this != &o) {
      SparseTensor c(o);
      *this = std::move(c);
    }
    return *this;
  }
  ~SparseTensor() {
    if (h_) tq_bs_destroy(h_);
  }

  T to_number() const {
    T v = T(0);
    detail::check(tq_bs_to_number(h_, &v));
    return v;
  }

  // initialize(source, indices) (sparse.cuh:147-160).
  void initialize(const T *source_data, const arma::uvec &element_indices) {
    if (!source_data) throw Error("Source data not allocated!");
    if (h_) tq_bs_destroy(h_);
    h_ = nullptr;
    build(source_data, element_indices);
  }

  void modify(const arma::uvec &at, const T number) {
    if (at.n_elem != rank) throw Error("Rank does not match");
    const auto idx = detail::flat(at);
    detail::check(tq_bs_modify(h_, rank ? idx.data() : nullptr, &number));
    refresh_indices();
  }

  T query(const arma::uvec &at) const {
    if (at.n_elem != rank) throw Error("Rank does not match");
    const auto idx = detail::flat(at);
    T v = T(0);
    detail::check(tq_bs_query(h_, rank ? idx.data() : nullptr, &v));
    return v;
  }

  // contract(handle, tensor, contracting_indices) (sparse.cuh:270-375).
  template <typename Handle>
  SparseTensor contract(Handle, const SparseTensor &tensor,
                        const arma::umat &contracting_indices) const {
    return contract(tensor, contracting_indices);
  }
  // Matching nonzeros are found by sorting both operands by their contracted
  // index (tq_bs_contract_elements), not by testing every pair; a contraction
  // over every leg (a scalar) takes the block path.
  SparseTensor contract(const SparseTensor &tensor, const arma::umat &contracting_indices) const {
    std::vector<int64_t> al, bl;
    detail::contract_legs(contracting_indices, al, bl);
    tq_bs *out = nullptr;
    if (rank + tensor.rank > 2 * al.size()) {
      detail::check(tq_bs_contract_elements(h_, tensor.h_, (int32_t)al.size(), al.data(),
                                            bl.data(), nullptr, &out));
    } else {
      const tq_contract_opts o = {TQ_PREC_NATIVE, TQ_LAYOUT_REDUCED, 0, 0, 0, 0};
      detail::check(tq_bs_contract(h_, tensor.h_, (int32_t)al.size(), al.data(), bl.data(), &o,
                                   nullptr, &out));
    }
    return SparseTensor(out);
  }

  // soft_transpose(permutation) (sparse.cuh:380-391): the element coordinates
  // follow the legs, the linear indices keep their values.
  void soft_transpose(const arma::uvec &permutation) {
    if (permutation.n_elem != rank)
      throw Error("The number of permutation does not match the rank of tensor");
    const auto p = detail::flat(permutation);
    tq_bs *out = nullptr;
    detail::check(tq_bs_hard_transpose(h_, p.data(), nullptr, &out));
    tq_bs_destroy(h_);
    h_ = out;
    dimension = detail::permuted(dimension, permutation);
    index_table = detail::permuted(index_table, permutation);
  }

  // hard_transpose(permutation) (sparse.cuh:395-430): a new tensor whose
  // linear indices follow the permuted dimensions.
  SparseTensor hard_transpose(const arma::uvec &permutation) const {
    if (permutation.n_elem != rank)
      throw Error("The number of permutation does not match the rank of tensor");
    const auto p = detail::flat(permutation);
    tq_bs *out = nullptr;
    detail::check(tq_bs_hard_transpose(h_, p.data(), nullptr, &out));
    return SparseTensor(out);
  }

  tq_bs *handle() const { return h_; }

 private:
  // a result of the library: column-major index table of its dimensions
  explicit SparseTensor(tq_bs *h) : h_(h) {
    detail::shape_of(h_, rank, dimension);
    index_table = detail::index_table_of(dimension);
    refresh_indices();
  }

  // one-element blocks at the coordinates of the linear indices (decoded
  // through the index table, largest stride first, as index_to_indices does
  // for a possibly permuted table, src/util/space.h:27-58)
  void build(const T *src, const arma::uvec &element_indices) {
    const auto d = detail::flat(dimension);
    const arma::uword n = element_indices.n_elem;
    if (rank == 0) {
      detail::check(tq_bs_create(detail::dtype<T>(), 0, nullptr, 0, nullptr, nullptr, nullptr,
                                 src, TQ_MEM_HOST, nullptr, &h_));
      indices.clear();
      return;
    }
    std::vector<arma::uword> order(rank);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(),
              [&](arma::uword a, arma::uword b) { return index_table(a) > index_table(b); });
    std::vector<int64_t> pts(n * rank);
    indices.resize(n);
    for (arma::uword e = 0; e < n; e++) {
      arma::uword x = element_indices(e);
      indices[e] = (int64_t)x;
      for (arma::uword q : order) {
        const arma::uword c = x / index_table(q);
        x %= index_table(q);
        if (c >= dimension(q)) throw Error("Indices out of boundary");
        pts[e * rank + q] = (int64_t)c;
      }
    }
    if (n == 0) {
      detail::check(tq_bs_create_empty(detail::dtype<T>(), (int32_t)rank, d.data(), &h_));
      return;
    }
    detail::check(tq_bs_create(detail::dtype<T>(), (int32_t)rank, d.data(), (int64_t)n,
                               pts.data(), pts.data(), nullptr, src, TQ_MEM_HOST, nullptr, &h_));
  }

  void refresh_indices() {
    tq_dtype dt;
    int32_t r = 0;
    int64_t nb = 0, ne = 0;
    detail::check(tq_bs_shape(h_, &dt, &r, &nb, &ne));
    indices.assign((size_t)nb, 0);
    if (!nb || !r) return;
    std::vector<int64_t> b(nb * r);
    detail::check(tq_bs_metadata(h_, nullptr, b.data(), nullptr, nullptr, nullptr));
    for (int64_t e = 0; e < nb; e++)
      for (int32_t l = 0; l < r; l++) indices[e] += b[e * r + l] * (int64_t)index_table(l);
  }

  tq_bs *h_ = nullptr;
};

}  // namespace gpu
}  // namespace torque
